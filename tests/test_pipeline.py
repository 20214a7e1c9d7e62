"""pipeline.py against the reference's own result-reduction tools.

The fixture (tests/golden/make_pipeline_golden.py) holds the reference's
published result directories (the run.log lines its aggregate.sh parses and
its timings.csv files), the output of its aggregate.sh on them in compute,
wall and reported mode (CUDA/aggregate.sh:26-160), the output of its
compute_gamma.py (model/compute_gamma.py), and result directories written
by pipeline.run() together with aggregate.sh's reduction of them.  Every
comparison here is byte for byte."""
from __future__ import annotations

import gzip
import json
import sys
import textwrap
from pathlib import Path

import pytest

from conftest import GOLDEN

import pipeline

FIX = json.load(gzip.open(GOLDEN / "pipeline_ref.json.gz", "rt", encoding="utf-8"))


def materialise(dirs: dict, root: Path) -> Path:
    for name, files in dirs.items():
        d = root / name
        d.mkdir(parents=True)
        for fname, text in files.items():
            (d / fname).write_text(text)
    return root


@pytest.mark.parametrize("key", sorted(FIX["sets"]))
@pytest.mark.parametrize("mode", ["compute", "wall", "reported"])
def test_aggregate_matches_reference(tmp_path, key, mode):
    s = FIX["sets"][key]
    root = materialise(s["dirs"], tmp_path)
    want = s["expected"][mode]
    if want == "ERROR":
        # the reference's tool finds no timed run it recognises (SYCL variant
        # names in compute mode); so does the port
        with pytest.raises(ValueError):
            pipeline.aggregate(root, mode)
        return
    assert pipeline.aggregate(root, mode) == want


@pytest.mark.parametrize("key", sorted(FIX["gamma"]))
def test_gamma_matches_reference(tmp_path, key):
    g = FIX["gamma"][key]
    (tmp_path / "summary.csv").write_text(g["summary"])
    rows = pipeline.gamma_rows(tmp_path / "summary.csv", g["exe"])
    pipeline.write_gamma_csv(rows, tmp_path / "g.csv")
    assert (tmp_path / "g.csv").read_text() == g["expected"]


def test_gamma_plateau_known_answer(tmp_path):
    """The reference's published plateau for 1-omp on H100 is the mean of its
    three largest grids: 6.4042e-11 s per point update."""
    g = FIX["gamma"]["h100_openmp"]
    (tmp_path / "summary.csv").write_text(g["summary"])
    rows = pipeline.gamma_rows(tmp_path / "summary.csv", "1-omp")
    assert [r["N"] for r in rows][-3:] == [1024, 1152, 1280]
    assert f"{pipeline.gamma_plateau(rows):.4e}" == "6.4042e-11"


def test_own_results_reduced_by_reference_tool(tmp_path):
    """Directories written by pipeline.run() reduce identically with the
    reference's aggregate.sh and with the port, in every mode, and gamma
    agrees with compute_gamma.py."""
    own = FIX["own"]
    root = materialise(own["dirs"], tmp_path)
    for mode in ("compute", "wall", "reported"):
        assert own["expected"][mode] != "ERROR"
        assert pipeline.aggregate(root, mode) == own["expected"][mode]
    (tmp_path / "summary.csv").write_text(own["expected"]["compute"])
    rows = pipeline.gamma_rows(tmp_path / "summary.csv", pipeline.DEFAULT_VARIANT)
    pipeline.write_gamma_csv(rows, tmp_path / "g.csv")
    assert (tmp_path / "g.csv").read_text() == own["gamma"]


def test_final_time_matches_reference_timings():
    """DT as submit.sh prints it: every (N, steps, dt) row of the reference's
    timings.csv files is reproduced."""
    seen = 0
    for key in ("h100_cuda", "h100_openmp"):
        for files in FIX["sets"][key]["dirs"].values():
            lines = files["timings.csv"].splitlines()
            head = lines[0].split(",")
            iN, idt, ist = head.index("N"), head.index("dt"), head.index("steps")
            for ln in lines[1:]:
                f = ln.split(",")
                if len(f) != len(head):
                    continue
                assert pipeline.final_time(int(f[iN]), int(f[ist])) == f[idt]
                seen += 1
    assert seen > 100


STAND_IN = textwrap.dedent('''\
    #!{py}
    import sys
    n = int(sys.argv[1]); T = float(sys.argv[2])
    h = 1.0 / (n - 1); dt = h * h / (12.0 * 0.95)
    t = 0.0; s = 0
    while t < T:
        t += dt; s += 1
    print("Estimated timesteps:     ~%d" % int(T / dt))
    print("\\n%d timesteps complete" % s)
    print("Time = %f seconds" % (1e-3 * n))
    sys.exit(3 if n == 13 else 0)
''')


def test_run_writes_reference_layout(tmp_path):
    drv = tmp_path / "drv"
    drv.write_text(STAND_IN.format(py=sys.executable))
    drv.chmod(0o755)
    made = pipeline.run([16, 13], reps=2, steps=10, driver=drv, out_dir=tmp_path / "res",
                        job_id="t")
    assert len(made) == 4 and all(d.name.startswith("results_t") for d in made)
    rows = []
    for d in made:
        csv_lines = (d / "timings.csv").read_text().splitlines()
        assert csv_lines[0] == pipeline.TIMINGS_HEADER
        rows.append(csv_lines[1].split(","))
        log = (d / "run.log").read_text()
        assert ">>> 1-cuda-gb300  gpus=1  mask=0  N=" in log
    status = {r[6]: r[-1] for r in rows}
    assert status == {"16": "ok", "13": "runtime_error"}
    assert all(r[7] == pipeline.final_time(int(r[6]), 10) for r in rows)
    assert [r[10] for r in rows if r[6] == "16"] == ["0.016000", "0.016000"]
    summ = pipeline.aggregate(tmp_path / "res", "compute").splitlines()
    # compute mode reads run.log, where the failed runs still printed a time
    assert summ[0] == pipeline.SUMMARY_COLUMNS
    assert summ[1].startswith("1-cuda-gb300,1,13,2,0,0.0130,0.0130,0.0130,0.0,")
    assert summ[2].startswith("1-cuda-gb300,1,16,2,0,0.0160,0.0160,0.0160,0.0,")
    wall = pipeline.aggregate(tmp_path / "res", "reported").splitlines()
    assert wall[1] == "1-cuda-gb300,1,13,0,2,N/A,N/A,N/A,runtime_error,10"
    assert wall[2] == "1-cuda-gb300,1,16,2,0,0.0160,0.0160,0.0160,0.0,10"


def test_compare_dumps(tmp_path):
    a = tmp_path / "a.txt"
    b = tmp_path / "b.txt"
    a.write_text("0\n1.5\n-2\n")
    b.write_text("0\n1.5000000000001\n-2\n")
    ok, worst, line, msg = pipeline.compare_dumps(a, b, 1e-10)
    assert ok and line == 2 and 0 < worst < 1e-12 and msg.endswith("PASS")
    b.write_text("0\n1.5\n-2.001\n")
    ok, worst, line, msg = pipeline.compare_dumps(a, b, 1e-10)
    assert not ok and line == 3 and msg.endswith("FAIL")
    b.write_text("0\n1.5\n")
    ok, _, _, msg = pipeline.compare_dumps(a, b, 1e-10)
    assert not ok and msg == "LINE COUNT MISMATCH (3 vs 2)"
