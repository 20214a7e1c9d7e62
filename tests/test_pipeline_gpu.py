"""The reference's timing and verification pipeline around the GB300 driver.

* heatdrv linked under a reference binary name (1-omp, 1-cuda) writes that
  binary's dump (u_openmp_1gpu.txt, u_cuda_1gpu.txt), which verify.sh's
  check (OpenMP/verify.sh:160-186, ported as pipeline.compare_dumps) accepts
  against the oracle's dump at its 1e-10 tolerance -- and which equals it
  byte for byte with --bitexact.
* pipeline.run() times the real driver into results_*/ directories that
  pipeline.aggregate() and the gamma reduction read."""
from __future__ import annotations

import os
import subprocess

import pytest

from conftest import PKG

import pipeline

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def drv(heat, cuda_device):
    return PKG / "heatdrv"


def run(cmd, cwd, env=None):
    e = {**os.environ, **(env or {})}
    return subprocess.run([str(c) for c in cmd], cwd=cwd, env=e, capture_output=True, text=True,
                          check=True).stdout


@pytest.mark.parametrize("name,dump", [("1-omp", "u_openmp_1gpu.txt"), ("1-cuda", "u_cuda_1gpu.txt")])
def test_reference_binary_names_verify(drv, oracle, tmp_path, name, dump):
    n, steps = 40, 50
    T = "%.17g" % oracle.verify_T(n, steps)
    (tmp_path / name).symlink_to(drv)
    run([oracle.CLI_PATH, n, T], tmp_path, {"WRITE_TXT": "1", "OMP_NUM_THREADS": "4"})
    out = run([f"./{name}", n, T], tmp_path, {"WRITE_TXT": "1"})
    assert f"Solution written to {dump}" in out
    ok, worst, _, msg = pipeline.compare_dumps(tmp_path / "u_ref.txt", tmp_path / dump, 1e-10)
    assert ok, msg
    run([f"./{name}", n, T, "--bitexact"], tmp_path, {"WRITE_TXT": "1"})
    assert (tmp_path / dump).read_bytes() == (tmp_path / "u_ref.txt").read_bytes()


def test_pipeline_run_aggregate_gamma(drv, tmp_path):
    made = pipeline.run([48, 72], reps=2, steps=30, driver=drv, out_dir=tmp_path, job_id="g")
    assert len(made) == 4
    for d in made:
        row = (d / "timings.csv").read_text().splitlines()[1].split(",")
        assert row[-1] == "ok" and row[10] != "N/A"
    summ = pipeline.aggregate(tmp_path, "compute").splitlines()
    assert summ[0] == pipeline.SUMMARY_COLUMNS
    assert [r.split(",")[2] for r in summ[1:]] == ["48", "72"]
    for r in summ[1:]:
        f = r.split(",")
        assert f[0] == pipeline.DEFAULT_VARIANT and f[3] == "2" and f[4] == "0"
        assert float(f[6]) > 0 and int(f[9]) in (30, 31)
    (tmp_path / "summary.csv").write_text("\n".join(summ) + "\n")
    rows = pipeline.gamma_rows(tmp_path / "summary.csv")
    assert [r["N"] for r in rows] == [48, 72]
    assert all(r["gamma_s_per_point"] > 0 for r in rows)
