"""Generate tests/golden/pipeline_ref.json.gz: inputs and outputs of the
reference's own result-reduction tools, to pin pipeline.py against them.

Run here, where the reference tree is present (it is not on the GPU machine):

    python tests/golden/make_pipeline_golden.py <reference checkout root>

What it records:

1. For the reference's published result sets (NVIDIA-H100 CUDA and OpenMP,
   Intel-1550 SYCL), the lines of every results_*/run.log that the reduction
   parses (">>> ..." headers, "Estimated timesteps:", "... timesteps
   complete", "Time = ...") and every results_*/timings.csv, then the output
   of the reference's aggregate.sh (3D_Heat_Benchmark/NVIDIA-H100/
   Source-Results/CUDA/aggregate.sh, the one that handles every schema) on
   those files in compute, wall and reported mode.  For the NVIDIA sets the
   compute-mode output is checked to equal the summary.csv the reference
   committed, so the extracted lines carry everything the reduction reads.
2. The reference's compute_gamma.py (model/compute_gamma.py) on those
   summaries (its gamma_single_gpu.csv, checked against the committed one for
   OpenMP).
3. Result directories written by pipeline.run() around a stand-in driver that
   prints heatdrv's output lines, and aggregate.sh's reduction of them: the
   reference's tool must read what this build writes.

The reference's scripts are run in a scratch directory under LC_ALL=C; the
fixture holds only their inputs and outputs, not their code.
"""
from __future__ import annotations

import gzip
import json
import os
import re
import subprocess
import sys
import tempfile
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path.insert(0, str(ROOT / "openmp-offloading-intranode-artifact_gb300"))
import pipeline  # noqa: E402

PARSED = re.compile(r"^>>> |^Estimated timesteps:|timesteps? complete|^Time = ")
SETS = {
    "h100_cuda": "3D_Heat_Benchmark/NVIDIA-H100/Source-Results/CUDA",
    "h100_openmp": "3D_Heat_Benchmark/NVIDIA-H100/Source-Results/OpenMP",
    "intel_sycl": "3D_Heat_Benchmark/Intel-1550/Source-Results/SYCL",
}
AGGREGATE = "3D_Heat_Benchmark/NVIDIA-H100/Source-Results/CUDA/aggregate.sh"
GAMMA = "3D_Heat_Benchmark/NVIDIA-H100/Source-Results/model/compute_gamma.py"

FAKE_DRIVER = r'''#!/usr/bin/env python3
import sys
n = int(sys.argv[1]); T = float(sys.argv[2])
h = 1.0 / (n - 1); dt = h * h / (12.0 * 0.95)
t = 0.0; s = 0
while t < T:
    t += dt; s += 1
sec = 1e-7 * (n - 2) ** 3 * s * (1.0 + 0.01 * (n % 7))
print("\n**** ONE GPU GB300 STARTS ****")
print("=== SIMULATION PARAMETERS ===")
print("Grid size (n):           %d" % n)
print("Final time (T):          %.6f" % T)
print("Estimated timesteps:     ~%d" % int(T / dt))
print("==============================\n")
print("\n=== SIMULATION STARTS ===")
print("\n%d timesteps complete" % s)
print("Time = %f seconds" % sec)
print("GLUP/s = %.3f" % ((n - 2) ** 3 * s / sec / 1e9))
print("=== SIMULATION ENDS ===")
'''


def reduce_with_reference(ref: Path, dirs: dict, mode: str) -> str:
    """Run the reference aggregate.sh over `dirs` (name -> {file: text})."""
    with tempfile.TemporaryDirectory() as td:
        for name, files in dirs.items():
            d = Path(td) / name
            d.mkdir()
            for fname, text in files.items():
                (d / fname).write_text(text)
        env = {**os.environ, "LC_ALL": "C", "TIME_FIELD": mode}
        p = subprocess.run(["bash", str(ref / AGGREGATE), "out.csv"], cwd=td, env=env,
                           capture_output=True, text=True)
        if p.returncode != 0:
            return "ERROR"
        return (Path(td) / "out.csv").read_text()


def gamma_with_reference(ref: Path, summary_text: str, exe: str) -> str:
    with tempfile.TemporaryDirectory() as td:
        (Path(td) / "summary.csv").write_text(summary_text)
        p = subprocess.run([sys.executable, str(ref / GAMMA), "--summary", "summary.csv",
                            "--exe", exe, "--output", "g.csv"], cwd=td, capture_output=True,
                           text=True)
        if p.returncode != 0:
            return "ERROR"
        return (Path(td) / "g.csv").read_text()


def main() -> None:
    if len(sys.argv) < 2:
        sys.exit("usage: make_pipeline_golden.py <reference checkout root>")
    ref = Path(sys.argv[1])
    out = {"sets": {}, "gamma": {}, "own": {}}
    for key, rel in SETS.items():
        base = ref / rel
        dirs = {}
        for d in sorted(base.glob("results_*")):
            files = {}
            if (d / "run.log").is_file():
                lines = [ln for ln in (d / "run.log").read_text(errors="replace").splitlines()
                         if PARSED.search(ln)]
                files["run.log"] = "\n".join(lines) + "\n"
            if (d / "timings.csv").is_file():
                files["timings.csv"] = (d / "timings.csv").read_text()
            dirs[d.name] = files
        expected = {m: reduce_with_reference(ref, dirs, m) for m in ("compute", "wall", "reported")}
        if (base / "summary.csv").is_file() and key.startswith("h100"):
            assert expected["compute"] == (base / "summary.csv").read_text(), key
        out["sets"][key] = {"dirs": dirs, "expected": expected}

    for key, exe in (("h100_openmp", "1-omp"), ("h100_cuda", "1-cuda")):
        summ = out["sets"][key]["expected"]["compute"]
        g = gamma_with_reference(ref, summ, exe)
        out["gamma"][key] = {"summary": summ, "exe": exe, "expected": g}
    committed = ref / SETS["h100_openmp"] / "gamma_single_gpu.csv"
    assert out["gamma"]["h100_openmp"]["expected"] == committed.read_text()

    # this build's result directories, reduced by the reference's tool
    with tempfile.TemporaryDirectory() as td:
        drv = Path(td) / "fake_heatdrv"
        drv.write_text(FAKE_DRIVER)
        drv.chmod(0o755)
        made = pipeline.run([48, 64, 80], reps=3, steps=20, driver=drv, out_dir=Path(td) / "res",
                            job_id="golden")
        dirs = {d.name: {f: (d / f).read_text() for f in ("run.log", "timings.csv")} for d in made}
    out["own"] = {"dirs": dirs,
                  "expected": {m: reduce_with_reference(ref, dirs, m) for m in ("compute", "wall", "reported")}}
    s = out["own"]["expected"]["compute"]
    out["own"]["gamma"] = gamma_with_reference(ref, s, pipeline.DEFAULT_VARIANT)

    dst = HERE / "pipeline_ref.json.gz"
    with gzip.open(dst, "wt", encoding="utf-8") as f:
        json.dump(out, f, sort_keys=True)
    print(f"wrote {dst} ({dst.stat().st_size} bytes)")


if __name__ == "__main__":
    main()
