"""Build libheat.so (sm_103a kernels + C ABI) and the heatdrv host driver in-tree.

    python openmp-offloading-intranode-artifact_gb300/heat_build.py [--force]

Translation units compile in parallel; a unit is rebuilt only when its source
or a header is newer than its object.  Device code targets sm_103a only.
The bit-exact kernels' unit is compiled with --fmad=false (the reference's
CUDA flag set, 3D_Heat_Benchmark/NVIDIA-H100/Source-Results/CUDA/Makefile:36-37).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
OBJ = PKG / "_build"
LIB = PKG / "libheat.so"
DRV = PKG / "heatdrv"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                      "-I", str(ROOT / "include"), "-I", str(CSRC)]
# Extra nvcc flags for every CUDA unit (e.g. -D switches), from the environment.
NVCC_COMMON += os.environ.get("HEAT_NVCC_EXTRA", "").split()
# Per-unit extra flags.
UNIT_FLAGS = {
    "heat_fp64_exact.cu": ["--fmad=false", "--prec-div=true", "--prec-sqrt=true", "--ftz=false"],
}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA 13 toolkit is required to build libheat")


def _cuda_include(nvcc: str) -> Path:
    return Path(nvcc).resolve().parent.parent / "include"


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n  " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(force: bool = False, verbose: bool = False) -> Path:
    nvcc = _nvcc()
    OBJ.mkdir(exist_ok=True)
    headers = list(CSRC.glob("*.h")) + list(CSRC.glob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    jobs = []
    for src in sorted(CSRC.glob("*.cu")):
        obj = OBJ / (src.name + ".o")
        if force or _stale(obj, [src] + headers):
            jobs.append([nvcc, *NVCC_COMMON, *UNIT_FLAGS.get(src.name, []), "-c", str(src), "-o", str(obj)])
    for src in sorted(CSRC.glob("*.cpp")):
        obj = OBJ / (src.name + ".o")
        if force or _stale(obj, [src] + headers):
            jobs.append(["g++", "-O3", "-fPIC", "-std=c++17", "-ffp-contract=off", "-pthread",
                         "-I", str(ROOT / "include"), "-I", str(CSRC), "-I", str(_cuda_include(nvcc)),
                         "-c", str(src), "-o", str(obj)])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for f in [ex.submit(_run, j) for j in jobs]:
                f.result()
    objs = sorted(OBJ.glob("*.o"))
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, *ARCH, "-shared", "-o", str(LIB), *map(str, objs), "-lpthread", "-ldl"])
    drv_src = PKG / "driver" / "heatdrv.c"
    if drv_src.exists() and (force or _stale(DRV, [drv_src, LIB, ROOT / "include" / "heat.h"])):
        _run(["gcc", "-O2", "-std=c11", "-D_DEFAULT_SOURCE", "-I", str(ROOT / "include"),
              "-o", str(DRV), str(drv_src), "-L", str(PKG), "-lheat", "-lm",
              "-Wl,-rpath,$ORIGIN"])
    if verbose:
        print(f"built {LIB}" + (f" and {DRV}" if DRV.exists() else ""))
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
