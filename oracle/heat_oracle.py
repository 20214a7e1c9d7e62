"""ORACLE -- TEST INFRASTRUCTURE ONLY.

ctypes wrapper of the CPU restatement of the reference's heat-update loop
(oracle/heat_ref.c) for the tests and for bench.py's CPU-baseline leg.
The product never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
LIB_PATH = BUILD / "libheat_oracle.so"
CLI_PATH = BUILD / "heat_ref"
REF_SERIAL = HERE / "_ref" / "serial"


def build() -> None:
    """Compile the restatement (and the reference serial where its source is present)."""
    subprocess.run(["bash", str(HERE / "build_ref.sh")], check=True, capture_output=True)


def ensure_built() -> None:
    srcs = [HERE / "heat_ref.c", HERE / "heat_ref_main.c", HERE / "heat_ref.h",
            HERE.parent / "openmp-offloading-intranode-artifact_gb300" / "csrc" / "heat_inputs.cpp"]
    if not LIB_PATH.exists() or not CLI_PATH.exists() or any(
            s.stat().st_mtime > LIB_PATH.stat().st_mtime for s in srcs):
        build()


_LIB = None


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        ensure_built()
        L = C.CDLL(str(LIB_PATH))
        dp = C.c_void_p
        L.heat_ref_factor.restype = C.c_double
        L.heat_ref_factor.argtypes = [C.c_double, C.c_double]
        L.heat_ref_update.restype = None
        L.heat_ref_update.argtypes = [dp, dp, dp, dp, C.c_int, C.c_int, C.c_int, C.c_double]
        L.heat_ref_steps.restype = C.c_int
        L.heat_ref_steps.argtypes = [dp, dp, dp, dp, C.c_int, C.c_int, C.c_int, C.c_double,
                                     C.c_int, C.POINTER(C.c_double)]
        L.heat_ref_run_T.restype = C.c_int
        L.heat_ref_run_T.argtypes = [dp, dp, dp, dp, C.c_int, C.c_int, C.c_int, C.c_double,
                                     C.c_double, C.c_double, C.POINTER(C.c_double)]
        L.heat_ref_count_steps.restype = C.c_int
        L.heat_ref_count_steps.argtypes = [C.c_double, C.c_double]
        L.heat_ref_norm.restype = None
        L.heat_ref_norm.argtypes = [dp, C.c_size_t, C.POINTER(C.c_double), C.POINTER(C.c_double)]
        L.heat_ref_threads.restype = C.c_int
        L.heat_inputs_reference.restype = C.c_int
        L.heat_inputs_reference.argtypes = [C.c_int, dp, dp, dp, C.POINTER(C.c_double),
                                            C.POINTER(C.c_double)]
        L.heat_inputs_config.restype = C.c_int
        L.heat_inputs_config.argtypes = [C.c_int, C.c_uint64, C.c_int, C.c_int, C.c_int, dp, dp,
                                         C.POINTER(C.c_double), C.POINTER(C.c_double)]
        _LIB = L
    return _LIB


def _p(a):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data


def factor(h: float, dt: float) -> float:
    return lib().heat_ref_factor(h, dt)


def steps(u0, kappa, h, dt, nsteps, rhs=None):
    """nsteps explicit reference steps from u0; returns the final field (new array)."""
    u = np.array(u0, dtype=np.float64, order="C", copy=True)
    w = u.copy()
    nz, ny, nx = u.shape
    kappa = np.ascontiguousarray(kappa, dtype=np.float64)
    rhs = None if rhs is None else np.ascontiguousarray(rhs, dtype=np.float64)
    lib().heat_ref_steps(_p(u), _p(w), _p(rhs), _p(kappa), nz, ny, nx, factor(h, dt), nsteps, None)
    return u


def run_T(u0, kappa, h, dt, T, rhs=None):
    """while (t < T) { step; t += dt; }; returns (field, steps)."""
    u = np.array(u0, dtype=np.float64, order="C", copy=True)
    w = u.copy()
    nz, ny, nx = u.shape
    kappa = np.ascontiguousarray(kappa, dtype=np.float64)
    rhs = None if rhs is None else np.ascontiguousarray(rhs, dtype=np.float64)
    s = lib().heat_ref_run_T(_p(u), _p(w), _p(rhs), _p(kappa), nz, ny, nx, factor(h, dt), T, dt, None)
    return u, s


def count_steps(T: float, dt: float) -> int:
    return lib().heat_ref_count_steps(T, dt)


def norm(u):
    u = np.ascontiguousarray(u, dtype=np.float64)
    l2, cs = C.c_double(), C.c_double()
    lib().heat_ref_norm(_p(u), u.size, C.byref(l2), C.byref(cs))
    return l2.value, cs.value


def inputs_reference(n: int):
    kappa, rhs, u0 = (np.empty((n, n, n)) for _ in range(3))
    h, dt = C.c_double(), C.c_double()
    rc = lib().heat_inputs_reference(n, _p(kappa), _p(rhs), _p(u0), C.byref(h), C.byref(dt))
    assert rc == 0
    return kappa, rhs, u0, h.value, dt.value


def inputs_config(cfg: int, seed: int, nx: int, ny: int, nz: int):
    kappa, u0 = np.empty((nz, ny, nx)), np.empty((nz, ny, nx))
    h, dt = C.c_double(), C.c_double()
    rc = lib().heat_inputs_config(cfg, seed, nx, ny, nz, _p(kappa), _p(u0), C.byref(h), C.byref(dt))
    assert rc == 0
    return kappa, u0, h.value, dt.value


def verify_T(n: int, nsteps: int, kappa_max: float = 0.95, fmt: str = "%.17g") -> float:
    """T the reference's verify pipeline passes for (n, STEPS): STEPS*dt printed
    with fmt (OpenMP/verify.sh:59-65 uses %.17g; submit.sh:107-109 %.7g)."""
    h = 1.0 / (n - 1)
    dt = h * h / (12.0 * kappa_max)
    return float(fmt % (nsteps * dt))


def cli(args, env=None, cwd=None) -> subprocess.CompletedProcess:
    ensure_built()
    e = dict(os.environ)
    if env:
        e.update(env)
    return subprocess.run([str(CLI_PATH), *map(str, args)], capture_output=True, text=True,
                          env=e, cwd=cwd, check=True)
