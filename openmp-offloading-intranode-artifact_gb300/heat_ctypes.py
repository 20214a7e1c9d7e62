"""ctypes binding of libheat's C ABI (include/heat.h).

The binding is deliberately thin: numpy arrays in, status codes turned into
HeatError.  It is what a Python caller of the reference's heat_update() /
solver loop binds, and what the tests and bench.py call through.  It never
falls back to anything: if libheat.so is missing or fails to load, import
raises.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import numpy as np

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libheat.so"

HEAT_OK = 0
HEAT_EINVAL = -1
HEAT_ENOMEM = -2
HEAT_ECUDA = -3
HEAT_ETIMEOUT = -4
HEAT_EBUDGET = -5
HEAT_ENODEV = -6
HEAT_ESTATE = -7

HEAT_FP64 = 0
HEAT_FP32C = 1

HEAT_BITEXACT = 0x1
HEAT_NAIVE = 0x2
HEAT_HWFP64 = 0x4
HEAT_NO_TEMPORAL = 0x8

HEAT_BATCH_NO_GRAPHS = 0x1
HEAT_BATCH_PERSISTENT = 0x2
HEAT_BATCH_SERIAL_FORMS = 0x4


class HeatError(RuntimeError):
    def __init__(self, what: str, status: int, msg: str):
        super().__init__(f"{what}: {msg} (status {status})")
        self.status = status


class HeatDesc(C.Structure):
    _fields_ = [
        ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
        ("h", C.c_double), ("dt", C.c_double),
        ("kappa", C.c_void_p), ("u0", C.c_void_p), ("rhs", C.c_void_p),
        ("precision", C.c_int), ("flags", C.c_uint),
        ("stream", C.c_void_p),
    ]


_dp = C.POINTER(C.c_double)


class HeatRequest(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("steps", C.c_longlong),
                ("precision", C.c_int), ("cfg", C.c_int), ("seed", C.c_uint64),
                ("field_out", C.c_void_p)]


class HeatResult(C.Structure):
    _fields_ = [("id", C.c_uint64), ("status", C.c_int), ("l2", C.c_double), ("checksum", C.c_double),
                ("submit_ms", C.c_double), ("admit_ms", C.c_double), ("done_ms", C.c_double),
                ("updates", C.c_double)]


class HeatTuneEntry(C.Structure):
    _fields_ = [("kchunk", C.c_int), ("rows", C.c_int), ("blocks_per_sm", C.c_int), ("depth", C.c_int)]


class HeatServerStats(C.Structure):
    _fields_ = [("submitted", C.c_longlong), ("admitted", C.c_longlong), ("completed", C.c_longlong),
                ("rejected", C.c_longlong), ("resident", C.c_longlong), ("queued", C.c_longlong),
                ("p50_ms", C.c_double), ("p99_ms", C.c_double), ("mean_ms", C.c_double),
                ("max_ms", C.c_double), ("glups", C.c_double), ("updates", C.c_double),
                ("busy_ms", C.c_double), ("budget_bytes", C.c_size_t), ("bytes_in_use", C.c_size_t),
                ("peak_bytes", C.c_size_t), ("batch_steps", C.c_longlong),
                ("kernel_launches", C.c_longlong), ("gpu_ms", C.c_double)]

# Every symbol include/heat.h declares, with its ctypes signature.
SIGNATURES = {
    "heat_init": (C.c_int, [C.POINTER(C.c_void_p), C.POINTER(HeatDesc)]),
    "heat_step": (C.c_int, [C.c_void_p, C.c_int]),
    "heat_run": (C.c_int, [C.c_void_p, C.c_double, C.POINTER(C.c_int)]),
    "heat_norm": (C.c_int, [C.c_void_p, _dp, _dp]),
    "heat_get_field": (C.c_int, [C.c_void_p, C.c_void_p]),
    "heat_set_field": (C.c_int, [C.c_void_p, C.c_void_p]),
    "heat_sync": (C.c_int, [C.c_void_p]),
    "heat_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong)]),
    "heat_destroy": (C.c_int, [C.c_void_p]),
    "heat_strerror": (C.c_char_p, [C.c_int]),
    "heat_update": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                              C.c_int, C.c_int, C.c_int, C.c_double, C.c_int]),
    "heat_update_async": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                    C.c_int, C.c_int, C.c_int, C.c_double, C.c_void_p]),
    "heat_norm_noalloc": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, _dp, _dp, C.c_void_p]),
    "heat_batch_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_void_p, C.c_uint]),
    "heat_batch_add": (C.c_int, [C.c_void_p, C.c_void_p, C.c_longlong]),
    "heat_batch_remove": (C.c_int, [C.c_void_p, C.c_void_p]),
    "heat_batch_pending": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_longlong)]),
    "heat_batch_run": (C.c_int, [C.c_void_p, C.c_longlong, C.POINTER(C.c_longlong)]),
    "heat_batch_stats": (C.c_int, [C.c_void_p, C.POINTER(C.c_longlong), C.POINTER(C.c_longlong),
                                   C.POINTER(C.c_longlong)]),
    "heat_batch_destroy": (C.c_int, [C.c_void_p]),
    "heat_tune_batch": (C.c_int, [C.c_int, C.c_uint, C.c_int, C.c_int]),
    "heat_tune_lookup": (C.c_int, [C.c_int, C.c_uint, C.c_int, C.POINTER(C.c_int)]),
    "heat_tune_choice": (C.c_int, [C.c_int, C.c_uint, C.c_int, C.POINTER(HeatTuneEntry)]),
    "heat_server_create": (C.c_int, [C.POINTER(C.c_void_p), C.c_size_t, C.c_int, C.c_int]),
    "heat_server_submit": (C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_uint64)]),
    "heat_server_poll": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_int)]),
    "heat_server_wait_idle": (C.c_int, [C.c_void_p]),
    "heat_server_stats": (C.c_int, [C.c_void_p, C.c_void_p]),
    "heat_server_destroy": (C.c_int, [C.c_void_p]),
    "heat_inputs_reference": (C.c_int, [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, _dp, _dp]),
    "heat_inputs_config": (C.c_int, [C.c_int, C.c_uint64, C.c_int, C.c_int, C.c_int,
                                     C.c_void_p, C.c_void_p, _dp, _dp]),
    # include/heat_diag.h
    "heat_diag_fp64_rate": (C.c_int, [_dp]),
    "heat_diag_field_diff": (C.c_int, [C.c_void_p, C.c_void_p, _dp, _dp]),
    "heat_diag_wait_timeout": (C.c_int, [C.c_uint, C.POINTER(C.c_int)]),
    "heat_diag_fp32c_timeout": (C.c_int, [C.c_void_p]),
    "heat_diag_fp64_timeout": (C.c_int, [C.c_void_p]),
}


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    lib = C.CDLL(str(path or LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


_LIB: C.CDLL | None = None


def lib() -> C.CDLL:
    global _LIB
    if _LIB is None:
        _LIB = load()
    return _LIB


def check(status: int, what: str) -> None:
    if status != HEAT_OK:
        raise HeatError(what, status, lib().heat_strerror(status).decode())


def _ptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data


def inputs_reference(n: int):
    """The reference's own initial data for an n^3 grid: (kappa, rhs, u0, h, dt)."""
    shape = (n, n, n)
    kappa, rhs, u0 = (np.empty(shape) for _ in range(3))
    h, dt = C.c_double(), C.c_double()
    check(lib().heat_inputs_reference(n, _ptr(kappa), _ptr(rhs), _ptr(u0), C.byref(h), C.byref(dt)),
          "heat_inputs_reference")
    return kappa, rhs, u0, h.value, dt.value


def inputs_config(cfg: int, seed: int, nx: int, ny: int, nz: int):
    """Seeded synthetic inputs of configuration cfg: (kappa, u0, h, dt), shape (nz, ny, nx)."""
    kappa, u0 = np.empty((nz, ny, nx)), np.empty((nz, ny, nx))
    h, dt = C.c_double(), C.c_double()
    check(lib().heat_inputs_config(cfg, seed, nx, ny, nz, _ptr(kappa), _ptr(u0), C.byref(h), C.byref(dt)),
          "heat_inputs_config")
    return kappa, u0, h.value, dt.value


def fp64_rate() -> float:
    """Measured FP64 FMA rate of the current device, Gop/s."""
    g = C.c_double()
    check(lib().heat_diag_fp64_rate(C.byref(g)), "heat_diag_fp64_rate")
    return g.value


def field_diff(a: "Solver", b: "Solver") -> tuple[float, float]:
    """(max |a-b|, ||a-b|| / ||b||) of two solvers' current fields, on the device."""
    mx, rl = C.c_double(), C.c_double()
    check(lib().heat_diag_field_diff(a._ctx, b._ctx, C.byref(mx), C.byref(rl)), "heat_diag_field_diff")
    return mx.value, rl.value


class Solver:
    """One heat_ctx: device-resident fields advanced by heat_step / heat_run."""

    def __init__(self, kappa: np.ndarray, u0: np.ndarray, h: float, dt: float,
                 rhs: np.ndarray | None = None, precision: int = HEAT_FP64,
                 flags: int = 0, stream: int | None = None):
        kappa = np.ascontiguousarray(kappa, dtype=np.float64)
        u0 = np.ascontiguousarray(u0, dtype=np.float64)
        if rhs is not None:
            rhs = np.ascontiguousarray(rhs, dtype=np.float64)
        if kappa.ndim != 3 or kappa.shape != u0.shape or (rhs is not None and rhs.shape != u0.shape):
            raise ValueError("kappa, u0 (and rhs) must be 3-D arrays of one shape (nz, ny, nx)")
        self.shape = u0.shape
        nz, ny, nx = self.shape
        d = HeatDesc(nx, ny, nz, h, dt, _ptr(kappa), _ptr(u0), _ptr(rhs), precision, flags, stream)
        self._ctx = C.c_void_p()
        check(lib().heat_init(C.byref(self._ctx), C.byref(d)), "heat_init")

    def step(self, nsteps: int) -> None:
        check(lib().heat_step(self._ctx, nsteps), "heat_step")

    def run(self, T: float) -> int:
        s = C.c_int()
        check(lib().heat_run(self._ctx, T, C.byref(s)), "heat_run")
        return s.value

    def norm(self) -> tuple[float, float]:
        l2, cs = C.c_double(), C.c_double()
        check(lib().heat_norm(self._ctx, C.byref(l2), C.byref(cs)), "heat_norm")
        return l2.value, cs.value

    def field(self, out: np.ndarray | None = None) -> np.ndarray:
        if out is None:
            out = np.empty(self.shape)
        check(lib().heat_get_field(self._ctx, _ptr(out)), "heat_get_field")
        return out

    def set_field(self, u: np.ndarray) -> None:
        u = np.ascontiguousarray(u, dtype=np.float64)
        check(lib().heat_set_field(self._ctx, _ptr(u)), "heat_set_field")

    def sync(self) -> None:
        check(lib().heat_sync(self._ctx), "heat_sync")

    def stats(self) -> tuple[int, int]:
        s, k = C.c_longlong(), C.c_longlong()
        check(lib().heat_stats(self._ctx, C.byref(s), C.byref(k)), "heat_stats")
        return s.value, k.value

    def close(self) -> None:
        if self._ctx:
            lib().heat_destroy(self._ctx)
            self._ctx = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """heat_batch: contexts advanced together by one persistent launch per step."""

    def __init__(self, stream: int | None = None, graphs: bool = True, flags: int = 0):
        self._b = C.c_void_p()
        fl = flags | (0 if graphs else HEAT_BATCH_NO_GRAPHS)
        check(lib().heat_batch_create(C.byref(self._b), stream, fl), "heat_batch_create")

    def add(self, solver: Solver, steps: int) -> None:
        check(lib().heat_batch_add(self._b, solver._ctx, steps), "heat_batch_add")

    def remove(self, solver: Solver) -> None:
        check(lib().heat_batch_remove(self._b, solver._ctx), "heat_batch_remove")

    def pending(self, solver: Solver) -> int:
        n = C.c_longlong()
        check(lib().heat_batch_pending(self._b, solver._ctx, C.byref(n)), "heat_batch_pending")
        return n.value

    def run(self, max_steps: int = -1) -> int:
        n = C.c_longlong()
        check(lib().heat_batch_run(self._b, max_steps, C.byref(n)), "heat_batch_run")
        return n.value

    def stats(self) -> tuple[int, int, int]:
        a, g, s = C.c_longlong(), C.c_longlong(), C.c_longlong()
        check(lib().heat_batch_stats(self._b, C.byref(a), C.byref(g), C.byref(s)), "heat_batch_stats")
        return a.value, g.value, s.value

    def close(self) -> None:
        if self._b:
            lib().heat_batch_destroy(self._b)
            self._b = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tune_batch(precision: int = HEAT_FP64, flags: int = 0, max_nz: int = 0, force: bool = False) -> None:
    check(lib().heat_tune_batch(precision, flags, max_nz, int(force)), "heat_tune_batch")


def tune_lookup(precision: int, flags: int, nz: int) -> int:
    k = C.c_int()
    check(lib().heat_tune_lookup(precision, flags, nz, C.byref(k)), "heat_tune_lookup")
    return k.value


def tune_choice(precision: int, flags: int, nz: int) -> dict:
    """The batch's choices for a grid of depth nz: kchunk, rows, blocks_per_sm, depth."""
    e = HeatTuneEntry()
    check(lib().heat_tune_choice(precision, flags, nz, C.byref(e)), "heat_tune_choice")
    return {k: getattr(e, k) for k, _ in HeatTuneEntry._fields_}


class Server:
    """heat_server: continuous-batching solves under an HBM budget."""

    def __init__(self, budget_bytes: int, tick_steps: int = 64, prep_threads: int = 4):
        self._s = C.c_void_p()
        self._keep = {}
        check(lib().heat_server_create(C.byref(self._s), budget_bytes, tick_steps, prep_threads),
              "heat_server_create")

    def submit(self, nx: int, ny: int, nz: int, steps: int, precision: int = HEAT_FP64,
               cfg: int = 0, seed: int = 0, field_out: np.ndarray | None = None) -> int:
        if field_out is not None:
            assert field_out.shape == (nz, ny, nx) and field_out.dtype == np.float64
            assert field_out.flags.c_contiguous
        r = HeatRequest(nx, ny, nz, steps, precision, cfg, seed,
                        None if field_out is None else field_out.ctypes.data)
        rid = C.c_uint64()
        check(lib().heat_server_submit(self._s, C.byref(r), C.byref(rid)), "heat_server_submit")
        if field_out is not None:
            self._keep[rid.value] = field_out
        return rid.value

    def poll(self, max_results: int = 1024) -> list[dict]:
        buf = (HeatResult * max_results)()
        n = C.c_int()
        check(lib().heat_server_poll(self._s, buf, max_results, C.byref(n)), "heat_server_poll")
        out = []
        for r in buf[: n.value]:
            out.append({k: getattr(r, k) for k, _ in HeatResult._fields_})
            self._keep.pop(r.id, None)
        return out

    def wait_idle(self) -> None:
        check(lib().heat_server_wait_idle(self._s), "heat_server_wait_idle")

    def stats(self) -> dict:
        st = HeatServerStats()
        check(lib().heat_server_stats(self._s, C.byref(st)), "heat_server_stats")
        return {k: getattr(st, k) for k, _ in HeatServerStats._fields_}

    def close(self) -> None:
        if self._s:
            lib().heat_server_destroy(self._s)
            self._s = C.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
