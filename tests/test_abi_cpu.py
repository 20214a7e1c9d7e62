"""C ABI checks that need no GPU: the library loads, exports every symbol the
header declares, rejects bad arguments before touching a device, and its
host-side input generators behave as specified."""
from __future__ import annotations

import ctypes as C
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, bits_equal

HEADERS = sorted((ROOT / "include").glob("*.h"))


def declared_functions():
    names = []
    for h in HEADERS:
        text = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(heat_[a-z_0-9]+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_the_solver_abi():
    names = declared_functions()
    for n in ("heat_init", "heat_step", "heat_run", "heat_norm", "heat_update", "heat_destroy"):
        assert n in names


def test_library_exports_every_declared_symbol(heat):
    lib = heat.lib()
    out = subprocess.run(["nm", "-D", "--defined-only", str(heat.LIB_PATH)], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\sT\s(heat_[a-z_0-9]+)$", out, flags=re.M))
    missing = [n for n in declared_functions() if n not in exported]
    assert not missing, missing
    for n in declared_functions():
        assert getattr(lib, n) is not None
    assert set(declared_functions()) <= set(heat.SIGNATURES)


def test_strerror_covers_codes(heat):
    lib = heat.lib()
    for code in range(0, -8, -1):
        assert lib.heat_strerror(code)
    assert lib.heat_strerror(-99) == b"unknown status"


def test_init_rejects_bad_arguments_without_a_device(heat):
    lib = heat.lib()
    ctx = C.c_void_p()
    assert lib.heat_init(None, None) == heat.HEAT_EINVAL
    assert lib.heat_init(C.byref(ctx), None) == heat.HEAT_EINVAL
    k = np.ones((4, 4, 4))
    for nx, ny, nz, h, dt in [(2, 4, 4, 0.1, 0.01), (4, 4, 4, 0.0, 0.01), (4, 4, 4, 0.1, -1.0),
                              (4, 4, 4, float("nan"), 0.01)]:
        d = heat.HeatDesc(nx, ny, nz, h, dt, k.ctypes.data, k.ctypes.data, None, 0, 0, None)
        assert lib.heat_init(C.byref(ctx), C.byref(d)) == heat.HEAT_EINVAL
    d = heat.HeatDesc(4, 4, 4, 0.1, 0.01, None, k.ctypes.data, None, 0, 0, None)
    assert lib.heat_init(C.byref(ctx), C.byref(d)) == heat.HEAT_EINVAL
    assert lib.heat_step(None, 1) == heat.HEAT_EINVAL
    assert lib.heat_destroy(None) == heat.HEAT_EINVAL
    assert lib.heat_update(None, None, None, None, 4, 4, 4, 0.1, 0) in (heat.HEAT_EINVAL, heat.HEAT_ECUDA)
    # the bounded-wait check: no output pointer, no attempts, or more attempts than the
    # kernels' own limit are refused before any device is touched
    t = C.c_int(-1)
    assert lib.heat_diag_wait_timeout(10, None) == heat.HEAT_EINVAL
    assert lib.heat_diag_wait_timeout(0, C.byref(t)) == heat.HEAT_EINVAL
    assert lib.heat_diag_wait_timeout((1 << 22) + 1, C.byref(t)) == heat.HEAT_EINVAL
    assert t.value == -1


def test_reference_inputs_match_oracle_generator(heat, oracle):
    """The library's and the oracle build's copies of the generator agree."""
    a = heat.inputs_reference(13)
    b = oracle.inputs_reference(13)
    for x, y in zip(a[:3], b[:3]):
        assert bits_equal(x, y)
    assert a[3:] == b[3:]


@pytest.mark.parametrize("cfg", [0, 1, 2, 3, 4])
def test_config_inputs_properties(heat, cfg):
    nx, ny, nz = 13, 9, 11
    kappa, u0, h, dt = heat.inputs_config(cfg, 7, nx, ny, nz)
    assert kappa.shape == (nz, ny, nx)
    assert h == 1.0 / (max(nx, ny, nz) - 1)
    assert np.all(kappa > 0)
    assert dt == pytest.approx(0.9 * h * h / (6 * kappa.max()), rel=1e-15)
    b = np.ones_like(u0, dtype=bool)
    b[1:-1, 1:-1, 1:-1] = False
    assert np.all(u0[b] == 0.0)
    assert np.all(u0[~b] >= 0.0) and np.all(u0[~b] < 1.0 + 1e-15)
    k2, u2, _, _ = heat.inputs_config(cfg, 7, nx, ny, nz)
    assert bits_equal(kappa, k2) and bits_equal(u0, u2)
    k3, u3, _, _ = heat.inputs_config(cfg, 8, nx, ny, nz)
    assert not bits_equal(u0, u3)


def test_config0_distributions(heat):
    kappa, u0, h, dt = heat.inputs_config(0, 1, 64, 64, 64)
    g = np.log(kappa) / 0.5
    assert abs(g.mean()) < 0.01 and abs(g.std() - 1.0) < 0.01
    inner = u0[1:-1, 1:-1, 1:-1]
    assert abs(inner.mean() - 0.5) < 0.01 and abs(inner.var() - 1 / 12) < 0.005


def test_config1_fields(heat):
    n = 33
    kappa, u0, h, dt = heat.inputs_config(1, 5, n, n, n)
    x = np.arange(n) * h
    kk = 1 + 0.9 * np.sin(2 * np.pi * x)[None, None, :] * np.sin(4 * np.pi * x)[None, :, None] * \
        np.cos(2 * np.pi * x)[:, None, None]
    assert np.allclose(kappa, kk, rtol=0, atol=1e-14)
    k, j, i = np.unravel_index(np.argmax(u0), u0.shape)
    assert 0.25 <= i * h <= 0.75 and 0.25 <= j * h <= 0.75 and 0.25 <= k * h <= 0.75
    assert u0.max() > 0.3


def test_config2_kappa_is_smoothed(heat):
    kappa, u0, h, dt = heat.inputs_config(2, 2, 24, 24, 24)
    raw, _, _, _ = heat.inputs_config(0, 2, 24, 24, 24)
    # smoothing shrinks the spread of log kappa well below sigma = 1
    assert np.log(kappa).std() < 0.5
    assert np.all(np.isfinite(kappa))


def test_tune_choice_rejects_bad_arguments_without_a_device(heat):
    lib = heat.lib()
    e = heat.HeatTuneEntry()
    assert lib.heat_tune_choice(heat.HEAT_FP64, 0, 64, None) == heat.HEAT_EINVAL
    assert lib.heat_tune_choice(heat.HEAT_FP64, 0, 2, C.byref(e)) == heat.HEAT_EINVAL
    assert lib.heat_tune_choice(7, 0, 64, C.byref(e)) == heat.HEAT_EINVAL


def test_tune_choice_reads_a_written_cache(heat, tmp_path, monkeypatch):
    """The cache is read again when its path changes; entries written before
    rows / minb / depth existed read with the defaults."""
    cache = tmp_path / "t.json"
    cache.write_text('{"device": "x", "entries": [\n'
                     ' {"form": 3, "nz_max": 128, "kchunk": 24, "rows": 2, "minb": 3, "depth": 2, "glups": 1.0},\n'
                     ' {"form": 0, "nz_max": 128, "kchunk": 40, "glups": 1.0}\n]}\n')
    monkeypatch.setenv("HEAT_TUNE_CACHE", str(cache))
    assert heat.tune_choice(heat.HEAT_FP32C, 0, 100) == {"kchunk": 24, "rows": 2, "blocks_per_sm": 3,
                                                        "depth": 2}
    assert heat.tune_choice(heat.HEAT_FP64, 0, 100) == {"kchunk": 40, "rows": 1, "blocks_per_sm": 3,
                                                       "depth": 1}
    assert heat.tune_lookup(heat.HEAT_FP64, 0, 100) == 40
    # another class of the same cache, not tuned: the defaults
    assert heat.tune_choice(heat.HEAT_FP32C, 0, 300) == {"kchunk": 32, "rows": 1, "blocks_per_sm": 4,
                                                        "depth": 1}


def test_bench_reads_the_traffic_record():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench", ROOT / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    t, src = bench.profile_traffic(510 ** 3)
    assert src and 30 < src["bytes_per_update"] < 60
    assert t == pytest.approx(src["bytes_per_update"] * 510 ** 3, rel=1e-3)


def test_bench_fp64_pipe_record():
    """The FP64-pipe rows of the default form: (j - 1) mod 8 < 4 of the interior
    rows, 7 operations per point."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench", ROOT / "bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    r = bench.fp64_pipe_record(10, 1.0, 100.0)  # interior rows 1..8: rows 1-4 on the FP64 pipe
    assert r["ops_per_launch"] == 8 * 8 * 4 * 7
    assert r["fp64_row_share"] == 0.5
    r = bench.fp64_pipe_record(512, 1.0, 500.0)  # 510 rows: 63 full groups of 8 and 6 more
    assert r["ops_per_launch"] == 510 * 510 * (63 * 4 + 4) * 7
    assert r["frac"] == pytest.approx(r["achieved_gops"] / 500.0, rel=1e-3)
