"""Edge cases of the default FP64 form's integer-pipe kernel: signed data,
subnormal and non-finite values, and the fall-back to the FP64-pipe kernel
when the fixed-point range check fails (a time step above the stability
limit)."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import metrics

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def H(heat, cuda_device):
    return heat


def run(H, kappa, u0, h, dt, steps, flags=0, rhs=None):
    with H.Solver(kappa, u0, h, dt, rhs=rhs, flags=flags) as s:
        s.step(steps)
        return s.field()


def test_signed_fields_and_source(H, oracle):
    nx, ny, nz = 45, 38, 29
    kappa, u0, h, dt = H.inputs_config(0, 21, nx, ny, nz)
    rng = np.random.default_rng(3)
    u0 = u0 * 2.0 - 1.0
    u0[0, :, :] = u0[-1, :, :] = 0.0
    rhs = rng.uniform(-1e-3, 1e-3, u0.shape)
    ref = oracle.steps(u0, kappa, h, dt, 40, rhs=rhs)
    for fl in (0, 4):
        m = metrics(ref, run(H, kappa, u0, h, dt, 40, flags=fl, rhs=rhs))
        assert m["max_rel"] <= 1e-12 or m["max_abs"] <= 1e-15, (fl, m)
        assert m["rel_l2"] <= 1e-13, (fl, m)


def test_wide_dynamic_range(H, oracle):
    """Neighbouring values 300 binary orders apart and exact zeros."""
    nx = ny = nz = 24
    kappa, u0, h, dt = H.inputs_config(0, 5, nx, ny, nz)
    rng = np.random.default_rng(9)
    u0 = u0 * np.exp2(rng.integers(-300, 40, u0.shape)).astype(np.float64)
    u0[rng.random(u0.shape) < 0.1] = 0.0
    u0[0], u0[-1], u0[:, 0], u0[:, -1], u0[:, :, 0], u0[:, :, -1] = 0, 0, 0, 0, 0, 0
    ref = oracle.steps(u0, kappa, h, dt, 5)
    got = run(H, kappa, u0, h, dt, 5)
    big = np.abs(ref) > 1e-200
    rel = np.abs(got[big] - ref[big]) / np.abs(ref[big])
    assert rel.max() <= 1e-13
    assert np.abs(got[~big] - ref[~big]).max() <= 1e-200 * 1e-12


def test_subnormal_values(H, oracle):
    nx = ny = nz = 12
    kappa, u0, h, dt = H.inputs_config(0, 6, nx, ny, nz)
    u0 = u0 * 1e-310          # every interior value subnormal
    ref = oracle.steps(u0, kappa, h, dt, 3)
    got = run(H, kappa, u0, h, dt, 3)
    assert np.abs(got - ref).max() <= 64 * 5e-324   # a few subnormal ulps per step


def test_non_finite_inputs_stay_non_finite(H, oracle):
    nx = ny = nz = 14
    kappa, u0, h, dt = H.inputs_config(0, 8, nx, ny, nz)
    u0 = u0.copy()
    u0[7, 7, 7] = np.nan
    u0[3, 9, 4] = np.inf
    ref = oracle.steps(u0, kappa, h, dt, 2)
    for fl in (0, 4):
        got = run(H, kappa, u0, h, dt, 2, flags=fl)
        assert np.array_equal(np.isfinite(got), np.isfinite(ref)), fl
        fin = np.isfinite(ref)
        assert metrics(ref[fin], got[fin])["max_rel"] <= 1e-12


def test_unstable_dt_falls_back_and_still_matches(H, oracle):
    """dt = 3x the stability limit: the fixed-point check fails, the context
    uses the FP64-pipe kernel; results still follow the reference (whose
    high-frequency modes grow) closely."""
    nx = ny = nz = 20
    kappa, u0, h, dt = H.inputs_config(0, 4, nx, ny, nz)
    dt3 = 3 * dt
    ref = oracle.steps(u0, kappa, h, dt3, 12)
    got = run(H, kappa, u0, h, dt3, 12)
    m = metrics(ref, got)
    assert m["rel_l2"] <= 1e-13, m


def test_integer_and_fp64_pipe_kernels_agree_closely(H):
    kappa, u0, h, dt = H.inputs_config(1, 3, 80, 72, 64)
    a = run(H, kappa, u0, h, dt, 200, flags=0)
    b = run(H, kappa, u0, h, dt, 200, flags=4)
    m = metrics(b, a)
    assert m["max_rel"] <= 1e-12 and m["rel_l2"] <= 1e-14, m
