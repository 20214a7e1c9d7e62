"""FP32C two-steps-per-launch kernel (TMA-staged plane tiles, temporal
blocking): bit-identical to one step per launch for every geometry, odd step
counts (a trailing single step), and it really takes the paired path."""
from __future__ import annotations

import pytest

from conftest import bits_equal

pytestmark = pytest.mark.gpu

SHAPES = [(3, 3, 3), (4, 5, 6), (33, 17, 9), (64, 48, 40), (130, 67, 21), (40, 40, 200),
          (97, 35, 50), (300, 20, 12)]


@pytest.fixture(scope="module")
def H(heat, cuda_device):
    return heat


@pytest.mark.parametrize("shape", SHAPES, ids=lambda s: "x".join(map(str, s)))
def test_two_step_equals_single_steps(H, shape):
    nx, ny, nz = shape
    kappa, u0, h, dt = H.inputs_config(2 if nx > 8 else 0, 13, nx, ny, nz)
    for steps in (2, 7, 24):
        with H.Solver(kappa, u0, h, dt, precision=H.HEAT_FP32C) as a, \
                H.Solver(kappa, u0, h, dt, precision=H.HEAT_FP32C, flags=H.HEAT_NO_TEMPORAL) as b:
            _, la0 = a.stats()
            a.step(steps)
            b.step(steps)
            a.sync()
            _, la1 = a.stats()
            assert la1 - la0 == steps // 2 + steps % 2   # paired launches taken
            assert bits_equal(a.field(), b.field()), steps
            assert a.norm() == b.norm()


def test_two_step_keeps_boundary(H):
    import numpy as np
    nx, ny, nz = 50, 41, 37
    kappa, u0, h, dt = H.inputs_config(0, 3, nx, ny, nz)
    u0 = u0.copy()
    bnd = np.ones(u0.shape, dtype=bool)
    bnd[1:-1, 1:-1, 1:-1] = False
    u0[bnd] = 0.75
    with H.Solver(kappa, u0, h, dt, precision=H.HEAT_FP32C) as s:
        f0 = s.field()
        s.step(10)
        f = s.field()
    assert np.array_equal(f[bnd], f0[bnd])
