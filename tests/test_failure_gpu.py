"""Failure paths on the GPU, made without faulting, trapping or hanging it.

  - a bounded device-side wait gives up: an mbarrier that nothing arrives at,
    waited on with the TMA kernels' own bounded wait (capped at a few
    milliseconds), returns HEAT_ETIMEOUT, and the device stays usable;
  - a context larger than the device returns HEAT_ENOMEM from its first device
    allocation (before any host data is read) and leaves nothing behind.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

from conftest import bits_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def H(heat, cuda_device):
    return heat


def small_solve_matches_oracle(H, oracle):
    kappa, u0, h, dt = H.inputs_config(0, 3, 17, 13, 11)
    with H.Solver(kappa, u0, h, dt, flags=H.HEAT_BITEXACT) as s:
        s.step(5)
        u = s.field()
    return bits_equal(u, oracle.steps(u0, kappa, h, dt, 5))


def test_bounded_wait_gives_up_and_the_device_stays_usable(H, oracle):
    timed_out = C.c_int(-1)
    st = H.lib().heat_diag_wait_timeout(1000, C.byref(timed_out))
    assert st == H.HEAT_ETIMEOUT and timed_out.value == 1
    assert small_solve_matches_oracle(H, oracle)


def test_bounded_wait_rejects_limits_above_the_kernels_own(H):
    timed_out = C.c_int(-1)
    assert H.lib().heat_diag_wait_timeout(0, C.byref(timed_out)) == H.HEAT_EINVAL
    assert H.lib().heat_diag_wait_timeout((1 << 22) + 1, C.byref(timed_out)) == H.HEAT_EINVAL


@pytest.mark.parametrize("precision", ["fp64", "fp32c"])
def test_context_larger_than_the_device_returns_enomem(H, oracle, precision):
    n = 5000  # 1 TB per FP64 field, 500 GB per FP32 one: the first allocation fails
    host = np.zeros(8)  # never read: heat_init allocates before it copies
    prec = H.HEAT_FP64 if precision == "fp64" else H.HEAT_FP32C
    d = H.HeatDesc(n, n, n, 1.0 / (n - 1), 1e-9, host.ctypes.data, host.ctypes.data, None, prec,
                   0, None)
    ctx = C.c_void_p()
    st = H.lib().heat_init(C.byref(ctx), C.byref(d))
    assert st == H.HEAT_ENOMEM and not ctx.value
    assert b"bytes" in H.lib().heat_strerror(st)
    assert small_solve_matches_oracle(H, oracle)
