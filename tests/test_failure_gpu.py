"""Failure paths on the GPU, made without faulting, trapping or hanging it.

  - a bounded device-side wait gives up: an mbarrier that nothing arrives at,
    waited on with the TMA kernels' own bounded wait (capped at a few
    milliseconds), returns HEAT_ETIMEOUT, and the device stays usable;
  - the product FP32C two-step kernel, launched with its wait limit at 0
    attempts, gives up, flags its context and returns; heat_sync, heat_norm,
    heat_get_field and heat_batch_run each report HEAT_ETIMEOUT (once), the
    context's field is untouched, and solves after it still match the oracle;
  - the same for the default FP64 form's TMA-staged launch;
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


def fp32c_ctx(H):
    kappa, u0, h, dt = H.inputs_config(0, 7, 40, 36, 30)
    return H.Solver(kappa, u0, h, dt, precision=H.HEAT_FP32C), (kappa, u0, h, dt)


def test_product_kernel_timeout_reaches_every_sync_point(H, oracle):
    s, (kappa, u0, h, dt) = fp32c_ctx(H)
    with s:
        s.step(4)
        before = s.field()
        lib = H.lib()
        # heat_sync reports it, once
        assert lib.heat_diag_fp32c_timeout(s._ctx) == H.HEAT_OK
        assert lib.heat_sync(s._ctx) == H.HEAT_ETIMEOUT
        assert lib.heat_sync(s._ctx) == H.HEAT_OK
        # heat_norm
        assert lib.heat_diag_fp32c_timeout(s._ctx) == H.HEAT_OK
        l2, cs = C.c_double(), C.c_double()
        assert lib.heat_norm(s._ctx, C.byref(l2), C.byref(cs)) == H.HEAT_ETIMEOUT
        # heat_get_field: the copy is made, the status says the launch gave up
        assert lib.heat_diag_fp32c_timeout(s._ctx) == H.HEAT_OK
        out = np.empty_like(before)
        assert lib.heat_get_field(s._ctx, out.ctypes.data) == H.HEAT_ETIMEOUT
        assert bits_equal(out, before)  # the failed launch wrote nothing
        assert s.stats()[0] == 4
        # heat_batch_run of a batch holding the context
        assert lib.heat_diag_fp32c_timeout(s._ctx) == H.HEAT_OK
        with H.Batch() as b:
            b.add(s, 2)
            n = C.c_longlong()
            assert lib.heat_batch_run(b._b, -1, C.byref(n)) == H.HEAT_ETIMEOUT
            assert n.value == 2
            b.remove(s)
        s.sync()
        # the context keeps working: its next steps equal a fresh context's
        s.step(2)
        got = s.field()
    with H.Solver(kappa, u0, h, dt, precision=H.HEAT_FP32C) as ref:
        ref.step(8)
        assert bits_equal(got, ref.field())
    assert small_solve_matches_oracle(H, oracle)


def test_product_kernel_timeout_needs_the_two_step_form(H):
    kappa, u0, h, dt = H.inputs_config(0, 7, 20, 18, 16)
    with H.Solver(kappa, u0, h, dt) as s:
        assert H.lib().heat_diag_fp32c_timeout(s._ctx) == H.HEAT_ESTATE
    with H.Solver(kappa, u0, h, dt, precision=H.HEAT_FP32C, flags=H.HEAT_NO_TEMPORAL) as s:
        assert H.lib().heat_diag_fp32c_timeout(s._ctx) == H.HEAT_ESTATE


def test_default_fp64_kernel_timeout(H, oracle):
    """The TMA-staged default FP64 launch's own failure path: both warpgroups
    give up at their first wait, nothing is written, the status surfaces once,
    and the context's next steps equal a fresh context's."""
    kappa, u0, h, dt = H.inputs_config(1, 4, 70, 45, 38)
    with H.Solver(kappa, u0, h, dt) as s:
        s.step(3)
        before = s.field()
        lib = H.lib()
        assert lib.heat_diag_fp64_timeout(s._ctx) == H.HEAT_OK
        out = np.empty_like(before)
        assert lib.heat_get_field(s._ctx, out.ctypes.data) == H.HEAT_ETIMEOUT
        assert bits_equal(out, before)
        assert lib.heat_sync(s._ctx) == H.HEAT_OK
        assert lib.heat_diag_fp64_timeout(s._ctx) == H.HEAT_OK
        assert lib.heat_sync(s._ctx) == H.HEAT_ETIMEOUT
        s.step(4)
        got = s.field()
    with H.Solver(kappa, u0, h, dt) as ref:
        ref.step(7)
        assert bits_equal(got, ref.field())
    # the same launch with a source term (the reference problem)
    kappa, rhs, u0, h, dt = H.inputs_reference(40)
    with H.Solver(kappa, u0, h, dt, rhs=rhs) as s:
        s.step(2)
        before = s.field()
        assert lib.heat_diag_fp64_timeout(s._ctx) == H.HEAT_OK
        out = np.empty_like(before)
        assert lib.heat_get_field(s._ctx, out.ctypes.data) == H.HEAT_ETIMEOUT
        assert bits_equal(out, before)
        s.step(3)
        got = s.field()
    with H.Solver(kappa, u0, h, dt, rhs=rhs) as ref:
        ref.step(5)
        assert bits_equal(got, ref.field())
    with H.Solver(kappa, u0, h, dt, flags=H.HEAT_BITEXACT) as s:
        assert H.lib().heat_diag_fp64_timeout(s._ctx) == H.HEAT_ESTATE
    assert small_solve_matches_oracle(H, oracle)
