"""heat_norm_noalloc: the allocation-free norm for callers that must not call
cudaMalloc/cudaFree while they run (a serving loop whose HBM is all committed,
or a monitoring hook between time steps that cannot take the device-wide stall
of an allocation).  Its scratch is a static device array, so it needs no
context; these tests check it through the C ABI against heat_norm, the entry
point that uses a context's allocated scratch, to the norm tolerance the other
tests use (1e-13 relative), on two calls in a row.

The file is named to be collected last, so a run that stops at the first
failure has run every other test before this one.  It also passes alone in a
fresh process (the first call on the device sets the scratch address up).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NORM_REL = 1e-13


@pytest.fixture(scope="module")
def H(heat, cuda_device):
    return heat


def noalloc_norm(H, t):
    """Call heat_norm_noalloc on a CUDA tensor of shape (nz, ny, nx)."""
    nz, ny, nx = t.shape
    l2, cs = C.c_double(), C.c_double()
    H.check(H.lib().heat_norm_noalloc(t.data_ptr(), nz, ny, nx, C.byref(l2), C.byref(cs), None),
            "heat_norm_noalloc")
    return l2.value, cs.value


def ctx_norm(H, field):
    """heat_norm of a context whose current field is `field`."""
    nz, ny, nx = field.shape
    kappa = np.ones_like(field)
    with H.Solver(kappa, field, 1.0 / (max(field.shape) - 1), 1e-6) as s:
        return s.norm()


@pytest.mark.parametrize("cfg,shape", [(0, (33, 45, 70)), (1, (64, 64, 64)), (2, (5, 97, 130))])
def test_noalloc_matches_heat_norm_twice(H, cuda_device, cfg, shape):
    torch = cuda_device
    nz, ny, nx = shape
    _, u0, _, _ = H.inputs_config(cfg, 31, nx, ny, nz)
    l2_ref, cs_ref = ctx_norm(H, u0)
    t = torch.from_numpy(u0).cuda()
    first = noalloc_norm(H, t)
    second = noalloc_norm(H, t)
    for l2, cs in (first, second):
        assert l2 == pytest.approx(l2_ref, rel=NORM_REL)
        assert cs == pytest.approx(cs_ref, rel=NORM_REL)
    assert first == second


def test_noalloc_follows_the_latest_field(H, cuda_device):
    """The shared scratch keeps the previous call's contents; a call on another
    field (fewer planes) must not see them."""
    torch = cuda_device
    _, big, _, _ = H.inputs_config(0, 1, 40, 40, 90)
    _, small, _, _ = H.inputs_config(0, 2, 40, 40, 7)
    tb, ts = torch.from_numpy(big).cuda(), torch.from_numpy(small).cuda()
    noalloc_norm(H, tb)
    got = noalloc_norm(H, ts)
    ref = ctx_norm(H, small)
    assert got[0] == pytest.approx(ref[0], rel=NORM_REL)
    assert got[1] == pytest.approx(ref[1], rel=NORM_REL)


def test_noalloc_after_time_steps(H, cuda_device):
    torch = cuda_device
    kappa, u0, h, dt = H.inputs_config(1, 5, 48, 40, 36)
    with H.Solver(kappa, u0, h, dt) as s:
        s.step(25)
        l2_ref, cs_ref = s.norm()
        field = s.field()
    t = torch.from_numpy(field).cuda()
    for _ in range(2):
        l2, cs = noalloc_norm(H, t)
        assert l2 == pytest.approx(l2_ref, rel=NORM_REL)
        assert cs == pytest.approx(cs_ref, rel=NORM_REL)


def test_noalloc_rejects_fields_beyond_its_scratch(H, cuda_device):
    torch = cuda_device
    t = torch.zeros(4, dtype=torch.float64, device="cuda")
    l2, cs = C.c_double(), C.c_double()
    too_many = 16384 + 1   # HEAT_NORM_NOALLOC_MAX_NZ + 1
    rc = H.lib().heat_norm_noalloc(t.data_ptr(), too_many, 1, 1, C.byref(l2), C.byref(cs), None)
    assert rc == H.HEAT_EINVAL
    assert H.lib().heat_norm_noalloc(None, 1, 1, 1, C.byref(l2), C.byref(cs), None) == H.HEAT_EINVAL
