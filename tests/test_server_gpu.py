"""Continuous-batching server: each request's result is the same alone and in
the mix (bit for bit: the batch runs the same column walks), the HBM budget is
respected and over-budget requests are rejected, and requests that arrive
while others are on the GPU join and finish without waiting for them."""
from __future__ import annotations

import random
import time

import numpy as np
import pytest

from conftest import bits_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def H(heat, cuda_device):
    return heat


def alone(H, nx, ny, nz, steps, precision, cfg, seed):
    kappa, u0, h, dt = H.inputs_config(cfg, seed, nx, ny, nz)
    with H.Solver(kappa, u0, h, dt, precision=precision) as s:
        s.step(steps)
        return s.norm(), s.field()


def test_alone_equals_mix(H):
    rng = random.Random(11)
    reqs = []
    for q in range(14):
        nx, ny, nz = (rng.randint(20, 90) for _ in range(3))
        reqs.append(dict(nx=nx, ny=ny, nz=nz, steps=rng.randint(5, 150), precision=q % 2,
                         cfg=0, seed=9000 + q))
    fields = {}
    with H.Server(budget_bytes=8 << 30, tick_steps=16, prep_threads=3) as srv:
        ids = []
        for q, r in enumerate(reqs):
            out = np.empty((r["nz"], r["ny"], r["nx"])) if q % 3 == 0 else None
            rid = srv.submit(**r, field_out=out)
            ids.append(rid)
            if out is not None:
                fields[rid] = out
            time.sleep(0.002)
        srv.wait_idle()
        res = {x["id"]: x for x in srv.poll()}
        st = srv.stats()
    assert st["completed"] == len(reqs) and st["rejected"] == 0
    for rid, r in zip(ids, reqs):
        x = res[rid]
        assert x["status"] == 0
        (l2, cs), f = alone(H, r["nx"], r["ny"], r["nz"], r["steps"], r["precision"], r["cfg"], r["seed"])
        assert x["l2"] == l2 and x["checksum"] == cs, r
        if rid in fields:
            assert bits_equal(fields[rid], f)
        assert x["submit_ms"] <= x["admit_ms"] <= x["done_ms"]


def test_budget_is_respected_and_oversize_rejected(H):
    budget = 96 << 20
    with H.Server(budget_bytes=budget, tick_steps=8, prep_threads=2) as srv:
        big = srv.submit(160, 160, 160, 10, cfg=0, seed=1)          # needs > 96 MiB
        small = [srv.submit(40, 40, 40, 30, precision=q % 2, seed=2 + q) for q in range(12)]
        srv.wait_idle()
        res = {x["id"]: x for x in srv.poll()}
        st = srv.stats()
    assert res[big]["status"] == -5   # HEAT_EBUDGET
    assert all(res[s]["status"] == 0 for s in small)
    assert 0 < st["peak_bytes"] <= budget
    assert st["rejected"] == 1 and st["completed"] == 12


def test_arrivals_join_while_others_run(H):
    """A long solve is on the GPU; short requests submitted afterwards are
    admitted at the next tick and finish long before it."""
    with H.Server(budget_bytes=8 << 30, tick_steps=8, prep_threads=2) as srv:
        long_id = srv.submit(128, 128, 128, 4000, seed=5)
        while srv.stats()["admitted"] < 1:
            time.sleep(0.001)
        short = [srv.submit(32, 32, 32, 20, precision=q % 2, seed=50 + q) for q in range(6)]
        srv.wait_idle()
        res = {x["id"]: x for x in srv.poll()}
        st = srv.stats()
    t_long = res[long_id]["done_ms"]
    for s in short:
        assert res[s]["status"] == 0
        assert res[s]["admit_ms"] < t_long and res[s]["done_ms"] < t_long
    assert st["p50_ms"] <= st["p99_ms"] <= st["max_ms"]
    assert st["glups"] > 0 and st["batch_steps"] >= 4000


def test_submit_validation(H):
    with H.Server(budget_bytes=1 << 30) as srv:
        with pytest.raises(H.HeatError):
            srv.submit(2, 10, 10, 5)
        with pytest.raises(H.HeatError):
            srv.submit(10, 10, 10, 5, precision=7)
        srv.wait_idle()
