"""Batched persistent kernel: every grid's result in a batch equals its result
alone (heat_step on its own context) bit for bit, for every form, uneven
sizes, graphs on and off, incremental scheduling, and a context stepped
outside the batch; the autotuner writes and reads its JSON cache."""
from __future__ import annotations

import json
import random

import numpy as np
import pytest

from conftest import bits_equal

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def H(heat, cuda_device):
    return heat


FORMS = [("fp64", 0, 0), ("fp64-hw", 0, 4), ("bitexact", 0, 1), ("fp32c", 1, 0)]


def make(H, shape, seed, precision, flags, cfg=0):
    nx, ny, nz = shape
    kappa, u0, h, dt = H.inputs_config(cfg, seed, nx, ny, nz)
    return H.Solver(kappa, u0, h, dt, precision=precision, flags=flags)


def alone(H, shape, seed, precision, flags, steps, cfg=0):
    with make(H, shape, seed, precision, flags, cfg) as s:
        s.step(steps)
        return s.field()


def test_batch_equals_alone_all_forms(H):
    rng = random.Random(5)
    specs = []
    for idx, (_, prec, fl) in enumerate(FORMS * 2):
        shape = tuple(rng.randint(12, 70) for _ in range(3))
        specs.append((shape, 100 + idx, prec, fl, rng.randint(3, 41)))
    solvers = [make(H, sh, sd, p, f) for sh, sd, p, f, _ in specs]
    with H.Batch() as b:
        for s, spec in zip(solvers, specs):
            b.add(s, spec[4])
        taken = b.run()
        assert taken == max(sp[4] for sp in specs)
        launches, graphs, steps = b.stats()
        assert steps == taken and launches >= taken
    for s, (sh, sd, p, f, n) in zip(solvers, specs):
        assert bits_equal(s.field(), alone(H, sh, sd, p, f, n)), (sh, p, f, n)
        assert s.stats()[0] == n
        s.close()


@pytest.mark.parametrize("graphs,flags", [(True, 0), (False, 0), (True, 2), (True, 4), (False, 6)])
def test_graphs_and_launch_shapes_agree(H, graphs, flags):
    """graphs on/off, persistent blocks (2), serial kinds (4)."""
    shapes = [(40, 33, 66), (90, 20, 18), (17, 48, 35)]
    solvers = [make(H, sh, 9 + i, 0, 0) for i, sh in enumerate(shapes)]
    solvers[1].close()
    solvers[1] = make(H, shapes[1], 10, 1, 0)   # one FP32C grid: two kinds present
    with H.Batch(graphs=graphs, flags=flags) as b:
        for s in solvers:
            b.add(s, 37)
        b.run()
        _, g, _ = b.stats()
        assert (g > 0) == graphs
    for i, (s, sh) in enumerate(zip(solvers, shapes)):
        assert bits_equal(s.field(), alone(H, sh, 9 + i, 1 if i == 1 else 0, 0, 37))
        s.close()


def test_incremental_scheduling_and_outside_steps(H):
    sh = (36, 30, 28)
    a, c = make(H, sh, 1, 0, 0), make(H, sh, 2, 1, 0)
    with H.Batch() as b:
        b.add(a, 10)
        b.add(c, 25)
        assert b.run(max_steps=7) == 7
        assert b.pending(a) == 3 and b.pending(c) == 18
        a.step(5)            # stepped outside the batch: the batch must notice
        b.add(a, 4)          # a has 3 + 4 scheduled
        b.run()
        assert b.pending(a) == 0 and b.pending(c) == 0
        b.remove(c)
        b.add(a, 2)
        b.run()
    assert bits_equal(a.field(), alone(H, sh, 1, 0, 0, 10 + 5 + 4 + 2))
    assert bits_equal(c.field(), alone(H, sh, 2, 1, 0, 25))
    a.close()
    c.close()


def test_batch_with_source_term(H, oracle):
    kappa, rhs, u0, h, dt = H.inputs_reference(30)
    with H.Solver(kappa, u0, h, dt, rhs=rhs, flags=H.HEAT_BITEXACT) as s, H.Batch() as b:
        b.add(s, 21)
        b.run()
        assert bits_equal(s.field(), oracle.steps(u0, kappa, h, dt, 21, rhs=rhs))


def test_config3_like_batch(H):
    """Half FP64 default, half FP32C, uneven sizes and step counts."""
    rng = random.Random(2026)
    specs = []
    for g in range(12):
        shape = tuple(rng.randint(48, 112) for _ in range(3))
        specs.append((shape, 500 + g, g % 2, 0, rng.randint(20, 90)))
    solvers = [make(H, sh, sd, p, f) for sh, sd, p, f, _ in specs]
    with H.Batch() as b:
        for s, sp in zip(solvers, specs):
            b.add(s, sp[4])
        b.run()
    for s, (sh, sd, p, f, n) in zip(solvers, specs):
        assert bits_equal(s.field(), alone(H, sh, sd, p, f, n))
        s.close()


def test_tuner_cache(H, tmp_path, monkeypatch):
    cache = tmp_path / "tune.json"
    monkeypatch.setenv("HEAT_TUNE_CACHE", str(cache))
    H.tune_batch(H.HEAT_FP32C, 0, max_nz=64, force=True)
    doc = json.loads(cache.read_text())
    ent = [e for e in doc["entries"] if e["form"] == 3 and e["nz_max"] == 64]
    assert ent and ent[0]["kchunk"] >= 1 and ent[0]["glups"] > 0
    e = ent[0]
    assert e["rows"] in (1, 2) and e["minb"] in (2, 3, 4) and e["depth"] in (1, 2)
    assert H.tune_lookup(H.HEAT_FP32C, 0, 40) == e["kchunk"]
    assert H.tune_choice(H.HEAT_FP32C, 0, 40) == {"kchunk": e["kchunk"], "rows": e["rows"],
                                                   "blocks_per_sm": e["minb"], "depth": e["depth"]}
    # the default FP64 form as well (its own entries)
    H.tune_batch(H.HEAT_FP64, 0, max_nz=64, force=True)
    doc = json.loads(cache.read_text())
    ent = [e for e in doc["entries"] if e["form"] == 0 and e["nz_max"] == 64]
    assert ent and ent[0]["depth"] == 1
    assert H.tune_choice(H.HEAT_FP64, 0, 64)["blocks_per_sm"] == ent[0]["minb"]


def write_cache(path, kchunk, rows, minb, depth):
    """A tuning cache with the same choices for every form and size class."""
    lines = [f' {{"form": {f}, "nz_max": {c}, "kchunk": {kchunk}, "rows": {rows}, "minb": {minb}, '
             f'"depth": {depth}, "glups": 1.0}}'
             for f in range(6) for c in (64, 128, 256, 384)]
    path.write_text('{"device": "test", "entries": [\n' + ",\n".join(lines) + "\n]}\n")


@pytest.mark.parametrize("kchunk,rows,minb,depth", [(16, 2, 2, 2), (8, 1, 3, 1), (64, 2, 4, 2),
                                                    (32, 1, 4, 1)])
@pytest.mark.parametrize("graphs", [True, False])
def test_tuned_variants_equal_alone(H, tmp_path, monkeypatch, kchunk, rows, minb, depth, graphs):
    """Every choice the autotuner can make -- z-chunk, rows per thread,
    blocks-per-SM variant, FP32C temporal depth 2 (the two-step TMA kernel on
    the table's tiles) -- leaves each grid's result bit-identical to its result
    alone, for every form, odd step counts and runs cut into uneven pieces."""
    cache = tmp_path / "tune.json"
    write_cache(cache, kchunk, rows, minb, depth)
    monkeypatch.setenv("HEAT_TUNE_CACHE", str(cache))
    assert H.tune_choice(H.HEAT_FP32C, 0, 40) == {"kchunk": kchunk, "rows": rows,
                                                   "blocks_per_sm": minb, "depth": depth}
    rng = random.Random(17 + kchunk)
    specs = []
    for idx, (_, prec, fl) in enumerate(FORMS * 2):
        shape = tuple(rng.randint(12, 72) for _ in range(3))
        specs.append((shape, 700 + idx, prec, fl, rng.choice([7, 16, 23, 40, 51])))
    solvers = [make(H, sh, sd, p, f) for sh, sd, p, f, _ in specs]
    with H.Batch(graphs=graphs) as b:
        for s, spec in zip(solvers, specs):
            b.add(s, spec[4])
        total = 0
        for piece in (5, 16, 1, 19, 2, 33, 100):
            total += b.run(piece)
        assert total == max(sp[4] for sp in specs)
    for s, (sh, sd, p, f, n) in zip(solvers, specs):
        assert bits_equal(s.field(), alone(H, sh, sd, p, f, n)), (sh, p, f, n)
        assert s.stats()[0] == n
        s.close()


@pytest.mark.parametrize("graphs", [True, False])
def test_solo_and_table_grids_mixed(H, monkeypatch, graphs):
    """Grids above the solo threshold step with their single-grid kernels
    (two FP32C steps per launch) beside the tile table; odd step counts and
    runs cut into uneven pieces exercise the buffer-swap bookkeeping and the
    graph-replay check.  Every grid equals its result alone."""
    monkeypatch.setenv("HEAT_BATCH_SOLO_POINTS", "30000")
    rng = random.Random(11)
    specs = []
    for idx, (_, prec, fl) in enumerate(FORMS * 2):
        big = idx % 2 == 0
        shape = tuple(rng.randint(36, 48) if big else rng.randint(10, 24) for _ in range(3))
        specs.append((shape, 300 + idx, prec, fl, rng.choice([17, 33, 40, 51, 64])))
    solvers = [make(H, sh, sd, p, f) for sh, sd, p, f, _ in specs]
    with H.Batch(graphs=graphs) as b:
        for s, spec in zip(solvers, specs):
            b.add(s, spec[4])
        total = 0
        for piece in (5, 16, 1, 19, 2, 33, 100):
            total += b.run(piece)
        assert total == max(sp[4] for sp in specs)
    for s, (sh, sd, p, f, n) in zip(solvers, specs):
        assert bits_equal(s.field(), alone(H, sh, sd, p, f, n)), (sh, p, f, n)
        assert s.stats()[0] == n
        s.close()
