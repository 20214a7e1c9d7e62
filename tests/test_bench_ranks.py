"""bench.py's N > 1 path on CPU: world-size-2 gloo ranks.  Each rank runs an
independent replica (the solver does not shard), the job's time is the
slowest rank's, and the value is every rank's updates over that time; the
reference arm runs on rank 0 only."""
from __future__ import annotations

import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, q) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = bench.max_over_ranks(10.0 + 5.0 * rank, dist, "cpu")
        v = bench.replica_value(1e9, world, t)
        q.put((rank, t, v))
    finally:
        dist.destroy_process_group()


def test_slowest_rank_sets_the_time_and_value_counts_all_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    world, port = 2, _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    assert [g[1] for g in got] == [15.0, 15.0]
    assert all(g[2] == pytest.approx(2 * 1e9 / 15.0 / 1e9) for g in got)


def test_single_process_needs_no_group():
    assert bench.max_over_ranks(3.5, None, "cpu") == 3.5
    assert bench.replica_value(2e9, 1, 2.0) == pytest.approx(1.0)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setattr("sys.argv", ["bench.py", "--impl", "reference", "--gpus", "2"])
    assert bench.reference_arm(bench.parse()) == 0
