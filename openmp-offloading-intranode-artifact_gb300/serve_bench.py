"""Configuration 4: a stream of solve requests served with continuous batching.

    python openmp-offloading-intranode-artifact_gb300/serve_bench.py [--requests 10000]
        [--rate 200] [--budget-gb 160] [--tick 32] [--seed 4]
        [--min-axis 32] [--max-axis 512] [--min-steps 50] [--max-steps 5000]

Requests arrive as a Poisson process at --rate per second; each axis is
log-uniform in [min-axis, max-axis], the step count log-uniform in
[min-steps, max-steps], the precision 50/50 FP64 default / FP32C, and each has
its own kappa/u0 seed (configuration-0 distributions).  Admission is by the
HBM budget with fields device-resident.  Prints one JSON line: offered load,
p50/p99/mean/max latency (submit to done), aggregate GLUP/s over the busy
span, and counts.  At the nominal rate the offered load exceeds one GPU's
throughput many times over, so latency there is queueing; run a lower --rate
for the sustainable operating point.
"""
from __future__ import annotations

import argparse
import json
import math
import random
import sys
import time
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent))
import heat_ctypes as H  # noqa: E402
from clocks import ClockSampler  # noqa: E402


def log_uniform(rng: random.Random, lo: float, hi: float) -> float:
    return math.exp(rng.uniform(math.log(lo), math.log(hi)))


def run(requests: int = 10000, rate: float = 200.0, budget_gb: float = 160.0, tick: int = 32,
        prep_threads: int = 4, seed: int = 4, min_axis: int = 32, max_axis: int = 512,
        min_steps: int = 50, max_steps: int = 5000, device: int = 0) -> dict:
    """Serve one Poisson request stream of configuration 4; returns the JSON record."""
    rng = random.Random(seed)
    reqs, t = [], 0.0
    for q in range(requests):
        t += rng.expovariate(rate)
        nx, ny, nz = (int(round(log_uniform(rng, min_axis, max_axis))) for _ in range(3))
        steps = int(round(log_uniform(rng, min_steps, max_steps)))
        reqs.append((t, nx, ny, nz, steps, H.HEAT_FP64 if rng.random() < 0.5 else H.HEAT_FP32C,
                     1_000_000 * seed + q))
    offered = sum((r[1] - 2) * (r[2] - 2) * (r[3] - 2) * r[4] for r in reqs)
    span = reqs[-1][0] if reqs else 0.0

    srv = H.Server(budget_bytes=int(budget_gb * (1 << 30)), tick_steps=tick,
                   prep_threads=prep_threads)
    with ClockSampler(device) as clk:
        t0 = time.perf_counter()
        for (ta, nx, ny, nz, steps, prec, sd) in reqs:
            delay = ta - (time.perf_counter() - t0)
            if delay > 0:
                time.sleep(delay)
            srv.submit(nx, ny, nz, steps, precision=prec, cfg=0, seed=sd)
        srv.wait_idle()
        wall = time.perf_counter() - t0
    res = srv.poll(max_results=requests + 16)
    st = srv.stats()
    srv.close()
    lat64 = sorted(x["done_ms"] - x["submit_ms"] for x, r in zip(sorted(res, key=lambda x: x["id"]), reqs)
                   if r[5] == H.HEAT_FP64 and x["status"] == 0)
    lat32 = sorted(x["done_ms"] - x["submit_ms"] for x, r in zip(sorted(res, key=lambda x: x["id"]), reqs)
                   if r[5] == H.HEAT_FP32C and x["status"] == 0)
    pct = lambda v, p: v[min(len(v) - 1, int(round(p * (len(v) - 1))))] if v else None
    return {"workload": f"config4: {requests} requests, Poisson {rate}/s, axes log-U[{min_axis},"
                        f"{max_axis}], steps log-U[{min_steps},{max_steps}], 50/50 FP64/FP32C, "
                        f"budget {budget_gb} GB, tick {tick}",
            "offered_updates": offered, "arrival_span_s": round(span, 2),
            "offered_glups": round(offered / span / 1e9, 1) if span > 0 else None,
            "wall_s": round(wall, 2), "p50_ms": round(st["p50_ms"], 2), "p99_ms": round(st["p99_ms"], 2),
            "mean_ms": round(st["mean_ms"], 2), "max_ms": round(st["max_ms"], 2),
            "p50_ms_fp64": pct(lat64, 0.5), "p99_ms_fp64": pct(lat64, 0.99),
            "p50_ms_fp32c": pct(lat32, 0.5), "p99_ms_fp32c": pct(lat32, 0.99),
            "glups": round(st["glups"], 2), "completed": st["completed"], "rejected": st["rejected"],
            "peak_gb": round(st["peak_bytes"] / (1 << 30), 2), "batch_steps": st["batch_steps"],
            "kernel_launches": st["kernel_launches"],
            "gpu_busy_frac": round(st["gpu_ms"] * 1e-3 / wall, 3) if wall > 0 else None,
            "clocks": clk.summary()}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--requests", type=int, default=10000)
    ap.add_argument("--rate", type=float, default=200.0)
    ap.add_argument("--budget-gb", type=float, default=160.0)
    ap.add_argument("--tick", type=int, default=32)
    ap.add_argument("--prep-threads", type=int, default=4)
    ap.add_argument("--seed", type=int, default=4)
    ap.add_argument("--min-axis", type=int, default=32)
    ap.add_argument("--max-axis", type=int, default=512)
    ap.add_argument("--min-steps", type=int, default=50)
    ap.add_argument("--max-steps", type=int, default=5000)
    a = ap.parse_args()
    out = run(a.requests, a.rate, a.budget_gb, a.tick, a.prep_threads, a.seed, a.min_axis,
              a.max_axis, a.min_steps, a.max_steps)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
