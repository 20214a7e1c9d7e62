"""Benchmark: the FP64 plain heat stencil on the 512^3 configuration.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (one bench "step"): one 512^3 solve of 1,000 explicit time steps with
the configuration-1 fields (smooth kappa = 1 + 0.9 sin(2 pi x) sin(4 pi y)
cos(2 pi z), Gaussian bump u0, zero Dirichlet boundary, dt = 0.9 of the
stability limit).  Metric: GLUP/s = (nx-2)(ny-2)(nz-2) * time steps / seconds.

  value : device-resident throughput of the default FP64 form through the C
          ABI (heat_step), timed with CUDA events on the solver's stream, max
          over ranks.  Each field is 1 GiB, far larger than the 129 MB L2, so
          no flush is needed between timed steps.
  e2e   : the same metric through the public ABI from pinned host buffers:
          heat_init (H2D of kappa and u0) + heat_step + heat_get_field (D2H of
          u) + heat_destroy, host wall clock.
  roofline, cpu_baseline, clocks, gpu_launches: see the keys' comments below.

--impl reference times the reference's CPU implementation of the loop (the
oracle restatement in the reference's operation order and OpenMP structure,
run on all host cores) on the same workload, a bounded number of time steps
per bench step.  With torchrun (N > 1) each rank runs an independent replica
of the solve on its own GPU (the solver does not shard: replicas only).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "openmp-offloading-intranode-artifact_gb300"
sys.path.insert(0, str(PKG))

from clocks import ClockSampler  # noqa: E402  (package module)

N = 512
TIME_STEPS = 1000
SEED = 1
CFG = 1
METRIC = "GLUP/s (FP64 plain heat stencil, 512^3, 1000 steps per solve)"
UNIT = "GLUP/s"
BYTES_PER_UPDATE = 24.0   # u read 8 + u write 8 + kappa read 8 (compulsory, FP64)
FP32C_BYTES_PER_UPDATE = 24.0  # one step: v 4+4, carry 2+2, three FP32 face weights 12
FP32C_BYTES_PER_UPDATE_TB2 = 12.0  # two steps per launch: the same 24 B per two updates
H100_1CUDA_N512 = 38.97   # reference 1-cuda, H100, N=512 (CUDA/summary.csv:2)


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--n", type=int, default=N)
    ap.add_argument("--time-steps", type=int, default=TIME_STEPS)
    ap.add_argument("--skip-cpu", action="store_true", help="omit the cpu_baseline leg")
    return ap.parse_args()


def updates(n, steps):
    return float((n - 2) ** 3) * steps


def workload(n, steps):
    return {"workload": f"config1: plain FP64 drop-in {n}^3, smooth kappa, Gaussian bump, "
                        f"zero Dirichlet, dt=0.9*stability, {steps} time steps per bench step",
            "nx": n, "ny": n, "nz": n, "time_steps_per_step": steps, "seed": SEED,
            "l2": "inputs larger than L2 (1 GiB per field), no flush"}


# ---------------------------------------------------------------- CPU legs
def cpu_threads():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


def run_oracle_cli(n, steps, threads):
    sys.path.insert(0, str(ROOT / "oracle"))
    import heat_oracle  # the checker / CPU baseline, never the measured product
    heat_oracle.ensure_built()
    env = {**os.environ, "OMP_NUM_THREADS": str(threads), "OMP_PROC_BIND": "spread",
           "OMP_PLACES": "cores"}
    r = subprocess.run([str(heat_oracle.CLI_PATH), "--config", str(CFG), "--n", str(n),
                        "--steps", str(steps), "--seed", str(SEED)],
                       capture_output=True, text=True, env=env, check=True)
    return json.loads(r.stdout.strip().splitlines()[-1])


def cpu_sample_steps(n, threads, budget_s):
    """Time steps whose CPU run lasts about budget_s (calibrated on 2 steps)."""
    probe = run_oracle_cli(n, 2, threads)
    per = max(probe["seconds"] / 2, 1e-6)
    return max(2, min(1000, int(budget_s / per)))


def cpu_baseline(n, threads):
    s = cpu_sample_steps(n, threads, 12.0)
    r = run_oracle_cli(n, s, threads)
    return {"value": round(r["glups"], 4), "unit": UNIT, "cores": r["threads"], "kind": "port",
            "sample": f"oracle restatement (reference operation order, OpenMP over k), config1 {n}^3, "
                      f"{s} time steps, {r['seconds']:.2f} s"}


def reference_arm(a):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    threads = cpu_threads()
    s = cpu_sample_steps(a.n, threads, 8.0)
    for _ in range(a.warmup):
        run_oracle_cli(a.n, max(2, s // 4), threads)
    vals, secs = [], 0.0
    for _ in range(a.steps):
        r = run_oracle_cli(a.n, s, threads)
        vals.append(r["glups"])
        secs += r["seconds"]
    v = statistics.median(vals)
    out = {"metric": METRIC, "value": round(v, 4), "unit": UNIT, "impl": "reference",
           "n_gpus": a.gpus, "steps": a.steps, "warmup": a.warmup,
           "ms_per_step": round(1e3 * secs / a.steps, 3), "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": workload(a.n, s),
           "cpu_baseline": {"value": round(v, 4), "unit": UNIT, "cores": threads, "kind": "port",
                            "sample": f"{s} time steps of config1 {a.n}^3 per bench step; the reference's "
                                      "serial solver is a fixed-problem x86 build here, so the oracle "
                                      "restatement of its loop runs the config"},
           "e2e": {"value": round(v, 4), "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    return 0


# ---------------------------------------------------------------- clocks
# ---------------------------------------------------------------- our arm
def profile_traffic():
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary."""
    p = ROOT / "profiles" / "fp64_default_512.md"
    if not p.exists():
        return None
    for ln in p.read_text().splitlines():
        if ln.startswith("traffic_bytes_per_launch:"):
            try:
                return float(ln.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def max_over_ranks(x, dist, device):
    """The largest of every rank's x (the slowest rank's time); x itself
    without a process group."""
    if dist is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(updates_per_rank, world, t_max_s):
    """Whole-job GLUP/s of `world` independent replicas: every rank's updates
    over the slowest rank's time."""
    return updates_per_rank * world / t_max_s / 1e9


def our_arm(a):
    import numpy as np
    import torch
    import heat_ctypes as H

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        torch.cuda.set_device(0)
    dev = torch.cuda.current_device()
    if not torch.cuda.is_available():
        raise SystemExit("bench.py needs a CUDA device")

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    n, ts = a.n, a.time_steps
    kappa, u0, h, dt = H.inputs_config(CFG, SEED, n, n, n)
    stream = torch.cuda.Stream()
    fp64_peak = H.fp64_rate()

    # ---- device-resident value
    s = H.Solver(kappa, u0, h, dt, stream=stream.cuda_stream)
    for _ in range(a.warmup):
        s.step(ts)
    s.sync()
    _, l0 = s.stats()
    barrier()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(dev) as clk:
        ev0.record(stream)
        for _ in range(a.steps):
            s.step(ts)
        ev1.record(stream)
        ev1.synchronize()
    barrier()
    _, l1 = s.stats()
    ms = ev0.elapsed_time(ev1)
    l2n, csum = s.norm()
    s.close()

    # ---- FP32-compensated form on the same workload (precision pattern)
    s32 = H.Solver(kappa, u0, h, dt, precision=H.HEAT_FP32C, stream=stream.cuda_stream)
    s32.step(max(1, ts // 10))
    s32.sync()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    s32.step(ts)
    e1.record(stream)
    e1.synchronize()
    ms32 = e0.elapsed_time(e1)
    s32.close()
    fp32c_value = updates(n, ts) / (ms32 * 1e-3) / 1e9
    t_max = max_over_ranks(ms, dist, "cuda")
    upd = updates(n, ts) * a.steps
    value = replica_value(upd, world, t_max * 1e-3)
    launch_ms = ms / (a.steps * ts)
    achieved_gbs = updates(n, 1) * BYTES_PER_UPDATE / (launch_ms * 1e-3) / 1e9

    # ---- end to end through the ABI from pinned host memory
    pk = torch.empty(kappa.shape, dtype=torch.float64, pin_memory=True)
    pu = torch.empty(u0.shape, dtype=torch.float64, pin_memory=True)
    pout = torch.empty(u0.shape, dtype=torch.float64, pin_memory=True)
    pk.numpy()[...] = kappa
    pu.numpy()[...] = u0
    del kappa, u0
    e2e_steps = max(1, min(a.steps, 3))
    with ClockSampler(dev) as e2e_clk:
        for i in range(e2e_steps + 1):   # first one is warm-up
            barrier()
            t0 = time.perf_counter()
            with H.Solver(pk.numpy(), pu.numpy(), h, dt, stream=stream.cuda_stream) as e:
                e.step(ts)
                e.field(pout.numpy())
            t1 = time.perf_counter()
            if i == 0:
                e2e_t = 0.0
            else:
                e2e_t += t1 - t0
    e2e_s = max_over_ranks(e2e_t / e2e_steps, dist, "cuda")
    e2e_value = replica_value(updates(n, ts), world, e2e_s)

    if rank == 0:
        peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
        hbm_peak = peaks.get("hbm_gbs", 6800.0)
        traffic = profile_traffic()
        out = {
            "metric": METRIC, "value": round(value, 3), "unit": UNIT, "n_gpus": world,
            "steps": a.steps, "warmup": a.warmup, "ms_per_step": round(t_max / a.steps, 3),
            "higher_is_better": True, "scaling": "weak",
            "vs_baseline": round(value / world / H100_1CUDA_N512, 3),
            "vs_baseline_ref": "reference 1-cuda on H100 at N=512: 38.97 GLUP/s (CUDA/summary.csv:2)",
            "dtype": "f64", "data": "synthetic (seeded config-1 fields)",
            "config": {**workload(n, ts), "kernel": "default FP64 form (weighted 7-point sum)",
                       "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "hbm", "achieved": round(achieved_gbs, 1), "peak": hbm_peak, "unit": "GB/s",
                         "frac": round(achieved_gbs / hbm_peak, 4),
                         "peak_source": "measured" if peaks else "fallback",
                         "traffic": traffic, "bytes_per_update": BYTES_PER_UPDATE,
                         "kernel_ms_per_launch": round(launch_ms, 4),
                         "fp64_pipe": {"peak_gops": round(fp64_peak, 1),
                                       "note": "measured FP64 FMA rate of this GPU (heat_diag_fp64_rate)"}},
            "e2e": {"value": round(e2e_value, 3), "unit": UNIT,
                    "h2d_bytes_per_step": int(pk.numel() * 8 + pu.numel() * 8),
                    "d2h_bytes_per_step": int(pout.numel() * 8),
                    "ms_per_step": round(e2e_s * 1e3, 3), "clocks": e2e_clk.summary()},
            "fp32c": {"value": round(fp32c_value, 3), "unit": UNIT,
                      "vs_fp64": round(fp32c_value / (value / world), 3),
                      "bytes_per_update": FP32C_BYTES_PER_UPDATE_TB2,
                      "hbm_frac": round(fp32c_value * FP32C_BYTES_PER_UPDATE_TB2 / hbm_peak, 4),
                      "hbm_frac_single_step_bytes": round(fp32c_value * FP32C_BYTES_PER_UPDATE / hbm_peak, 4),
                      "note": "FP32 u + BF16 Kahan carry, FP32 face weights, two steps per launch "
                              "(TMA-staged temporal blocking); same workload, "
                              f"{ts} steps, CUDA events; errors: profiles/fp32c_precision.md"},
            "gpu_launches": int(l1 - l0),
            "clocks": clk.summary(),
            "result": {"l2": l2n, "checksum": csum},
        }
        if not a.skip_cpu:
            try:
                out["cpu_baseline"] = cpu_baseline(n, cpu_threads())
            except Exception as ex:  # report, do not hide
                out["cpu_baseline"] = {"error": str(ex)}
        print(json.dumps(out), flush=True)
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


def main():
    a = parse()
    if a.impl == "reference":
        return reference_arm(a)
    return our_arm(a)


if __name__ == "__main__":
    sys.exit(main())
