"""Error and speed of the FP32-compensated form against the FP64 form.

    python openmp-offloading-intranode-artifact_gb300/precision_report.py \
        [--cfg 2] [--n 1024] [--checkpoints 100,1000,10000] [--seed 2]

Runs the default FP64 form and the FP32C form side by side on the same seeded
inputs (configuration 2 by default: 1024^3, log-normal kappa smoothed by three
3^3 box passes, u0 ~ U[0,1)), and at each checkpoint prints one JSON line with
max |u32 - u64|, ||u32 - u64|| / ||u64|| (computed on the device) and each
form's GLUP/s over the steps since the previous checkpoint.  The FP64 form is
the reference side: a CPU FP64 oracle run at 1024^3 x 10,000 steps would take
hours; the FP64 form itself matches the oracle to <= 1e-12 (tests).
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

sys.path.insert(0, str(Path(__file__).resolve().parent))
import heat_ctypes as H  # noqa: E402


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--cfg", type=int, default=2)
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--checkpoints", default="100,1000,10000")
    ap.add_argument("--seed", type=int, default=2)
    a = ap.parse_args()
    cps = sorted(int(x) for x in a.checkpoints.split(","))
    t0 = time.perf_counter()
    kappa, u0, h, dt = H.inputs_config(a.cfg, a.seed, a.n, a.n, a.n)
    gen_s = time.perf_counter() - t0
    f64 = H.Solver(kappa, u0, h, dt)
    f32 = H.Solver(kappa, u0, h, dt, precision=H.HEAT_FP32C)
    del kappa, u0
    upd = float((a.n - 2) ** 3)
    done = 0
    print(json.dumps({"cfg": a.cfg, "n": a.n, "seed": a.seed, "dt": dt, "h": h,
                      "input_generation_s": round(gen_s, 2)}), flush=True)
    for cp in cps:
        k = cp - done
        t = time.perf_counter()
        f64.step(k)
        f64.sync()
        t64 = time.perf_counter() - t
        t = time.perf_counter()
        f32.step(k)
        f32.sync()
        t32 = time.perf_counter() - t
        done = cp
        mx, rl = H.field_diff(f32, f64)
        l2, cs = f64.norm()
        print(json.dumps({"steps": cp, "max_abs": mx, "rel_l2": rl, "l2_fp64": l2,
                          "glups_fp64": round(upd * k / t64 / 1e9, 2),
                          "glups_fp32c": round(upd * k / t32 / 1e9, 2)}), flush=True)
    f64.close()
    f32.close()


if __name__ == "__main__":
    main()
