"""Timing and verification pipeline with the reference's file formats.

The reference times its binaries with Slurm job scripts and reduces the
results with shell/awk and Python tools:

* ``run.sh`` runs each binary as ``./<binary> N DT`` and writes, per job, a
  directory ``results_<job>_<timestamp>/`` holding ``run.log`` (the job banner,
  a ``>>> <binary>  gpus=G  mask=M  N=N`` line before each run, the binary's
  own output) and ``timings.csv`` (``rep,job_id,variant,family,gpus,cuda_mask,
  N,dt,steps,wall_sec,reported_sec,status``)
  (3D_Heat_Benchmark/NVIDIA-H100/Source-Results/CUDA/run.sh:100-160,
  OpenMP/run.sh:116-120,300-330);
* ``submit.sh`` sets ``DT = STEPS * h^2 / (12 kappa_max)`` printed ``%.7g``
  (OpenMP/submit.sh:107-109);
* ``aggregate.sh`` merges the result directories into ``summary.csv``: one
  row per (variant, gpus, N) with samples, failures, min/median/max seconds,
  spread and steps, from the solver's ``Time = `` line (compute mode) or from
  ``timings.csv`` (wall / reported modes) (CUDA/aggregate.sh:26-160);
* ``model/compute_gamma.py`` turns single-GPU rows of ``summary.csv`` into the
  machine constant gamma = T1 / (steps (N-2)^3) and its plateau over the
  largest grids (model/compute_gamma.py:1-27,120-190);
* ``verify.sh`` compares a binary's ``%.17g`` dump with the serial
  reference's, line by line, on max |diff| against a tolerance
  (OpenMP/verify.sh:160-186).

This module produces and reads the same files for the GB300 build, so the
reference's own aggregate/gamma/plot scripts accept its results unchanged,
and so its results can be reduced on a machine without Slurm.  The binary
it times is the C driver ``heatdrv`` (or a link to it named like a reference
binary, e.g. ``1-omp``).

    python pipeline.py run --n 512 640 --reps 5 --steps 500
    python pipeline.py aggregate [--time-field compute|wall|reported] [-o summary.csv]
    python pipeline.py gamma --summary summary.csv --exe 1-cuda-gb300
    python pipeline.py verify u_serial.txt u_openmp_1gpu.txt --tol 1e-10
"""
from __future__ import annotations

import argparse
import csv
import io
import math
import os
import re
import subprocess
import sys
import time
from datetime import datetime
from pathlib import Path
from typing import Iterable, Optional

HERE = Path(__file__).resolve().parent
DRIVER = HERE / "heatdrv"
DEFAULT_VARIANT = "1-cuda-gb300"
TIMINGS_HEADER = "rep,job_id,variant,family,gpus,cuda_mask,N,dt,steps,wall_sec,reported_sec,status"
SUMMARY_COLUMNS = "variant,gpus,N,samples,failed,min_sec,median_sec,max_sec,rel_spread_pct,steps"
# A variant token in a ">>> " line: the reference's binary names (1-omp,
# 2-cuda-stream, ...), and this build's (1-cuda-gb300).
_VARIANT_TOKEN = re.compile(r"^[0-9]+-(omp|cuda|acc)")


# ---------------------------------------------------------------- run -------
def final_time(n: int, steps: int, kappa_max: float = 0.95) -> str:
    """DT argument for N and STEPS as submit.sh computes and prints it."""
    h = 1.0 / (n - 1)
    dt = h * h / (12.0 * kappa_max)
    return _c_format("%.7g", steps * dt)


def _c_format(fmt: str, x: float) -> str:
    # Python's %-formatting of floats is C's printf for these conversions.
    return fmt % x


def _solver_time(stdout: str) -> Optional[str]:
    """The third field of the first line starting 'Time = ' (run.sh's parse)."""
    for line in stdout.splitlines():
        if line.startswith("Time = "):
            f = line.split()
            return f[2] if len(f) > 2 else None
    return None


def run(ns: Iterable[int], reps: int = 1, steps: int = 500, variant: str = DEFAULT_VARIANT,
        driver: Path = DRIVER, out_dir: Path = Path("."), job_id: Optional[str] = None,
        timeout: float = 1800.0, extra_args: Iterable[str] = (), kappa_max: float = 0.95,
        env: Optional[dict] = None) -> list[Path]:
    """Time `driver N DT` for every N and repetition; one results directory
    per (N, repetition), as one run.sh job each.  Returns the directories."""
    driver = Path(driver).resolve()
    if not driver.exists():
        raise FileNotFoundError(f"driver not found: {driver} (build it with heat_build.py)")
    out_dir = Path(out_dir)
    out_dir.mkdir(parents=True, exist_ok=True)
    made = []
    base_job = job_id or f"local{os.getpid()}"
    serial = 0
    for n in list(ns):
        dt_arg = final_time(n, steps, kappa_max)
        for rep in range(1, reps + 1):
            serial += 1
            job = f"{base_job}{serial:03d}"
            stamp = datetime.now().strftime("%Y%m%d_%H%M%S")
            rdir = out_dir / f"results_{job}_{stamp}"
            k = 1
            while rdir.exists():
                rdir = out_dir / f"results_{job}_{stamp}_{k}"
                k += 1
            rdir.mkdir()
            log = io.StringIO()
            log.write("=" * 60 + "\n")
            log.write(f"Host               : {os.uname().nodename}\n")
            log.write(f"Job ID             : {job}\n")
            log.write(f"Repetition         : {rep}\n")
            log.write(f"Timestamp          : {stamp}\n")
            log.write(f"Results dir        : {rdir.name}\n")
            log.write(f"N                  : {n}\n")
            log.write(f"DT                 : {dt_arg}\n")
            log.write(f"STEPS              : {steps}\n")
            log.write("=" * 60 + "\n\n")
            log.write("Starting benchmarks\n===========================\n")
            log.write(f"N = {n}   dt = {dt_arg}\n===========================\n\n")
            log.write(f">>> {variant}  gpus=1  mask=0  N={n}\n")
            cmd = [str(driver), str(n), dt_arg, *extra_args]
            run_env = dict(os.environ if env is None else env)
            run_env.setdefault("WRITE_TXT", "0")
            t0 = time.time()
            try:
                p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                                   text=True, timeout=timeout, env=run_env, cwd=rdir)
                status = "ok" if p.returncode == 0 else "runtime_error"
                stdout = p.stdout
            except subprocess.TimeoutExpired as e:
                status = "timeout"
                stdout = e.stdout.decode() if isinstance(e.stdout, bytes) else (e.stdout or "")
            wall = f"{(round((time.time() - t0) * 1000.0)) / 1000.0:.4f}"
            reported = _solver_time(stdout) or "N/A"
            log.write(stdout)
            log.write(f"    -> wall={wall}s  reported={reported}s  status={status}\n")
            (rdir / "run.log").write_text(log.getvalue())
            with open(rdir / "timings.csv", "w") as f:
                f.write(TIMINGS_HEADER + "\n")
                f.write(f"{rep},{job},{variant},1gpu,1,0,{n},{dt_arg},{steps},{wall},{reported},{status}\n")
            made.append(rdir)
    return made


# ------------------------------------------------------------ aggregate -----
def _median_sorted(a: list[float]) -> float:
    n = len(a)
    m = (n + 1) // 2
    return a[m - 1] if n % 2 else (a[m - 1] + a[m]) / 2.0


def _awk_num(s: str) -> float:
    """Numeric value of a string as awk takes it (leading numeric prefix)."""
    m = re.match(r"\s*[-+]?(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?", s)
    return float(m.group(0)) if m else 0.0


def _summary_row(key: str, vals: list[float], failed: int, steps: str) -> str:
    a = sorted(vals)
    med = _median_sorted(a)
    lo, hi = a[0], a[-1]
    spread = 100.0 * (hi - lo) / med if med > 0 else 0.0
    return f"{key},{len(a)},{failed},{lo:.4f},{med:.4f},{hi:.4f},{spread:.1f},{steps}"


def _sorted_output(header: str, rows: list[str]) -> str:
    hier = header.startswith("hier,")

    def sort_key(line: str):
        f = line.split(",")
        if hier:
            return (f[0], f[1], _awk_num(f[3]) if len(f) > 3 else 0.0, line)
        return (f[0], _awk_num(f[2]) if len(f) > 2 else 0.0, line)

    return "\n".join([header] + sorted(rows, key=sort_key)) + "\n"


def _result_dirs(root: Path) -> list[Path]:
    return sorted(p for p in Path(root).glob("results_*") if p.is_dir())


def aggregate_compute(root: Path = Path(".")) -> str:
    """summary.csv from the solver's own 'Time = ' lines in results_*/run.log."""
    logs = [d / "run.log" for d in _result_dirs(root) if (d / "run.log").is_file()]
    if not logs:
        raise FileNotFoundError("no results_*/run.log found")
    timed = []   # (variant, gpus, N, seconds-string, steps-string)
    for log in logs:
        variant = gpus = n = steps = ""
        armed = False
        for line in log.read_text(errors="replace").splitlines():
            fields = line.split()
            if line.startswith(">>> "):
                variant = gpus = n = steps = ""
                armed = False
                for tok in fields[1:]:
                    t = tok[2:] if tok.startswith("./") else tok
                    if _VARIANT_TOKEN.match(t):
                        variant = t
                    if tok.startswith("gpus="):
                        gpus = tok.split("=")[1]
                    if tok.startswith("N="):
                        n = tok.split("=")[1]
                armed = bool(variant and gpus and n)
                continue
            if not armed:
                continue
            if line.startswith("Estimated timesteps:"):
                s = fields[2] if len(fields) > 2 else ""
                steps = s[1:] if s.startswith("~") else s
            if re.search(r"timesteps? complete", line):
                steps = fields[0] if fields else ""
            if line.startswith("Time = "):
                timed.append((variant, gpus, n, fields[2] if len(fields) > 2 else "", steps))
                armed = False
    if not timed:
        raise ValueError("no 'Time = ' lines matched")
    vals: dict[str, list[float]] = {}
    st: dict[str, str] = {}
    for variant, gpus, n, sec, steps in timed:
        key = f"{variant},{gpus},{n}"
        vals.setdefault(key, []).append(_awk_num(sec))
        if steps != "":
            st[key] = steps
    rows = [_summary_row(k, v, 0, st.get(k, "")) for k, v in vals.items()]
    return _sorted_output(SUMMARY_COLUMNS, rows)


def aggregate_csv(root: Path = Path("."), time_field: str = "wall") -> str:
    """summary.csv from results_*/timings.csv on wall or reported seconds.
    Columns are found by header name; rows whose unquoted comma mask added
    fields are shifted back; rows that did not finish are counted as failed."""
    csvs = [d / "timings.csv" for d in _result_dirs(root) if (d / "timings.csv").is_file()]
    if not csvs:
        raise FileNotFoundError("no results_*/timings.csv found")
    lines = csvs[0].read_text().splitlines()[:1]
    for f in csvs:
        lines += f.read_text().splitlines()[1:]
    head = [h.strip(" \t") for h in lines[0].split(",")]
    col = {}
    maskcol = 0
    for i, h in enumerate(head, start=1):
        col[h] = i
        if h.endswith("_mask"):
            maskcol = i
    hier = "hier" in col
    has_steps = "steps" in col
    width = len(head)
    seen: list[str] = []
    cnt: dict[str, list[float]] = {}
    bad: dict[str, int] = {}
    why: dict[str, str] = {}
    st: dict[str, str] = {}

    for line in lines[1:]:
        f = line.split(",")
        off = max(len(f) - width, 0)

        def get(name: str) -> str:
            i = col[name]
            if i > maskcol:
                i += off
            return f[i - 1] if 1 <= i <= len(f) else ""

        key = (f[col["hier"] - 1] + "," if hier else "") + \
              f"{f[col['variant'] - 1]},{f[col['gpus'] - 1]},{get('N')}"
        if key not in seen:
            seen.append(key)
        steps = get("steps") if has_steps else ""
        if steps not in ("", "N/A"):
            st[key] = steps
        status = f[-1]
        if status != "ok":
            bad[key] = bad.get(key, 0) + 1
            why[key] = status
            continue
        t = get("wall_sec") if time_field == "wall" else get("reported_sec")
        if t in ("N/A", ""):
            t = get("wall_sec")
        if t in ("N/A", ""):
            bad[key] = bad.get(key, 0) + 1
            why[key] = "unparseable"
            continue
        cnt.setdefault(key, []).append(_awk_num(t))

    header = ("hier," if hier else "") + SUMMARY_COLUMNS
    rows = []
    suspect = False
    for key in seen:
        v = cnt.get(key, [])
        if not v:
            rows.append(f"{key},0,{bad.get(key, 0)},N/A,N/A,N/A,{why.get(key, '')},{st.get(key, '')}")
            continue
        if _median_sorted(sorted(v)) < 0.01:
            suspect = True
        rows.append(_summary_row(key, v, bad.get(key, 0), st.get(key, "")))
    if suspect:
        print("WARNING: medians < 0.01 s -- reported_sec holds DT. Use the compute time field.",
              file=sys.stderr)
    return _sorted_output(header, rows)


def aggregate(root: Path = Path("."), time_field: str = "compute") -> str:
    if time_field == "compute":
        return aggregate_compute(root)
    if time_field not in ("wall", "reported"):
        raise ValueError(f"time field must be compute, wall or reported (got {time_field!r})")
    return aggregate_csv(root, time_field)


# ---------------------------------------------------------------- gamma -----
GAMMA_COLUMNS = ["N", "interior_points", "timesteps", "T1_seconds", "gamma_s_per_point"]


def gamma_rows(summary: Path, exe: str = DEFAULT_VARIANT, time_column: str = "median_sec") -> list[dict]:
    """Per-grid gamma = T1 / (steps (N-2)^3) for the rows of one variant,
    sorted by N; rows with missing or non-positive values are skipped."""
    out = []
    with open(summary, newline="", encoding="utf-8") as fh:
        rd = csv.DictReader(fh)
        need = {"variant", "N", "steps", time_column}
        missing = need.difference(rd.fieldnames or [])
        if missing:
            raise ValueError(f"{summary} lacks column(s): {', '.join(sorted(missing))}")
        for row in rd:
            if (row.get("variant") or "").strip() != exe:
                continue
            try:
                n = int(row["N"])
                steps = int(row["steps"])
                t1 = float(row[time_column])
            except (TypeError, ValueError):
                continue
            if not math.isfinite(t1) or n <= 2 or steps <= 0 or t1 <= 0:
                continue
            interior = (n - 2) ** 3
            out.append({"N": n, "interior_points": interior, "timesteps": steps,
                        "T1_seconds": t1, "gamma_s_per_point": t1 / (steps * interior)})
    out.sort(key=lambda r: r["N"])
    return out


def gamma_plateau(rows: list[dict], tail: int = 3) -> float:
    last = rows[-min(tail, len(rows)):]
    return sum(r["gamma_s_per_point"] for r in last) / len(last)


def write_gamma_csv(rows: list[dict], path: Path) -> None:
    path = Path(path)
    path.parent.mkdir(parents=True, exist_ok=True)
    with open(path, "w", newline="", encoding="utf-8") as fh:
        w = csv.DictWriter(fh, fieldnames=GAMMA_COLUMNS)
        w.writeheader()
        w.writerows(rows)


# --------------------------------------------------------------- verify -----
def compare_dumps(ref: Path, out: Path, tol: float = 1e-10) -> tuple[bool, float, int, str]:
    """verify.sh's check of two dumps: max |diff| of the last field of each
    line, and equal line counts.  Returns (pass, worst, line, message)."""
    a = [ln.split()[-1] if ln.split() else "" for ln in Path(ref).read_text().splitlines()]
    b = [ln.split()[-1] if ln.split() else "" for ln in Path(out).read_text().splitlines()]
    worst, where = 0.0, 0
    for i in range(min(len(a), len(b))):
        d = abs(_awk_num(a[i]) - _awk_num(b[i]))
        if d > worst:
            worst, where = d, i + 1
    if len(a) != len(b):
        return False, worst, where, f"LINE COUNT MISMATCH ({len(a)} vs {len(b)})"
    ok = worst <= tol
    return ok, worst, where, f"max|diff| = {worst:.6e} at line {where} -> {'PASS' if ok else 'FAIL'}"


# ------------------------------------------------------------------ CLI -----
def main(argv: Optional[list[str]] = None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    sub = ap.add_subparsers(dest="cmd", required=True)

    r = sub.add_parser("run", help="time the driver; write results_*/run.log and timings.csv")
    r.add_argument("--n", type=int, nargs="+", default=[512, 640, 768, 896, 1024, 1152, 1280])
    r.add_argument("--reps", type=int, default=5)
    r.add_argument("--steps", type=int, default=500)
    r.add_argument("--kappa-max", type=float, default=0.95)
    r.add_argument("--variant", default=DEFAULT_VARIANT)
    r.add_argument("--driver", default=str(DRIVER))
    r.add_argument("--out", default=".")
    r.add_argument("--job-id", default=None)
    r.add_argument("--timeout", type=float, default=1800.0)
    r.add_argument("driver_args", nargs="*", help="extra driver flags (e.g. --bitexact)")

    g = sub.add_parser("aggregate", help="results_*/ -> summary.csv")
    g.add_argument("dir", nargs="?", default=".")
    g.add_argument("--time-field", default=os.environ.get("TIME_FIELD", "compute"),
                   choices=("compute", "wall", "reported"))
    g.add_argument("-o", "--output", default="summary.csv")

    m = sub.add_parser("gamma", help="summary.csv -> gamma per grid and plateau")
    m.add_argument("--summary", default="summary.csv")
    m.add_argument("--exe", default=DEFAULT_VARIANT)
    m.add_argument("--time-column", default="median_sec", choices=("min_sec", "median_sec", "max_sec"))
    m.add_argument("--tail", type=int, default=3)
    m.add_argument("--output", default=None)

    v = sub.add_parser("verify", help="compare a dump with the serial reference's")
    v.add_argument("ref")
    v.add_argument("out")
    v.add_argument("--tol", type=float, default=1e-10)

    a = ap.parse_args(argv)
    if a.cmd == "run":
        dirs = run(a.n, a.reps, a.steps, a.variant, Path(a.driver), Path(a.out), a.job_id,
                   a.timeout, a.driver_args, a.kappa_max)
        for d in dirs:
            print(d)
        return 0
    if a.cmd == "aggregate":
        text = aggregate(Path(a.dir), a.time_field)
        Path(a.output).write_text(text)
        sys.stdout.write(text)
        return 0
    if a.cmd == "gamma":
        if a.tail <= 0:
            ap.error("--tail must be positive")
        rows = gamma_rows(Path(a.summary), a.exe, a.time_column)
        if not rows:
            print(f"no usable rows for variant {a.exe!r} in {a.summary}", file=sys.stderr)
            return 1
        for row in rows:
            print(f"{row['N']:>6} {row['interior_points']:>18} {row['timesteps']:>7} "
                  f"{row['T1_seconds']:>12.6f} {row['gamma_s_per_point']:>15.4e} "
                  f"{row['gamma_s_per_point'] * 1e12:>15.3f}")
        plateau = gamma_plateau(rows, a.tail)
        print(f"plateau gamma: {plateau:.4e} s/point-update ({plateau * 1e12:.2f} ps/point-update)")
        out = Path(a.output) if a.output else Path(a.summary).parent / "gamma_single_gpu.csv"
        write_gamma_csv(rows, out)
        print(f"wrote {out}")
        return 0
    ok, _, _, msg = compare_dumps(Path(a.ref), Path(a.out), a.tol)
    print(msg)
    return 0 if ok else 1


if __name__ == "__main__":
    sys.exit(main())
