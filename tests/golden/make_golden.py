"""Regenerate the golden fixtures from the UNMODIFIED reference serial solver.

    python tests/golden/make_golden.py

Needs the reference tree (its serial solver is compiled from its own source by
oracle/build_ref.sh into oracle/_ref/serial).  For each case the serial runs
the reference problem exactly as the reference's verify pipeline does
(N, T = STEPS*dt printed %.17g, WRITE_TXT=1; 3D_Heat_Benchmark/NVIDIA-H100/
Source-Results/OpenMP/verify.sh:53-65,145-158) and its u_serial.txt is parsed.

  small cases  -> ref_n<N>_s<STEPS>.npz   inputs (kappa, rhs, u0) + output u
  larger cases -> summary.json            sha256 of inputs and output, L2, sum

The inputs are recomputed with the same expressions the reference uses and
stored, so a fixture can be replayed on a machine whose libm rounds sin/cos
differently.  The script asserts that the oracle restatement reproduces the
serial's output bit-for-bit from those inputs before it writes anything.
"""
from __future__ import annotations

import hashlib
import json
import os
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(ROOT / "oracle"))
import heat_oracle as orc  # noqa: E402

SMALL = [(5, 3), (12, 10), (12, 50), (17, 20), (24, 37)]
LARGE = [(n, s) for n in (51, 64, 128, 256) for s in (1, 50, 100)]


def sha(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


def run_serial(n: int, T: str) -> tuple[np.ndarray, int]:
    with tempfile.TemporaryDirectory() as td:
        r = subprocess.run([str(orc.REF_SERIAL), str(n), T], cwd=td, capture_output=True, text=True,
                           env={**os.environ, "WRITE_TXT": "1", "OMP_NUM_THREADS": "8"}, check=True)
        steps = int(r.stdout.split(" timesteps complete")[0].split()[-1])
        u = np.loadtxt(Path(td) / "u_serial.txt", dtype=np.float64).reshape(n, n, n)
    return u, steps


def main() -> None:
    orc.build()
    if not orc.REF_SERIAL.exists():
        sys.exit("reference serial not built: the reference source tree is required")
    summary = {"generator": "tests/golden/make_golden.py", "cases": []}
    for n, s in SMALL + LARGE:
        T = "%.17g" % (s * ((1.0 / (n - 1)) ** 2 / (12.0 * 0.95)))
        u_ref, steps = run_serial(n, T)
        kappa, rhs, u0, h, dt = orc.inputs_reference(n)
        u_port, steps_port = orc.run_T(u0, kappa, h, dt, float(T), rhs=rhs)
        assert steps_port == steps, (n, s, steps, steps_port)
        assert np.array_equal(u_port.view(np.uint64), u_ref.view(np.uint64)), f"oracle != serial at n={n}"
        l2, cs = orc.norm(u_ref)
        case = {"n": n, "verify_steps": s, "T": T, "steps": steps, "h": h, "dt": dt,
                "sha_kappa": sha(kappa), "sha_rhs": sha(rhs), "sha_u0": sha(u0), "sha_u": sha(u_ref),
                "l2": l2, "checksum": cs}
        if (n, s) in SMALL:
            fn = f"ref_n{n}_s{s}.npz"
            np.savez_compressed(HERE / fn, kappa=kappa, rhs=rhs, u0=u0, u=u_ref,
                                meta=np.array([n, steps, h, dt, float(T)]))
            case["file"] = fn
        summary["cases"].append(case)
        print(f"n={n:4d} verify_steps={s:4d} steps={steps:4d}  l2={l2:.17g}")
    (HERE / "summary.json").write_text(json.dumps(summary, indent=1) + "\n")


if __name__ == "__main__":
    main()
