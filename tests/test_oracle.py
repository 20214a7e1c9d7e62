"""The oracle is pinned before it is trusted (CPU only).

- against the committed golden fixtures made by the unmodified reference serial
  (tests/golden/make_golden.py), bit for bit;
- against the reference serial itself, run here, where its source is present;
- the step-count semantics of while (t < T) { t += dt; }.
"""
from __future__ import annotations

import hashlib
import os
import subprocess
import tempfile
from pathlib import Path

import numpy as np
import pytest

from conftest import bits_equal, golden_cases, golden_npz


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a, dtype="<f8").tobytes()).hexdigest()


@pytest.mark.parametrize("path", golden_npz(), ids=lambda p: p.stem)
def test_oracle_replays_golden_bitwise(oracle, path):
    z = np.load(path)
    n, steps, h, dt, T = z["meta"]
    u, s = oracle.run_T(z["u0"], z["kappa"], h, dt, T, rhs=z["rhs"])
    assert s == int(steps)
    assert bits_equal(u, z["u"])


@pytest.mark.parametrize("case", [c for c in golden_cases() if c["n"] <= 128], ids=lambda c: f"n{c['n']}_s{c['verify_steps']}")
def test_oracle_matches_golden_summary(oracle, case):
    n = case["n"]
    kappa, rhs, u0, h, dt = oracle.inputs_reference(n)
    assert h == case["h"] and dt == case["dt"]
    if (sha(kappa), sha(rhs), sha(u0)) != (case["sha_kappa"], case["sha_rhs"], case["sha_u0"]):
        pytest.skip("this host's libm rounds the reference's sin/cos inputs differently")
    u, s = oracle.run_T(u0, kappa, h, dt, float(case["T"]), rhs=rhs)
    assert s == case["steps"]
    assert sha(u) == case["sha_u"]
    l2, cs = oracle.norm(u)
    assert l2 == pytest.approx(case["l2"], rel=1e-15) and cs == pytest.approx(case["checksum"], rel=1e-15)


def test_golden_inputs_are_the_reference_expressions(oracle):
    """Stored inputs equal the ones the reference's formulas give on this host."""
    for path in golden_npz():
        z = np.load(path)
        n = int(z["meta"][0])
        kappa, rhs, u0, h, dt = oracle.inputs_reference(n)
        if not (bits_equal(kappa, z["kappa"]) and bits_equal(rhs, z["rhs"])):
            pytest.skip("this host's libm rounds sin/cos differently")
        assert bits_equal(u0, z["u0"])
        assert h == z["meta"][2] and dt == z["meta"][3]


@pytest.mark.parametrize("n,steps", [(9, 7), (20, 13), (33, 11)])
def test_oracle_cli_equals_reference_serial(oracle, n, steps):
    """heat_ref N T prints the same step count and writes the same dump as serial."""
    oracle.build()
    if not oracle.REF_SERIAL.exists():
        pytest.skip("the reference serial is built only where the reference source tree is present")
    T = "%.17g" % oracle.verify_T(n, steps)
    with tempfile.TemporaryDirectory() as td:
        env = {**os.environ, "WRITE_TXT": "1", "OMP_NUM_THREADS": "4"}
        a = subprocess.run([str(oracle.REF_SERIAL), str(n), T], cwd=td, env=env, capture_output=True,
                           text=True, check=True)
        b = oracle.cli([n, T], env={"WRITE_TXT": "1", "OMP_NUM_THREADS": "3"}, cwd=td)
        line = lambda s: [x for x in s.splitlines() if "timesteps complete" in x][0]
        assert line(a.stdout) == line(b.stdout)
        assert (Path(td) / "u_serial.txt").read_bytes() == (Path(td) / "u_ref.txt").read_bytes()


@pytest.mark.parametrize("n,steps,fmt,expect", [(512, 500, "%.7g", 501), (64, 100, "%.17g", 100),
                                                 (256, 100, "%.17g", 101)])
def test_step_count_semantics(oracle, n, steps, fmt, expect):
    """The implicit count of while (t < T) (heat3D_variable_coeff.c:161-192):
    STEPS=500 at N=512 with %.7g T gives 501 (OpenMP/summary.csv:2)."""
    h = 1.0 / (n - 1)
    dt = h * h / (12.0 * 0.95)
    assert oracle.count_steps(oracle.verify_T(n, steps, fmt=fmt), dt) == expect


def test_oracle_thread_count_does_not_change_results(oracle):
    kappa, u0, h, dt = oracle.inputs_config(0, 3, 19, 14, 11)
    outs = []
    for t in ("1", "3"):
        r = subprocess.run([str(oracle.CLI_PATH), "--config", "0", "--nx", "19", "--ny", "14", "--nz", "11",
                            "--steps", "9", "--seed", "3", "--l2"], capture_output=True, text=True,
                           env={**os.environ, "OMP_NUM_THREADS": t}, check=True)
        outs.append(r.stdout.split('"l2"')[1])
    assert outs[0] == outs[1]
