"""heatdrv keeps the reference's command-line surface: `heatdrv N T` runs the
reference problem, prints "<s> timesteps complete" and "Time = <sec> seconds"
(the lines the reference's aggregate.sh parses) and writes a %.17g k-j-i dump
when WRITE_TXT allows; with --bitexact the dump equals the oracle's dump of
the same run byte for byte, as the reference's verify.sh compares them."""
from __future__ import annotations

import os
import re
import subprocess

import numpy as np
import pytest

from conftest import PKG, metrics

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def drv(heat, cuda_device):
    return PKG / "heatdrv"


def run(cmd, cwd, env=None):
    e = {**os.environ, **(env or {})}
    return subprocess.run([str(c) for c in cmd], cwd=cwd, env=e, capture_output=True, text=True,
                          check=True).stdout


@pytest.mark.parametrize("n,steps", [(33, 40), (64, 100)])
def test_driver_matches_oracle_dump(drv, oracle, tmp_path, n, steps):
    T = "%.17g" % oracle.verify_T(n, steps)
    out = run([drv, n, T, "--bitexact"], tmp_path, {"WRITE_TXT": "1"})
    ref = run([oracle.CLI_PATH, n, T], tmp_path, {"WRITE_TXT": "1", "OMP_NUM_THREADS": "4"})
    s_out = int(re.search(r"^(\d+) timesteps complete", out, re.M).group(1))
    s_ref = int(re.search(r"^(\d+) timesteps complete", ref, re.M).group(1))
    assert s_out == s_ref
    assert re.search(r"^Time = \d+\.\d+ seconds$", out, re.M)
    assert "Solution written to u_gb300_1gpu.txt" in out
    assert (tmp_path / "u_gb300_1gpu.txt").read_bytes() == (tmp_path / "u_ref.txt").read_bytes()
    # default form: within 1e-12 of the same dump
    out2 = run([drv, n, T], tmp_path, {"WRITE_TXT": "1"})
    assert re.search(r"^L2 norm = ", out2, re.M)
    a = np.loadtxt(tmp_path / "u_gb300_1gpu.txt")
    b = np.loadtxt(tmp_path / "u_ref.txt")
    assert metrics(b, a)["max_rel"] <= 1e-12


def test_driver_write_txt_off_and_config_mode(drv, tmp_path):
    out = run([drv, "--config", "c1", "--n", 48, "--steps", 25], tmp_path, {"WRITE_TXT": "0"})
    assert "25 timesteps complete" in out
    assert not (tmp_path / "u_gb300_1gpu.txt").exists()
    glups = float(re.search(r"^GLUP/s = ([0-9.]+)", out, re.M).group(1))
    assert glups > 0
