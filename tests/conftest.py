"""Shared test setup.

Markers: `gpu` = needs a CUDA device (runs on GB300 only).  Everything else
runs on the CPU.  The product is reached only through libheat's C ABI (the
ctypes binding in the package); the oracle is the CPU restatement under
oracle/ and is used here as the checker.
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "openmp-offloading-intranode-artifact_gb300"
GOLDEN = ROOT / "tests" / "golden"
for p in (str(PKG), str(ROOT / "oracle"), str(ROOT)):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def metrics(ref: np.ndarray, cand: np.ndarray) -> dict:
    """Error metrics as the reference's compare.py (OpenMP/compare.py:47-76):
    max-rel is taken where |ref| > 1e-12."""
    ref = np.asarray(ref, dtype=np.float64).ravel()
    cand = np.asarray(cand, dtype=np.float64).ravel()
    d = cand - ref
    ad, ar = np.abs(d), np.abs(ref)
    mask = ar > 1e-12
    max_rel = float((ad[mask] / ar[mask]).max()) if mask.any() else 0.0
    nrm = float(np.linalg.norm(ref))
    return {"max_abs": float(ad.max()) if ad.size else 0.0, "max_rel": max_rel,
            "rel_l2": float(np.linalg.norm(d) / nrm) if nrm > 0 else float(np.linalg.norm(d)),
            "n_nan": int(np.isnan(cand).sum())}


def bits_equal(a: np.ndarray, b: np.ndarray) -> bool:
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


def golden_cases():
    return json.loads((GOLDEN / "summary.json").read_text())["cases"]


def golden_npz():
    return sorted(GOLDEN.glob("ref_n*_s*.npz"))


@pytest.fixture(scope="session")
def heat():
    """libheat's ctypes binding, built in-tree first (no-op when current)."""
    import heat_build  # the package's build script
    heat_build.build()
    import heat_ctypes
    return heat_ctypes


@pytest.fixture(scope="session")
def oracle():
    import heat_oracle
    heat_oracle.ensure_built()
    return heat_oracle


@pytest.fixture(scope="session")
def cuda_device():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch
