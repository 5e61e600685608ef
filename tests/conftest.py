"""Shared fixtures.  GPU tests are marked `gpu`; everything else runs on CPU."""
from __future__ import annotations

import glob
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def _cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if _cuda_available():
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


@pytest.fixture(scope="session")
def port():
    from oracle import Port
    return Port()  # builds oracle/_build/libfdb_oracle.so on first use


@pytest.fixture(scope="session")
def reference():
    from oracle import Reference
    if not Reference.available():
        pytest.skip("reference harness not built in this tree (oracle/_ref)")
    return Reference()


def golden_files(pattern: str = "*.npz"):
    return sorted(glob.glob(os.path.join(GOLDEN, pattern)))


def load_golden(name: str) -> dict:
    with np.load(os.path.join(GOLDEN, name if name.endswith(".npz") else name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def rel_maxnorm(a, b) -> float:
    a = np.asarray(a, dtype=np.float64).reshape(-1)
    b = np.asarray(b, dtype=np.float64).reshape(-1)
    den = np.max(np.abs(b))
    if den == 0.0:
        return float(np.max(np.abs(a)))
    return float(np.max(np.abs(a - b)) / den)


@pytest.fixture(scope="session")
def fdb():
    """The product package on the GPU (built in-tree; no fallback)."""
    if not _cuda_available():
        pytest.skip("no CUDA device")
    import fidibench_gb300
    return fidibench_gb300
