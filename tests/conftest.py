"""Test configuration: the ``gpu`` marker, the repository on sys.path, and shared helpers.

Tests marked ``gpu`` need a CUDA device and the built library; everything else runs on the CPU (the oracle against
the golden fixtures, host logic, the C-ABI exports, multi-process gloo runs).
"""

from __future__ import annotations

import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = Path(__file__).resolve().parent / "golden"
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and libcitrus_gb300.so")


def golden(name: str) -> dict:
    """Arrays of one fixture generated from the reference (``tests/golden/make_golden.py``)."""
    with np.load(GOLDEN / f"{name}.npz") as data:
        return {k: data[k] for k in data.files}


def rel_err(a, b) -> float:
    """max |a - b| / max |b|, in float64."""
    a = np.asarray(a.detach().cpu().double() if hasattr(a, "detach") else a, dtype=np.float64)
    b = np.asarray(b.detach().cpu().double() if hasattr(b, "detach") else b, dtype=np.float64)
    scale = np.abs(b).max()
    return float(np.abs(a - b).max() / (scale if scale > 0 else 1.0))


@pytest.fixture(scope="session")
def cuda_device():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs CUDA")
    from citrus_gb300.build import build

    build()
    return torch.device("cuda")
