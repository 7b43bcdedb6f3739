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


def elementwise_rel_err(a, b, floor: float = 1e-3) -> float:
    """max over elements of |a - b| / |b|, over the elements with |b| above ``floor`` times max |b|."""
    a = np.asarray(a.detach().cpu().double() if hasattr(a, "detach") else a, dtype=np.float64)
    b = np.asarray(b.detach().cpu().double() if hasattr(b, "detach") else b, dtype=np.float64)
    mask = np.abs(b) > floor * np.abs(b).max()
    return float((np.abs(a - b)[mask] / np.abs(b)[mask]).max())


def block_means(image, n: int = 8) -> np.ndarray:
    """Means of an image over n x n blocks, rows and channels split as numpy.array_split does (the layout of the
    reference's regression cases, its ``tests/test_quadrature_grid.py:54-59``)."""
    image = np.asarray(image.detach().cpu().double() if hasattr(image, "detach") else image, dtype=np.float64)
    r = np.array_split(np.arange(image.shape[0]), n)
    c = np.array_split(np.arange(image.shape[1]), n)
    return np.array([[image[np.ix_(ri, ci)].mean() for ci in c] for ri in r])


def check_regression_case(scatter, primary, iterations, final_change, g, name: str, tolerance: float) -> None:
    """A solve against one regression case of the reference (its ``_check_reference``,
    ``tests/test_quadrature_grid.py:62-71``): 8 x 8 block means and sums of both signals, source-iteration count and
    final change."""
    assert list(np.shape(scatter)) == list(g[f"{name}_image_shape"])
    assert rel_err(block_means(scatter), g[f"{name}_scatter_signal_blocks"]) < tolerance
    assert rel_err(block_means(primary), g[f"{name}_primary_signal_blocks"]) < tolerance
    s = float(np.asarray(scatter.detach().cpu().double() if hasattr(scatter, "detach") else scatter).sum())
    p = float(np.asarray(primary.detach().cpu().double() if hasattr(primary, "detach") else primary).sum())
    assert abs(s / float(g[f"{name}_scatter_signal_sum"]) - 1) < tolerance
    assert abs(p / float(g[f"{name}_primary_signal_sum"]) - 1) < tolerance
    assert int(iterations) == int(g[f"{name}_si_iterations"])
    expected = float(g[f"{name}_si_final_change"])
    assert abs(final_change - expected) <= max(1e-3, tolerance) * abs(expected)


@pytest.fixture(scope="session")
def cuda_device():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("needs CUDA")
    from citrus_gb300.build import build

    build()
    return torch.device("cuda")
