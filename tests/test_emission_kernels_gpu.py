"""The two kernels of the image's attenuated emission give the same bits.

``citrus_attenuated_emission`` runs the (point, direction) kernel (one thread per point and direction with all of its
groups) for G <= 16; ``CITRUS_EMISSION_KERNEL=groups`` selects the group-lane kernel (one thread per point and group).
Both form every group value, the signal sums and the per-block height sums in the same order, so their outputs are
equal bit for bit, on seeded inputs that cover per-group optical depths and traced path lengths, one and two points
per cell axis, signal-weighted and per-group outputs, G a multiple of four (float4 rows) or not, and a last block of
directions that is not full.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from citrus_gb300 import _lib
from citrus_gb300.cross_sections import BONE, WATER, spectral_library
from citrus_gb300.geometry import ConeGeometry, Grid
from citrus_gb300.ray_tracing import HostArgs
from citrus_gb300.uncollided import _FCArgs
from citrus_gb300.workloads import bremsstrahlung_spectrum

pytestmark = pytest.mark.gpu


def _emission(cuda_device, groups, q, traced, signal, K, seed=0):
    rng = np.random.default_rng(seed)
    dev = lambda x: torch.as_tensor(np.asarray(x), dtype=torch.float32, device=cuda_device)  # noqa: E731
    library = spectral_library(np.linspace(120.0, 30.0, groups + 1), bremsstrahlung_spectrum(seed=0), [WATER, BONE],
                               1, num_eta=101, fine_per_group=2)
    cells = (5, 7, 6)
    grid = Grid(tuple(c * q for c in cells), 1.6 / q)
    V, NC, G = grid.num_voxels, int(np.prod(cells)), groups
    rho = rng.random((2, *grid.shape)) * [[[[1.0]]], [[[0.0]]]]
    rho[1, 2:5, 3:9, 1:4] = 1.85                                    # bone in a few points, zero elsewhere
    phi = rng.random((G, *grid.shape)) * 1e-3 + 1e-4
    geo = ConeGeometry(100.0, 150.0, 32, 48, 0.4, 0.4, use_curved_detector=True)
    fc = _FCArgs(library, dev(rho), dev(phi), grid, geo, 0.7)
    u = rng.standard_normal((K, 3))
    omegas = dev(u / np.linalg.norm(u, axis=1, keepdims=True))
    if traced:
        tau = dev(rng.random((K, NC, 2)) * 6.0)
        tau_mu = dev(library.mu_t)                                  # [2, G]
    else:
        tau = dev(rng.random((K, NC, G)) * 3.0)
        tau_mu = None
    mu = dev(rng.random((G, NC)) * 0.3)
    multiple = dev(rng.random((K, NC, G)) * 1e-3)
    heights = dev(rng.standard_normal(V) * 5.0)
    weight = dev(rng.random((K, G))) if signal else None
    host = HostArgs()
    deltas = host.doubles(grid.deltas)
    nblocks = -(-V // 32)
    out = torch.empty(K, V, 1 if signal else G, device=cuda_device)
    partial = torch.empty(K * nblocks * 2, device=cuda_device)
    sums = torch.empty(K, 2, device=cuda_device)
    _lib.call("citrus_attenuated_emission", *fc.common(), q, deltas, fc.focal, fc.table.data_ptr(), fc.num_eta,
              fc.eta_lo, fc.eta_hi, omegas.data_ptr(), K, tau.data_ptr(),
              None if tau_mu is None else tau_mu.data_ptr(), 2 if traced else 0, mu.data_ptr(), multiple.data_ptr(),
              heights.data_ptr(), None if weight is None else weight.data_ptr(), out.data_ptr(), partial.data_ptr(),
              partial.numel(), sums.data_ptr(), fc.stream)
    torch.cuda.synchronize()
    return out, partial, sums


@pytest.mark.parametrize("groups, q, traced, signal, K", [
    (8, 1, True, True, 64),     # the batched-views form: float4 rows, traced densities, signal sums
    (8, 2, False, False, 40),   # per-group depths, offsets inside the cells, per-group output, a partial block
    (16, 1, True, False, 70),
    (12, 1, False, True, 64),   # G a multiple of four below its padded 16
    (3, 2, True, True, 33),     # scalar rows
    (1, 1, False, False, 20),
])
def test_direction_warp_emission_equals_group_lane_emission(cuda_device, monkeypatch, groups, q, traced, signal, K):
    monkeypatch.delenv("CITRUS_EMISSION_KERNEL", raising=False)
    new = _emission(cuda_device, groups, q, traced, signal, K)
    monkeypatch.setenv("CITRUS_EMISSION_KERNEL", "groups")
    old = _emission(cuda_device, groups, q, traced, signal, K)
    for a, b in zip(new, old):
        assert torch.equal(a, b)
    assert float(new[0].abs().max()) > 0 and float(new[2][:, 0].abs().min()) > 0
