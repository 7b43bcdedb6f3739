"""CPU checks of the learned proposal: the float64 autograd oracle of the network against finite differences (so that
the GPU gradients are checked against a pinned oracle), and the random phantoms of the training set."""

from __future__ import annotations

import numpy as np
import torch

from citrus_gb300.geometry import Grid
from citrus_gb300.workloads import INSERT_DENSITIES, ellipsoid_phantom, learned_proposal
from oracle import learned as oracle


def _layer_shapes(c_in, c_out, channels):
    """Weight shapes of the U-Net layers by name (the topology of citrus_gb300.learned.ConvNet3D)."""
    shapes = {}
    for level, c in enumerate(channels):
        prev = c_in if level == 0 else channels[level - 1]
        shapes[f"enc{level}a"] = (c, prev, 3, 3, 3)
        shapes[f"enc{level}b"] = (c, c, 3, 3, 3)
    for level in reversed(range(len(channels) - 1)):
        shapes[f"dec{level}a"] = (channels[level], channels[level] + channels[level + 1], 3, 3, 3)
        shapes[f"dec{level}b"] = (channels[level], channels[level], 3, 3, 3)
    shapes["out"] = (c_out, channels[0], 1, 1, 1)
    return shapes


def test_oracle_gradients_match_finite_differences():
    gen = torch.Generator().manual_seed(0)
    channels = (2, 3, 4)
    shapes = _layer_shapes(2, 2, channels)
    w = {n: torch.randn(*s, generator=gen, dtype=torch.float64) * 0.4 for n, s in shapes.items()}
    b = {n: torch.randn(s[0], generator=gen, dtype=torch.float64) * 0.1 for n, s in shapes.items()}
    x = torch.randn(1, 2, 4, 4, 8, generator=gen, dtype=torch.float64)
    t = torch.randn(1, 2, 4, 4, 8, generator=gen, dtype=torch.float64)
    ref = oracle.loss_and_gradients(w, b, x, t, len(channels))
    rng = np.random.default_rng(0)
    for name in ("enc0a", "enc2b", "dec0a", "dec1b", "out"):
        for _ in range(3):
            idx = tuple(int(rng.integers(0, n)) for n in shapes[name])
            h = 1e-6
            wp = {k: v.clone() for k, v in w.items()}
            wm = {k: v.clone() for k, v in w.items()}
            wp[name][idx] += h
            wm[name][idx] -= h
            lp = oracle.loss_and_gradients(wp, b, x, t, len(channels))["loss"]
            lm = oracle.loss_and_gradients(wm, b, x, t, len(channels))["loss"]
            fd = (lp - lm) / (2 * h)
            assert abs(fd - float(ref[name + ".weight"][idx])) <= 1e-6 + 1e-4 * abs(fd), (name, idx)
        j = int(rng.integers(0, shapes[name][0]))
        bp = {k: v.clone() for k, v in b.items()}
        bm = {k: v.clone() for k, v in b.items()}
        bp[name][j] += 1e-6
        bm[name][j] -= 1e-6
        fd = (oracle.loss_and_gradients(w, bp, x, t, len(channels))["loss"]
              - oracle.loss_and_gradients(w, bm, x, t, len(channels))["loss"]) / 2e-6
        assert abs(fd - float(ref[name + ".bias"][j])) <= 1e-6 + 1e-4 * abs(fd)


def test_random_phantoms():
    grid = Grid((24, 24, 16), 1.6)
    seen = set()
    for seed in range(12):
        rho = ellipsoid_phantom(grid, seed)
        assert rho.shape == (2, 24, 24, 16)
        water, bone = rho
        assert set(np.unique(water)) <= {0.0, 0.0012, 1.0, 1.04}
        assert set(np.unique(bone)) <= {0.0, 1.85}
        assert not np.any((water > 0) & (bone > 0))
        assert np.all((water > 0) | (bone > 0))
        seen |= set(np.unique(water)) | set(np.unique(bone))
        assert np.array_equal(rho, ellipsoid_phantom(grid, seed))          # seeded
    assert {1.0, *INSERT_DENSITIES} <= seen
    w = learned_proposal(1)
    assert w.grid.shape == (96, 96, 64) and abs(w.grid.delta_voxel - 0.4) < 1e-12
    assert w.library.num_groups == 12 and w.num_polar * w.num_azimuthal == 168 and w.num_views == 120
