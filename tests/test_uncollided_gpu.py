"""Parity of the uncollided-fluence and first-collision kernels with the reference fixtures and the oracle."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import golden, rel_err
from citrus_gb300.ray_tracing import GB300Projectors
from citrus_gb300.responses import SourceModel
from citrus_gb300.uncollided import (first_collision_moments_at_directions, first_collision_sampling_correction,
                                     first_collision_source_at_directions, group_transmission, uncollided_fluence)
from oracle import physics
from test_oracle_golden import _uncollided_setup

pytestmark = pytest.mark.gpu
F32_REL = 1e-5


@pytest.mark.parametrize("name", ["flat", "curved"])
def test_uncollided_and_first_collision_match_reference(cuda_device, name):
    g = golden("uncollided_small")
    library, grid, geos = _uncollided_setup()
    geo, angle = geos[name], 0.3
    dev = lambda x: torch.as_tensor(x, dtype=torch.float32, device=cuda_device)  # noqa: E731
    rho = dev(g["rho"])
    phi = uncollided_fluence(library, rho, grid, geo, angle, SourceModel(), GB300Projectors())
    assert rel_err(phi, g[f"{name}_phi"]) < 2e-6
    om, w = dev(g["omega"]), dev(g["weight"])
    src = first_collision_source_at_directions(library, rho, phi, grid, geo, angle, om[::4])
    assert rel_err(src, g[f"{name}_source"]) < F32_REL
    corr = first_collision_sampling_correction(library, rho, phi, grid, geo, angle, om, w)
    assert rel_err(corr.scale, g[f"{name}_scale"]) < F32_REL
    assert rel_err(corr.beta, g[f"{name}_beta"]) < 1e-4
    mom = first_collision_moments_at_directions(library, rho, phi, grid, geo, angle, om[::4], corr, 2,
                                                cell_major=False)
    assert rel_err(mom, g[f"{name}_moments"]) < F32_REL


def test_group_transmission_matches_oracle(cuda_device):
    library, _, _ = _uncollided_setup()
    rng = np.random.default_rng(2)
    path = rng.random((2, 7, 9)) * 20.0
    got = group_transmission(library, torch.as_tensor(path, dtype=torch.float32, device=cuda_device))
    assert rel_err(got, physics.group_transmission(library, path)) < 2e-6
    # a subset of materials, as the uncollided fluence traces only the present ones
    got = group_transmission(library, torch.as_tensor(path[1:], dtype=torch.float32, device=cuda_device), [1])
    assert rel_err(got, physics.group_transmission(library, path[1:], [1])) < 2e-6


def test_config_library_first_collision_on_refined_grid(cuda_device):
    """The eight-group Klein-Nishina library of the batched-views workload on a q = 3 quadrature grid."""
    from citrus_gb300.geometry import ConeGeometry, Grid
    from citrus_gb300.quadrature import product_quadrature
    from citrus_gb300.workloads import batched_views
    w = batched_views()
    library = w.library
    grid = Grid((6, 9, 6), 0.5)
    geo = ConeGeometry(100.0, 150.0, 192, 256, 0.16, 0.16, use_curved_detector=True)
    rng = np.random.default_rng(9)
    rho = rng.random((2, *grid.shape)) * np.array([1.0, 1.85])[:, None, None, None]
    phi = physics.uncollided_fluence(library, rho, grid, geo, 1.1)
    q = product_quadrature(6, 20)
    dev = lambda x: torch.as_tensor(x, dtype=torch.float32, device=cuda_device)  # noqa: E731
    scale, beta, _, _ = physics.correction(library, rho, phi, grid, geo, 1.1, q.omega, q.weight)
    corr = first_collision_sampling_correction(library, dev(rho), dev(phi), grid, geo, 1.1, dev(q.omega),
                                               dev(q.weight))
    assert rel_err(corr.scale, scale) < 1e-5
    assert np.abs(corr.beta.cpu().numpy() - beta).max() < 1e-4
    ref = physics.first_collision_moments(library, rho, phi, grid, geo, 1.1, q.omega[:16], scale, beta, 3)
    got = first_collision_moments_at_directions(library, dev(rho), dev(phi), grid, geo, 1.1, dev(q.omega[:16]), corr,
                                                3, cell_major=False)
    assert rel_err(got, ref) < 2e-5
    # the kept source values read back at scattered rows give the same moments
    kept = first_collision_sampling_correction(library, dev(rho), dev(phi), grid, geo, 1.1, dev(q.omega),
                                               dev(q.weight), keep_cache=True)
    assert torch.equal(kept.scale, corr.scale) and torch.equal(kept.beta, corr.beta)
    rows = torch.tensor([5, 0, 77, 119, 31, 64], device=cuda_device)
    cached = first_collision_moments_at_directions(library, dev(rho), dev(phi), grid, geo, 1.1,
                                                   dev(q.omega)[rows], kept, 3, cell_major=False,
                                                   direction_index=rows)
    direct = first_collision_moments_at_directions(library, dev(rho), dev(phi), grid, geo, 1.1, dev(q.omega)[rows],
                                                   kept, 3, cell_major=False)
    assert rel_err(cached, direct) < 1e-6
    ref_rows = physics.first_collision_moments(library, rho, phi, grid, geo, 1.1, q.omega[rows.cpu().numpy()], scale,
                                               beta, 3)
    assert rel_err(cached, ref_rows) < 2e-5


@pytest.mark.parametrize("groups", [8, 3, 12])
def test_direction_warp_correction_equals_group_lane_correction(cuda_device, monkeypatch, groups):
    """The (point, direction) form of the sampling correction against the group-lane form
    (CITRUS_FC_KERNEL=groups): the kept source values bit for bit (same terms in the same order), the quadrature sums
    and the factors to rounding (the sums over the directions run in another order)."""
    from citrus_gb300.cross_sections import BONE, WATER, spectral_library
    from citrus_gb300.geometry import ConeGeometry, Grid
    from citrus_gb300.quadrature import product_quadrature
    from citrus_gb300.workloads import bremsstrahlung_spectrum
    library = spectral_library(np.linspace(120.0, 30.0, groups + 1), bremsstrahlung_spectrum(seed=0), [WATER, BONE],
                               1, num_eta=201, fine_per_group=2)
    grid = Grid((9, 7, 11), 0.6)
    geo = ConeGeometry(100.0, 150.0, 64, 64, 0.4, 0.4)
    rng = np.random.default_rng(groups)
    rho = rng.random((2, *grid.shape)) * np.array([1.0, 0.0])[:, None, None, None]
    rho[1, 2:5, 1:4, 3:8] = 1.85
    q = product_quadrature(6, 20)
    dev = lambda x: torch.as_tensor(x, dtype=torch.float32, device=cuda_device)  # noqa: E731
    phi = dev(rng.random((groups, *grid.shape)) * 1e-3 + 1e-4)
    out = []
    for form in ("warps", "groups"):
        if form == "groups":
            monkeypatch.setenv("CITRUS_FC_KERNEL", "groups")
        else:
            monkeypatch.delenv("CITRUS_FC_KERNEL", raising=False)
        out.append(first_collision_sampling_correction(library, dev(rho), phi, grid, geo, 0.9, dev(q.omega),
                                                       dev(q.weight), keep_sums=True, keep_cache=True))
    a, b = out
    assert torch.equal(a.cache, b.cache)
    assert rel_err(a.sums, b.sums) < 1e-6
    assert rel_err(a.scale, b.scale) < 1e-5
    assert float((a.beta - b.beta).abs().max()) < 1e-5
