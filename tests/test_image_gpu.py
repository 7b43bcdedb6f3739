"""Parity of the collapsed-cone image and the primary on sm_103a with the reference fixtures."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import rel_err
from citrus_gb300 import _lib
from citrus_gb300.ray_tracing import GB300Projectors
from citrus_gb300.responses import SourceModel, no_grid
from citrus_gb300.scatter_image import (combined_scatter_image, make_direction_context, panel_direction_set,
                                        primary_image)
from citrus_gb300.uncollided import uncollided_fluence
from test_oracle_golden import _image_setup

pytestmark = pytest.mark.gpu
IMAGE_REL = 1e-4  # scatter image, float32 vs the reference's float64


@pytest.mark.parametrize("name", ["flat", "curved"])
def test_combined_image_and_primary_match_reference(cuda_device, name):
    g, library, grid_q, det, geos = _image_setup()
    geo, angle = geos[name], 0.8
    grid_c = grid_q.coarsen(2)
    dev = lambda x: torch.as_tensor(x, dtype=torch.float32, device=cuda_device)  # noqa: E731
    rho = dev(g["rho"])
    rho_c = rho.reshape(2, 3, 2, 3, 2, 2, 2).mean(dim=(2, 4, 6))
    mu_c = torch.einsum("mg,mijk->gijk", library.tensor("mu_t", cuda_device), rho_c).contiguous()
    proj = GB300Projectors()
    phi = uncollided_fluence(library, rho, grid_q, geo, angle, SourceModel(), proj)
    assert rel_err(phi, g[f"{name}_phi"]) < 2e-6
    cone = panel_direction_set(geo, angle, (3, 6), max_polar_angle=grid_c)
    ctx = make_direction_context(cone, geo, angle, det, no_grid(), library, cuda_device, chunk=5)
    T = dev(g["T"])
    full = combined_scatter_image(library, rho, phi, grid_q, 2, T, 2, geo, angle, mu_c, proj, ctx, grid_c)
    assert rel_err(full["fluence"], g[f"{name}_fluence"]) < IMAGE_REL
    assert rel_err(full["planar_fluence"], g[f"{name}_planar"]) < IMAGE_REL
    assert rel_err(full["signal_per_group"], g[f"{name}_signal_pg"]) < IMAGE_REL
    assert rel_err(full["signal"], g[f"{name}_signal"]) < IMAGE_REL
    sig = combined_scatter_image(library, rho, phi, grid_q, 2, T, 2, geo, angle, mu_c, proj, ctx, grid_c,
                                 signal_only=True)["signal"]
    assert rel_err(sig, g[f"{name}_signal_only"]) < IMAGE_REL
    prim = primary_image(library, rho, grid_q, geo, angle, SourceModel(), proj, det, no_grid())
    assert rel_err(prim["signal"], g[f"{name}_primary_signal"]) < 2e-6
    assert rel_err(prim["fluence"], g[f"{name}_primary_fluence"]) < 2e-6


def test_box_blur_matches_dense_box_matrix(cuda_device):
    """The windowed blur equals the reference's dense overlap-matrix product (scatter_image.box_matrix)."""
    from oracle.image import box_matrix
    rng = np.random.default_rng(1)
    k, lines, N = 4, 6, 37
    x = rng.standard_normal((k, lines, N))
    widths = np.array([0.3, 1.0, 4.7, 60.0])
    xin = torch.as_tensor(x, dtype=torch.float32, device=cuda_device)
    out = torch.empty_like(xin)
    w = torch.as_tensor(widths, dtype=torch.float32, device=cuda_device)
    _lib.call("citrus_box_blur", xin.data_ptr(), out.data_ptr(), k, lines, N, lines * N, N, 1, lines * N, N, 1,
              w.data_ptr(), None, None, 0, 1.0, 0.0, _lib.stream_handle(cuda_device))
    assert rel_err(out, np.einsum("kcj,klj->klc", box_matrix(N, widths), x)) < 1e-6
    dense = torch.empty(k, N, N, device=cuda_device)
    _lib.call("citrus_box_matrix", w.data_ptr(), k, N, dense.data_ptr(), _lib.stream_handle(cuda_device))
    assert rel_err(dense, box_matrix(N, widths)) < 1e-6


@pytest.mark.parametrize("signal", [False, True])
def test_emission_with_fused_source_moments_matches_product_form(cuda_device, signal):
    """citrus_attenuated_emission_moments (Y T formed per point) against citrus_attenuated_emission fed the product
    Y T from the small-K GEMM (the reference's interface): same emission, same height sums."""
    from citrus_gb300 import kernels
    from citrus_gb300.ray_tracing import HostArgs
    from citrus_gb300.uncollided import _FCArgs
    g, library, grid_q, det, geos = _image_setup()
    geo, angle = geos["curved"], 0.8
    grid_c = grid_q.coarsen(2)
    dev = lambda x: torch.as_tensor(x, dtype=torch.float32, device=cuda_device)  # noqa: E731
    rho = dev(g["rho"])
    rho_c = rho.reshape(2, 3, 2, 3, 2, 2, 2).mean(dim=(2, 4, 6))
    mu_c = torch.einsum("mg,mijk->gijk", library.tensor("mu_t", cuda_device), rho_c).contiguous()
    proj = GB300Projectors()
    phi = uncollided_fluence(library, rho, grid_q, geo, angle, SourceModel(), proj)
    cone = panel_direction_set(geo, angle, (3, 6), max_polar_angle=grid_c)
    ctx = make_direction_context(cone, geo, angle, det, no_grid(), library, cuda_device, chunk=64)
    G, NC, V, L = library.num_groups, grid_c.num_voxels, grid_q.num_voxels, 2
    N_sh = (L + 1) ** 2
    T = dev(g["T"]).permute(1, 2, 3, 4, 0).reshape(N_sh, NC * G).contiguous()
    Y = ctx.harmonics(L).contiguous()
    K = Y.shape[0]
    dirs = ctx.omega
    tau = proj.downstream_cumulative(mu_c, grid_c, geo, angle, dirs, voxel_major=True)
    assert torch.equal(tau.permute(0, 2, 1).reshape(K, G, *grid_c.shape),
                       proj.downstream_cumulative(mu_c, grid_c, geo, angle, dirs))
    multiple = torch.empty(K, NC * G, device=cuda_device)
    kernels.small_k_gemm(Y, T, multiple)
    heights, _ = ctx.footprint(grid_q)
    fc = _FCArgs(library, rho, phi, grid_q, geo, angle)
    host = HostArgs()
    deltas = host.doubles(grid_q.deltas)
    mu = mu_c.reshape(G, NC).contiguous()
    weight = dev(np.random.default_rng(2).random((K, G))) if signal else None
    stream = _lib.stream_handle(cuda_device)
    results = []
    for fused in (False, True):
        out = torch.empty(K, V, 1 if signal else G, device=cuda_device)
        partial = torch.empty(K * (-(-V // 32)) * 2, device=cuda_device)
        sums = torch.empty(K, 2, device=cuda_device)
        head = (*fc.common(), 2, deltas, fc.focal, fc.table.data_ptr(), fc.num_eta, fc.eta_lo, fc.eta_hi,
                dirs.data_ptr(), K, tau.data_ptr(), None, 0, mu.data_ptr())
        tail = (heights.data_ptr(), None if weight is None else weight.data_ptr(), out.data_ptr(), partial.data_ptr(),
                partial.numel(), sums.data_ptr(), stream)
        if fused:
            _lib.call("citrus_attenuated_emission_moments", *head, Y.data_ptr(), T.data_ptr(), N_sh, *tail)
        else:
            _lib.call("citrus_attenuated_emission", *head, multiple.data_ptr(), *tail)
        results.append((out, sums))
    assert rel_err(results[1][0], results[0][0]) < 1e-6
    assert rel_err(results[1][1], results[0][1]) < 1e-6
    assert float(results[0][0].abs().max()) > 0


@pytest.mark.parametrize("response", ["ideal_counting", "energy_weighted"])
def test_curved_separable_detector_signal_matches_oracle(cuda_device, response):
    """A curved panel with a detector response that separates in energy and incidence takes the group-summed
    emission with per-channel weights in the direction sum; its signal equals the oracle's and the full path's."""
    from oracle import image as oimage, physics
    from citrus_gb300 import responses
    g, library, grid_q, _, geos = _image_setup()
    det = getattr(responses, f"{response}_response")()
    geo, angle = geos["curved"], 0.8
    grid_c = grid_q.coarsen(2)
    dev = lambda x: torch.as_tensor(x, dtype=torch.float32, device=cuda_device)  # noqa: E731
    rho_np = g["rho"]
    rho_c = rho_np.reshape(2, 3, 2, 3, 2, 2, 2).mean(axis=(2, 4, 6))
    mu_c = np.einsum("mg,mijk->gijk", library.mu_t, rho_c)
    phi_np = physics.uncollided_fluence(library, rho_np, grid_q, geo, angle)
    cone = panel_direction_set(geo, angle, (3, 6), max_polar_angle=grid_c)
    ref = oimage.combined_image(library, rho_np, phi_np, grid_q, 2, g["T"], 2, geo, angle, cone.omega, cone.weight,
                                cone.cell_width, mu_c, det)
    ctx = make_direction_context(cone, geo, angle, det, no_grid(), library, cuda_device, chunk=5)
    assert ctx.signal_column_weight is not None and ctx.signal_group_weight is not None
    proj = GB300Projectors()
    args = (library, dev(rho_np), dev(phi_np), grid_q, 2, dev(g["T"]), 2, geo, angle, dev(mu_c), proj, ctx, grid_c)
    sig = combined_scatter_image(*args, signal_only=True)["signal"]
    full = combined_scatter_image(*args)["signal"]
    assert rel_err(sig, ref["signal"]) < IMAGE_REL
    assert rel_err(sig, full) < 1e-5


@pytest.mark.parametrize("signal_only", [False, True])
def test_density_traced_optical_depth_matches_attenuation_traced(cuda_device, signal_only):
    """Downstream optical depths traced through the cell densities and combined per group in the emission give the
    image of the G attenuation channels traced directly."""
    g, library, grid_q, det, geos = _image_setup()
    geo, angle = geos["flat"], 0.8
    grid_c = grid_q.coarsen(2)
    dev = lambda x: torch.as_tensor(x, dtype=torch.float32, device=cuda_device)  # noqa: E731
    rho = dev(g["rho"])
    rho_c = rho.reshape(2, 3, 2, 3, 2, 2, 2).mean(dim=(2, 4, 6)).contiguous()
    table = library.tensor("mu_t", cuda_device)
    mu_c = torch.einsum("mg,mijk->gijk", table, rho_c).contiguous()
    proj = GB300Projectors()
    phi = uncollided_fluence(library, rho, grid_q, geo, angle, SourceModel(), proj)
    cone = panel_direction_set(geo, angle, (3, 6), max_polar_angle=grid_c)
    ctx = make_direction_context(cone, geo, angle, det, no_grid(), library, cuda_device, chunk=5)
    args = (library, rho, phi, grid_q, 2, dev(g["T"]), 2, geo, angle, mu_c, proj, ctx, grid_c)
    direct = combined_scatter_image(*args, signal_only=signal_only)
    traced = combined_scatter_image(*args, signal_only=signal_only, rho_coarse=rho_c, attenuation=table)
    for key in direct:
        assert rel_err(traced[key], direct[key]) < 1e-5, key
    assert rel_err(traced["signal"], g["flat_signal_only" if signal_only else "flat_signal"]) < IMAGE_REL
