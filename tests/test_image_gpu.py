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
