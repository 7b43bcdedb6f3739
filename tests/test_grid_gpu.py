"""The scatter image and the primary behind an anti-scatter grid that varies over the panel, and the uncollided
fluence and primary of a source with an emission profile, an off-focal table and a beam filter, on sm_103a, against
the reference's own values (``tests/golden/grid_and_source.npz``) and the float64 oracle."""

from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest
import torch

from conftest import golden, rel_err
from citrus_gb300 import _lib
from citrus_gb300.geometry import Grid
from citrus_gb300.ray_tracing import GB300Projectors, HostArgs
from citrus_gb300.responses import SourceModel
from citrus_gb300.scatter_image import (combined_scatter_image, make_direction_context, panel_direction_set,
                                        primary_image)
from citrus_gb300.uncollided import source_field, uncollided_fluence
from test_oracle_golden import _image_setup
from test_responses import fixture_grid, fixture_source, image_geometry

pytestmark = pytest.mark.gpu
IMAGE_REL = 1e-4  # float32 against the reference's float64, as the image without a grid
ROUTES = ("flat_rows", "flat_channels", "flat_crossed", "curved_rows", "curved_pixel", "curved_crossed")


def _route(name):
    grid = fixture_grid()
    rows = replace(grid, septa_along="rows")
    return {"flat_rows": (False, grid), "flat_channels": (False, rows),
            "flat_crossed": (False, replace(grid, crossed=rows)), "curved_rows": (True, rows),
            "curved_pixel": (True, grid), "curved_crossed": (True, replace(grid, crossed=rows))}[name]


@pytest.mark.parametrize("name", ROUTES)
def test_image_behind_grid_matches_reference(cuda_device, name):
    g = golden("grid_and_source")
    _, library, grid_q, det, _ = _image_setup()
    curved, response = _route(name)
    geo, angle = image_geometry(curved), 0.8
    grid_c = grid_q.coarsen(2)
    dev = lambda x: torch.as_tensor(x, dtype=torch.float32, device=cuda_device)  # noqa: E731
    rho = dev(g["image_rho"])
    rho_c = rho.reshape(2, 3, 2, 3, 2, 2, 2).mean(dim=(2, 4, 6))
    mu_c = torch.einsum("mg,mijk->gijk", library.tensor("mu_t", cuda_device), rho_c).contiguous()
    proj = GB300Projectors()
    phi = uncollided_fluence(library, rho, grid_q, geo, angle, SourceModel(), proj)
    assert rel_err(phi, g[f"image_{name}_phi"]) < 2e-6
    cone = panel_direction_set(geo, angle, (3, 6), max_polar_angle=grid_c)
    ctx = make_direction_context(cone, geo, angle, det, response, library, cuda_device, chunk=5)
    T = dev(g["image_T"])
    full = combined_scatter_image(library, rho, phi, grid_q, 2, T, 2, geo, angle, mu_c, proj, ctx, grid_c)
    assert rel_err(full["fluence"], g[f"image_{name}_fluence"]) < IMAGE_REL
    assert rel_err(full["signal_per_group"], g[f"image_{name}_signal_pg"]) < IMAGE_REL
    assert rel_err(full["signal"], g[f"image_{name}_signal"]) < IMAGE_REL
    sig = combined_scatter_image(library, rho, phi, grid_q, 2, T, 2, geo, angle, mu_c, proj, ctx, grid_c,
                                 signal_only=True)["signal"]
    assert rel_err(sig, g[f"image_{name}_signal_only"]) < IMAGE_REL
    prim = primary_image(library, rho, grid_q, geo, angle, SourceModel(), proj, det, response)
    assert rel_err(prim["signal"], g[f"image_{name}_primary"]) < 2e-6


@pytest.mark.parametrize("name", ["flat_crossed", "curved_pixel", "curved_crossed"])
def test_image_behind_grid_matches_oracle(cuda_device, name):
    """A larger panel and another view against the oracle, which evaluates the grid angles at every direction and
    pixel directly (no per-row, per-channel or direction-plus-pixel factoring)."""
    from citrus_gb300.geometry import ConeGeometry
    from oracle import image as oimage
    _, library, grid_q, det, _ = _image_setup()
    curved, response = _route(name)
    geo = ConeGeometry(50.0, 80.0, 24, 30, 0.7, 0.8, det_row_offset=-0.6, use_curved_detector=curved)
    angle = 2.1
    grid_c = grid_q.coarsen(2)
    rng = np.random.default_rng(4)
    rho = rng.random((2, *grid_q.shape)) * np.array([1.0, 0.6])[:, None, None, None]
    rho_c = rho.reshape(2, 3, 2, 3, 2, 2, 2).mean(axis=(2, 4, 6))
    mu_c = np.einsum("mg,mijk->gijk", library.mu_t, rho_c)
    T = rng.random((library.num_groups, 9, *grid_c.shape)) * 1e-4
    from oracle import physics
    phi = physics.uncollided_fluence(library, rho, grid_q, geo, angle)
    cone = panel_direction_set(geo, angle, (3, 8), max_polar_angle=grid_c)
    ref = oimage.combined_image(library, rho, phi, grid_q, 2, T, 2, geo, angle, cone.omega, cone.weight,
                                cone.cell_width, mu_c, det, grid=response)
    dev = lambda x: torch.as_tensor(x, dtype=torch.float32, device=cuda_device)  # noqa: E731
    ctx = make_direction_context(cone, geo, angle, det, response, library, cuda_device, chunk=7)
    full = combined_scatter_image(library, dev(rho), dev(phi), grid_q, 2, dev(T), 2, geo, angle, dev(mu_c),
                                  GB300Projectors(), ctx, grid_c)
    assert rel_err(full["signal_per_group"], ref["signal_per_group"]) < IMAGE_REL
    sig = combined_scatter_image(library, dev(rho), dev(phi), grid_q, 2, dev(T), 2, geo, angle, dev(mu_c),
                                 GB300Projectors(), ctx, grid_c, signal_only=True)["signal"]
    assert rel_err(sig, ref["signal"]) < IMAGE_REL


@pytest.mark.parametrize("curved", [False, True])
def test_source_profile_off_focal_and_filter_match_reference(cuda_device, curved):
    g = golden("grid_and_source")
    _, library, _, det, _ = _image_setup()
    pre = "curved" if curved else "flat"
    geo = image_geometry(curved)
    src = fixture_source(g, pre)
    big = Grid((8, 10, 6), 3.0)
    w, path = source_field(src, geo, 0.8, big, cuda_device, divide_by_distance_squared=False)
    assert rel_err(w, g[f"source_{pre}_b"]) < 1e-6
    assert rel_err(path, g[f"source_{pre}_filter_path"]) < 1e-6
    rho = torch.as_tensor(g[f"source_{pre}_rho"], dtype=torch.float32, device=cuda_device)
    phi = uncollided_fluence(library, rho, big, geo, 0.8, src, GB300Projectors())
    assert rel_err(phi, g[f"source_{pre}_phi"]) < 2e-6
    prim = primary_image(library, rho, big, geo, 0.8, src, GB300Projectors(), det, fixture_grid(g))
    assert rel_err(prim["signal"], g[f"source_{pre}_primary"]) < 2e-6
    assert rel_err(prim["fluence"], g[f"source_{pre}_primary_fluence"]) < 2e-6
    prim2 = primary_image(library, rho, big, geo, 0.8, src, GB300Projectors(), det, fixture_grid(g),
                          samples_per_pixel_axis=2)
    assert rel_err(prim2["signal"], g[f"source_{pre}_primary_n2"]) < 2e-6


def test_grid_signal_sum_kernel_against_float64(cuda_device):
    """The kernel's weighted sum against a float64 product of the same factors (two septa sets, row weights, channel
    weights, an image read through rows-outer strides)."""
    rng = np.random.default_rng(7)
    k, G, Rd, Cd = 5, 3, 7, 9
    img = rng.random((k, Rd, G, Cd))
    W = rng.random((k, G, Cd))
    rows = rng.random((k, G, Rd))
    sets = []
    for T1, T2 in ((11, 2), (6, 5)):
        n1 = np.sort(rng.random(T1)) * 0.8
        n2 = np.sort(rng.random(T2)) * 0.9
        sets.append(dict(tc=rng.normal(0, 0.3, (2, k, Cd)), tp=rng.normal(0, 0.2, (2, Rd, Cd)),
                         table=rng.random((G, T1, T2)), n1=n1, n2=n2))
    ref = img.transpose(0, 2, 1, 3) * W[:, :, None, :] * rows[:, :, :, None]
    for s in sets:
        th1 = np.abs(s["tc"][0][:, None, :] + s["tp"][0][None])       # [k, Rd, Cd]
        th2 = np.abs(s["tc"][1][:, None, :] + s["tp"][1][None])
        t = np.stack([[_bilinear(s["table"][g], s["n1"], s["n2"], th1[kk], th2[kk]) for g in range(G)]
                      for kk in range(k)])                             # [k, G, Rd, Cd]
        ref = ref * t
    ref_pg = ref.sum(0)
    dev = lambda x: torch.as_tensor(np.ascontiguousarray(x), dtype=torch.float32, device=cuda_device)  # noqa: E731
    keep = [dict((key, dev(v)) for key, v in s.items()) for s in sets]
    host = HostArgs()
    out = torch.zeros(G, Rd, Cd, device=cuda_device)
    x, W_dev, rows_dev = dev(img), dev(W), dev(rows)
    ptrs = lambda key: host.pointers([s[key].data_ptr() for s in keep])  # noqa: E731
    args = (x.data_ptr(), k, G, Rd, Cd, Rd * G * Cd, Cd, G * Cd, 1, W_dev.data_ptr(), Cd, rows_dev.data_ptr(), 2,
            ptrs("tc"), ptrs("tp"), ptrs("table"), ptrs("n1"), host.int64s([11, 6]), ptrs("n2"),
            host.int64s([2, 5]))
    _lib.call("citrus_grid_signal_sum", *args, out.data_ptr(), 1, 0, _lib.stream_handle(cuda_device))
    assert rel_err(out, ref_pg) < 2e-6
    total = torch.zeros(Rd, Cd, device=cuda_device)
    _lib.call("citrus_grid_signal_sum", *args, total.data_ptr(), 0, 0, _lib.stream_handle(cuda_device))
    assert rel_err(total, ref_pg.sum(0)) < 2e-6


def _bilinear(table, n1, n2, x1, x2):
    """[...] bilinear value of table [T1, T2] at x1, x2 (clamped to the end nodes)."""
    def idx(nodes, x):
        xc = np.clip(x, nodes[0], nodes[-1])
        hi = np.clip(np.searchsorted(nodes, xc, side="right"), 1, nodes.size - 1)
        lo = hi - 1
        return lo, hi, np.clip((xc - nodes[lo]) / (nodes[hi] - nodes[lo]), 0, 1)
    a0, a1, w1 = idx(n1, x1)
    b0, b1, w2 = idx(n2, x2)
    lo = table[a0, b0] * (1 - w2) + table[a0, b1] * w2
    hi = table[a1, b0] * (1 - w2) + table[a1, b1] * w2
    return lo * (1 - w1) + hi * w1
