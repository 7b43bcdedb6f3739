"""The anti-scatter grid and the source model on the host, and their oracle, against the reference's own values
(``tests/golden/grid_and_source.npz``, made by ``make_golden.py grid_and_source``)."""

from __future__ import annotations

import math
from dataclasses import replace

import numpy as np
import pytest
import torch

from conftest import golden
from citrus_gb300.geometry import ConeGeometry, Grid
from citrus_gb300.responses import (FilterMaterial, GridResponse, SourceModel, focused_1d_grid, grid_angles, no_grid,
                                    panel_interpolate_np)
from oracle import responses as oresp

FOCALS = ((None, "default"), (math.inf, "unfocused"), (120.0, "f120"))


def fixture_grid(g=None) -> GridResponse:
    """The reference's focused 1-D grid, rebuilt from its lead attenuation at the table energies."""
    g = golden("grid_and_source") if g is None else g
    e, mu = g["grid_energy"], g["lead_mu"]
    return focused_1d_grid(lambda x: np.interp(x, e, mu), energies=e)


def filter_attenuation(e):
    """The synthetic filter attenuation the fixture was made with."""
    return 0.16 + 4.0 * (np.asarray(e, dtype=np.float64) / 30.0) ** -2.8


def fixture_source(g, name) -> SourceModel:
    return SourceModel(emission_profile=g[f"source_{name}_profile"], field_margin_channels_cm=0.5,
                       field_margin_rows_cm=0.25, off_focal_distance_cm=[0.0, 1.0, 3.0],
                       off_focal_fraction=[0.3, 0.1, 0.02],
                       filter_material=FilterMaterial("filter", 2.7, filter_attenuation),
                       filter_thickness_cm=g[f"source_{name}_thickness"])


def image_geometry(curved: bool) -> ConeGeometry:
    return ConeGeometry(50.0, 80.0, 10, 14, 1.5, 1.5, det_channel_offset=0.4, use_curved_detector=curved)


def test_focused_grid_table_matches_reference():
    g = golden("grid_and_source")
    grid = fixture_grid(g)
    assert grid.focal_distance_cm == float(g["grid_focal"])
    np.testing.assert_array_equal(grid.theta1_rad, g["grid_theta1"])
    np.testing.assert_array_equal(grid.theta2_rad, g["grid_theta2"])
    np.testing.assert_allclose(grid.transmission, g["grid_table"], rtol=0, atol=1e-15)
    # falls with the angle, symmetric in its sign, independent of theta2, transmission 1 without a grid
    th1 = np.array([0.0, 0.01, 0.03, 0.06, 0.2])
    e = np.array([30.0, 60.0])
    t = grid.at(e, th1, 0 * th1)
    assert np.all(t[:, 1:] < t[:, :-1]) and np.all((t > 0) & (t <= 1))
    np.testing.assert_array_equal(grid.at(e, -th1, 0 * th1), t)
    np.testing.assert_array_equal(grid.at(e, th1, 0.4 + 0 * th1), t)
    assert np.all(no_grid().at(e, th1, th1) == 1)


@pytest.mark.parametrize("curved", [False, True])
@pytest.mark.parametrize("septa", ["channels", "rows"])
def test_grid_angles_match_reference(curved, septa):
    g = golden("grid_and_source")
    geo = ConeGeometry(100.0, 150.0, 5, 7, 4.0, 4.0, det_row_offset=1.0, use_curved_detector=curved)
    pix = geo.pixel_centers_np(0.9)
    pre = "curved" if curved else "flat"
    for focal, fname in FOCALS:
        for th1, th2 in (grid_angles(g["angles_omega"], pix, geo, 0.9, focal, septa),
                         oresp.grid_angles(g["angles_omega"], pix, geo, 0.9, focal, septa)):
            assert th1.shape == (6, 5, 7)
            np.testing.assert_allclose(th1, g[f"angles_{pre}_{septa}_{fname}_theta1"], rtol=0, atol=1e-13)
            np.testing.assert_allclose(th2, g[f"angles_{pre}_{septa}_{fname}_theta2"], rtol=0, atol=1e-13)
    sep = replace(fixture_grid(g), septa_along=septa)
    np.testing.assert_allclose(sep.transmission_at(g["angles_energy"], g["angles_omega"], pix, geo, 0.9),
                               g[f"transmission_{pre}_{septa}"], rtol=1e-13, atol=1e-15)


@pytest.mark.parametrize("curved", [False, True])
def test_crossed_grid_transmission_matches_reference(curved):
    g = golden("grid_and_source")
    geo = ConeGeometry(100.0, 150.0, 5, 7, 4.0, 4.0, det_row_offset=1.0, use_curved_detector=curved)
    grid = fixture_grid(g)
    crossed = replace(grid, crossed=replace(grid, septa_along="rows"))
    assert crossed.depends_on_angles and len(crossed.septa_sets()) == 2
    ref = g[f"transmission_{'curved' if curved else 'flat'}_crossed"]
    got = crossed.transmission_at(g["angles_energy"], g["angles_omega"], geo.pixel_centers_np(0.9), geo, 0.9)
    np.testing.assert_allclose(got, ref, rtol=1e-13, atol=1e-15)
    oracle = oresp.grid_transmission(crossed, g["angles_omega"], geo, 0.9, g["angles_energy"])
    np.testing.assert_allclose(oracle.transpose(1, 0, 2, 3), ref, rtol=1e-12, atol=1e-15)


@pytest.mark.parametrize("curved", [False, True])
def test_source_weight_and_filter_path_match_reference(curved):
    """b(Omega) with field margins, an off-focal table and an emission profile, and the filter path, at points
    inside, at the margins and past the field edge."""
    g = golden("grid_and_source")
    pre = "curved" if curved else "flat"
    geo = image_geometry(curved)
    src = fixture_source(g, pre)
    d = (Grid((8, 10, 6), 3.0).center_coordinates(dtype=torch.float64).reshape(-1, 3).numpy()
         - np.asarray(geo.source_position(0.8)))
    ref_b, ref_f = g[f"source_{pre}_b"], g[f"source_{pre}_filter_path"]
    assert (ref_b == 0).any() and ((ref_b > 0) & (ref_b < 1)).any()   # the sample reaches the off-focal table
    np.testing.assert_allclose(src.angular_weight_np(d, geo, 0.8), ref_b, rtol=1e-13, atol=1e-15)
    np.testing.assert_allclose(src.filter_path_np(d, geo, 0.8), ref_f, rtol=1e-13, atol=1e-15)
    ob = oresp.source_weight(geo, 0.8, d, (0.5, 0.25), ([0.0, 1.0, 3.0], [0.3, 0.1, 0.02]),
                             g[f"source_{pre}_profile"])
    np.testing.assert_allclose(ob, ref_b, rtol=1e-12, atol=1e-15)
    of = oresp.filter_path(geo, 0.8, d, g[f"source_{pre}_thickness"], 2.7)
    np.testing.assert_allclose(of, ref_f, rtol=1e-12, atol=1e-15)


def test_septa_dependence_of_the_image_routes():
    """How the context factors each grid (the reference's scatter-image routes): per row, per channel, per pixel."""
    from citrus_gb300.responses import ideal_counting_response
    from citrus_gb300.scatter_image import make_direction_context, panel_direction_set
    from test_oracle_golden import _uncollided_setup
    library, _, _ = _uncollided_setup()
    grid = fixture_grid()
    rows = replace(grid, septa_along="rows")
    crossed = replace(grid, crossed=rows)
    expect = {"flat_rows": (False, grid, ("rows",)), "flat_channels": (False, rows, ("channels",)),
              "flat_crossed": (False, crossed, ("rows", "channels")), "curved_rows": (True, rows, ("channels",)),
              "curved_pixel": (True, grid, ("sum",)), "curved_crossed": (True, crossed, ("sum", "channels")),
              "none": (False, no_grid(), ("none",))}
    for name, (curved, response, kinds) in expect.items():
        geo = image_geometry(curved)
        cone = panel_direction_set(geo, 0.8, (3, 6), max_polar_angle=Grid((3, 3, 2), 4.0))
        ctx = make_direction_context(cone, geo, 0.8, ideal_counting_response(), response, library, "cpu", chunk=5)
        assert ctx.septa_kinds == kinds, name
        assert ctx.grid_varies_over_panel == (name in ("flat_rows", "flat_crossed", "curved_pixel",
                                                       "curved_crossed")), name
        assert (ctx.signal_group_weight is not None) == (name == "none"), name


def test_panel_interpolation_holds_the_edges():
    geo = ConeGeometry(50.0, 80.0, 3, 4, 1.0, 2.0, det_channel_offset=0.5)
    img = np.arange(12.0).reshape(3, 4)
    u, v = geo.pixel_uv()
    np.testing.assert_allclose(panel_interpolate_np(img, u[None, :], v[:, None], geo), img, atol=1e-12)
    assert panel_interpolate_np(img, np.array(1e3), np.array(-1e3), geo) == img[0, -1]
    mid = panel_interpolate_np(img, np.array(0.5 * (u[0] + u[1])), np.array(v[1]), geo)
    assert mid == pytest.approx(0.5 * (img[1, 0] + img[1, 1]))


def test_grid_and_source_reject_bad_tables():
    e, t = np.array([1.0, 100.0]), np.array([0.0, 1.0])
    with pytest.raises(ValueError, match="transmission must be"):
        GridResponse(e, t, t, np.ones((2, 3, 2)))
    with pytest.raises(ValueError, match="septa_along"):
        GridResponse(e, t, t, np.ones((2, 2, 2)), septa_along="diagonal")
    g = GridResponse(e, t, t, np.ones((2, 2, 2)))
    with pytest.raises(ValueError, match="crossed"):
        replace(g, crossed=g)
    angled = GridResponse(e, t, t, np.arange(8.0).reshape(2, 2, 2))
    with pytest.raises(ValueError, match="transmission_at"):
        angled.at_energy([50.0])
    with pytest.raises(ValueError, match="together"):
        SourceModel(off_focal_distance_cm=[1.0])
    with pytest.raises(ValueError, match="ascending"):
        SourceModel(off_focal_distance_cm=[1.0, 0.5], off_focal_fraction=[0.1, 0.1])
    with pytest.raises(ValueError, match="together"):
        SourceModel(filter_thickness_cm=[0.1, 0.2])
    with pytest.raises(ValueError, match="emission_profile_angles"):
        SourceModel(emission_profile=np.ones((2, 3, 4)))
    src = SourceModel(emission_profile=np.stack([np.ones((3, 4)), 2 * np.ones((3, 4))]),
                      emission_profile_angles=[0.0, 1.0])
    assert src.profile_at(0.9)[0, 0] == 2.0 and src.profile_at(0.2)[0, 0] == 1.0


def test_group_averaged_responses_match_reference():
    """Detector and crossed-grid tables averaged over each group's fine energies, as the reference's
    ``group_averaged_responses`` makes them for ``SolverConfig.group_averaged_responses``."""
    from citrus_gb300.responses import DetectorResponse, group_averaged_responses
    from test_oracle_golden import _uncollided_setup
    g = golden("grid_and_source")
    library, _, _ = _uncollided_setup()
    ig = golden("image_small")
    det = DetectorResponse(ig["det_e"], ig["det_theta"], ig["det_table"])
    grid = fixture_grid(g)
    crossed = replace(grid, crossed=replace(grid, septa_along="rows"))
    avg_det, avg_grid = group_averaged_responses(det, crossed, library)
    np.testing.assert_allclose(avg_det.energy_kev, g["avg_det_energy"], rtol=1e-15)
    np.testing.assert_allclose(avg_det.response, g["avg_det_table"], rtol=1e-13)
    np.testing.assert_allclose(avg_grid.energy_kev, g["avg_grid_energy"], rtol=1e-15)
    np.testing.assert_allclose(avg_grid.transmission, g["avg_grid_table"], rtol=1e-13)
    np.testing.assert_allclose(avg_grid.crossed.energy_kev, g["avg_crossed_energy"], rtol=1e-15)
    np.testing.assert_allclose(avg_grid.crossed.transmission, g["avg_crossed_table"], rtol=1e-13)
    # evaluated at a group energy, the averaged table returns the group's mean
    e = np.asarray(library.group_energy)
    np.testing.assert_allclose(avg_det.at(e, [0.0])[:, 0], avg_det.response[1::2, 0][::-1], rtol=1e-13)


@pytest.mark.parametrize("curved", [False, True])
def test_oracle_primary_and_uncollided_with_source_and_grid_match_reference(curved):
    """The oracle's primary (2 x 2 sub-rays and one ray per pixel) behind the focused grid and its uncollided fluence,
    both with the profiled, off-focal, filtered source, against the reference's own float64 runs."""
    from oracle import image as oimage
    from oracle import physics
    from test_oracle_golden import _image_setup
    g = golden("grid_and_source")
    _, library, _, det, _ = _image_setup()
    pre = "curved" if curved else "flat"
    geo = image_geometry(curved)
    big = Grid((8, 10, 6), 3.0)
    source = dict(margins=(0.5, 0.25), off_focal=([0.0, 1.0, 3.0], [0.3, 0.1, 0.02]),
                  profile=g[f"source_{pre}_profile"], thickness=g[f"source_{pre}_thickness"], filter_density=2.7,
                  filter_mu=filter_attenuation(library.fine_energy))
    for n, key in ((1, f"source_{pre}_primary"), (2, f"source_{pre}_primary_n2")):
        got = oimage.primary_with_source(library, g[f"source_{pre}_rho"], big, geo, 0.8, det, n=n,
                                         grid_response=fixture_grid(g), **source)
        np.testing.assert_allclose(got, g[key], rtol=0, atol=1e-12 * np.abs(g[key]).max())
    phi = physics.uncollided_fluence_with_source(library, g[f"source_{pre}_rho"], big, geo, 0.8, **source)
    ref = g[f"source_{pre}_phi"]
    np.testing.assert_allclose(phi, ref, rtol=0, atol=1e-12 * np.abs(ref).max())


@pytest.mark.parametrize("name", ["flat_rows", "flat_channels", "flat_crossed", "curved_rows", "curved_pixel",
                                  "curved_crossed"])
def test_oracle_image_behind_grid_matches_reference(name):
    """The oracle's collapsed-cone image with the grid's transmission evaluated at every direction and pixel against
    the reference's image of the same route (its own per-row, per-channel and per-pixel factoring)."""
    from citrus_gb300.scatter_image import panel_direction_set
    from oracle import image as oimage
    from test_oracle_golden import _image_setup
    g = golden("grid_and_source")
    _, library, grid_q, det, _ = _image_setup()
    grid = fixture_grid(g)
    rows = replace(grid, septa_along="rows")
    curved, response = {"flat_rows": (False, grid), "flat_channels": (False, rows),
                        "flat_crossed": (False, replace(grid, crossed=rows)), "curved_rows": (True, rows),
                        "curved_pixel": (True, grid), "curved_crossed": (True, replace(grid, crossed=rows))}[name]
    geo, angle = image_geometry(curved), 0.8
    grid_c = grid_q.coarsen(2)
    rho = g["image_rho"]
    rho_c = rho.reshape(2, 3, 2, 3, 2, 2, 2).mean(axis=(2, 4, 6))
    mu_c = np.einsum("mg,mijk->gijk", library.mu_t, rho_c)
    cone = panel_direction_set(geo, angle, (3, 6), max_polar_angle=grid_c)
    got = oimage.combined_image(library, rho, g[f"image_{name}_phi"], grid_q, 2, g["image_T"], 2, geo, angle,
                                cone.omega, cone.weight, cone.cell_width, mu_c, det, grid=response)
    ref = g[f"image_{name}_signal_pg"]
    np.testing.assert_allclose(got["signal_per_group"], ref, rtol=0, atol=1e-10 * np.abs(ref).max())
