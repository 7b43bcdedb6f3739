"""The oracle and the host set-up tables against fixtures generated from the reference (CPU only)."""

from __future__ import annotations

import numpy as np
import pytest

from conftest import check_regression_case, golden, rel_err
from citrus_gb300.geometry import Grid
from citrus_gb300.quadrature import Quadrature, hemisphere_quadrature, product_quadrature, real_spherical_harmonics
from citrus_gb300.transport_sweep import build_sweep_plan
from oracle import sweep as osweep


def test_product_quadrature_and_harmonics_match_reference():
    g = golden("quadrature_tables")
    for p, a, L in ((4, 12, 3), (6, 20, 5), (10, 24, 7)):
        q = product_quadrature(p, a)
        np.testing.assert_allclose(q.omega, g[f"omega_{p}x{a}"], rtol=0, atol=1e-15)
        np.testing.assert_allclose(q.weight, g[f"weight_{p}x{a}"], rtol=0, atol=1e-15)
        np.testing.assert_allclose(real_spherical_harmonics(L, q.omega), g[f"Y_{p}x{a}_L{L}"], rtol=0, atol=1e-13)


def test_cone_set_with_cell_widths_matches_reference():
    g = golden("quadrature_tables")
    cone = hemisphere_quadrature([0.3, -0.9, 0.1], 8, 16, 0.4, tangent_axes=((0.9, 0.3, 0.0), (0.0, 0.0, 1.0)))
    np.testing.assert_allclose(cone.omega, g["cone_omega"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(cone.weight, g["cone_weight"], rtol=0, atol=1e-15)
    np.testing.assert_allclose(cone.cell_width, g["cone_width"], rtol=1e-12, atol=1e-14)


def test_sweep_plan_matches_reference():
    g = golden("sweep_small")
    plan = build_sweep_plan(tuple(g["shape"]))
    np.testing.assert_array_equal(plan.plane_offsets, g["plane_offsets"])
    np.testing.assert_array_equal(plan.octant, g["octant"])
    np.testing.assert_array_equal(plan.cell, g["cell"])
    np.testing.assert_array_equal(plan.upstream, g["upstream"])
    offsets, octant, cell, upstream = osweep.plan(tuple(g["shape"]))
    np.testing.assert_array_equal(offsets, g["plane_offsets"])
    np.testing.assert_array_equal(upstream, g["upstream"])


def test_octant_reordering_matches_reference():
    g = golden("sweep_small")
    q = product_quadrature(4, 8)
    perm = q.by_octant()
    np.testing.assert_array_equal(perm, g["permutation"])
    np.testing.assert_allclose(q.omega[perm], g["omega"], atol=0)


def test_oracle_sweep_matches_reference():
    g = golden("sweep_small")
    phi, psi = osweep.sweep(tuple(g["shape"]), tuple(g["deltas"]), g["omega"], g["weight"], int(g["L"]), g["mu"],
                            g["source"], direction_chunk=3)
    assert rel_err(psi, g["psi"]) < 1e-13
    assert rel_err(phi, g["phi"]) < 1e-13


def test_oracle_scatter_moments_matches_reference():
    g = golden("scatter_moments_small")
    assert rel_err(osweep.scatter_moments(g["transfer"], g["phi4"]), g["T4"]) < 1e-14
    assert rel_err(osweep.scatter_moments(g["transfer"], g["phi1"]), g["T1"]) < 1e-14


@pytest.mark.parametrize("axis, sign", [(a, s) for a in range(3) for s in (1, -1)])
def test_oracle_slab_against_one_dimensional_solution(axis, sign):
    """A slab along one axis, direction along that axis: the 3-D LD solve reduces to the 1-D textbook cell equations
    (reference tests/oracles/linear_discontinuous_slab_1d.py), solved here independently."""
    rng = np.random.default_rng(10 + axis)
    K, G = 7, 2
    deltas = (0.7, 1.3, 0.9)
    shape = [2, 2, 2]
    dim = {0: 1, 1: 0, 2: 2}[axis]
    shape[dim] = K
    direction = np.zeros(3)
    direction[axis] = sign
    # one direction per octant; the slab direction replaces its own octant's entry
    base = np.array([0.3, 0.5, 0.81]) / np.linalg.norm([0.3, 0.5, 0.81])
    omega = base[None] * osweep.SIGNS
    code = int((direction < 0) @ np.array([4, 2, 1]))
    omega[code] = direction
    weight = np.full(8, 4 * np.pi / 8)
    mu1 = rng.random((G, K)) * 1.5 + 0.05
    S0, S1 = rng.random((G, K)), rng.standard_normal((G, K)) * 0.3

    def along(v):
        view = [G, 1, 1, 1]
        view[1 + dim] = K
        return np.broadcast_to(v.reshape(view), (G, *shape)).copy()

    mu = along(mu1)
    src = np.zeros((8, G, 4, *shape))
    src[:, :, 0] = along(S0)
    src[:, :, 1 + axis] = along(S1)
    _, psi = osweep.sweep(tuple(shape), deltas, omega, weight, 1, mu, src)
    c = 1.0 / deltas[axis]
    for g in range(G):
        p0, p1 = np.zeros(K), np.zeros(K)
        psi_in = 0.0
        for kk in (range(K) if sign > 0 else range(K - 1, -1, -1)):
            A = np.array([[c + mu1[g, kk], c], [-3 * c, 3 * c + mu1[g, kk]]])
            b = np.array([S0[g, kk] + c * psi_in, sign * S1[g, kk] - 3 * c * psi_in])
            a0, a1 = np.linalg.solve(A, b)
            p0[kk], p1[kk] = a0, sign * a1
            psi_in = a0 + a1
        np.testing.assert_allclose(psi[code, g, 0], along(p0[None].repeat(G, 0))[g], atol=1e-12)
        np.testing.assert_allclose(psi[code, g, 1 + axis], along(p1[None].repeat(G, 0))[g], atol=1e-12)


def _siddon_setup():
    from citrus_gb300.geometry import ConeGeometry
    grid = Grid((6, 7, 5), 1.1, 0.9, 1.3, recon_slice_offset=0.4)
    geos = {name: ConeGeometry(30.0, 45.0, 5, 7, 1.7, 1.9, det_row_offset=0.3, det_channel_offset=-0.2,
                               use_curved_detector=curved) for name, curved in (("flat", False), ("curved", True))}
    return grid, geos


def finite_rel_err(a, b):
    a, b = np.asarray(a, dtype=np.float64), np.asarray(b, dtype=np.float64)
    assert np.array_equal(np.isinf(a), np.isinf(b))
    m = np.isfinite(b)
    return rel_err(a[m], b[m])


@pytest.mark.parametrize("name", ["flat", "curved"])
def test_oracle_siddon_matches_reference(name):
    from oracle import siddon
    g = golden("siddon_small")
    grid, geos = _siddon_setup()
    geo, angle, vol = geos[name], 0.7, g["volume"]
    np.testing.assert_allclose(geo.pixel_centers_np(angle), g[f"{name}_pixels"], atol=1e-12)
    src = geo.source_position(angle)
    assert rel_err(siddon.upstream_to_points(vol, grid, src, siddon.centers(grid).reshape(-1, 3)).reshape(vol.shape),
                   g[f"{name}_upstream"]) < 1e-12
    assert rel_err(siddon.upstream_to_points(vol, grid, src, g["points"]), g[f"{name}_to_points"]) < 1e-12
    assert rel_err(siddon.primary_project(vol, grid, geo, angle), g[f"{name}_primary"]) < 1e-12
    assert finite_rel_err(siddon.downstream_cumulative(vol, grid, geo, angle, g["omegas"]),
                          g[f"{name}_downstream"]) < 1e-12
    assert rel_err(siddon.oblique_project(vol, grid, geo, angle, g["omegas"]), g[f"{name}_oblique"]) < 1e-12


def test_c_oracle_sweep_matches_numpy_oracle():
    from oracle import native
    rng = np.random.default_rng(4)
    shape, G, Dc = (4, 5, 3), 3, 2
    N = int(np.prod(shape))
    c = rng.random((8, Dc, 3)) + 0.1
    mu = rng.random((N, G)) + 0.2
    src = rng.standard_normal((8, Dc, N, G, 4))
    expected = osweep.sweep_chunk(shape, c, mu, src)
    got = native.sweep_chunk(osweep.plan(shape), c, mu, src)
    assert rel_err(got, expected) < 1e-14


def _uncollided_setup():
    from citrus_gb300.cross_sections import BONE, WATER, spectral_library
    from citrus_gb300.geometry import ConeGeometry
    from citrus_gb300.workloads import bremsstrahlung_spectrum
    library = spectral_library(np.linspace(120.0, 40.0, 4), bremsstrahlung_spectrum(seed=3), [WATER, BONE], 3,
                               num_eta=101, fine_per_group=4)
    grid = Grid((4, 4, 6), 1.5)
    geos = {name: ConeGeometry(40.0, 60.0, 30, 40, 1.0, 1.0, use_curved_detector=curved)
            for name, curved in (("flat", False), ("curved", True))}
    return library, grid, geos


@pytest.mark.parametrize("name", ["flat", "curved"])
def test_oracle_uncollided_and_first_collision_match_reference(name):
    from oracle import physics
    g = golden("uncollided_small")
    library, grid, geos = _uncollided_setup()
    geo, angle, rho = geos[name], 0.3, g["rho"]
    phi = physics.uncollided_fluence(library, rho, grid, geo, angle)
    assert rel_err(phi, g[f"{name}_phi"]) < 1e-12
    om = g["omega"]
    assert rel_err(physics.first_collision_source(library, rho, phi, grid, geo, angle, om[::4]),
                   g[f"{name}_source"]) < 1e-12
    scale, beta, _, _ = physics.correction(library, rho, phi, grid, geo, angle, om, g["weight"])
    assert rel_err(scale, g[f"{name}_scale"]) < 1e-11 and rel_err(beta, g[f"{name}_beta"]) < 1e-10
    assert np.abs(g[f"{name}_beta"]).max() > 1e-3  # a non-trivial correction (Klein-Nishina kernel)
    assert rel_err(physics.first_collision_moments(library, rho, phi, grid, geo, angle, om[::4], scale, beta, 2),
                   g[f"{name}_moments"]) < 1e-12


def _image_setup():
    from citrus_gb300.geometry import ConeGeometry
    from citrus_gb300.responses import DetectorResponse
    g = golden("image_small")
    library, _, _ = _uncollided_setup()
    grid_q = Grid((6, 6, 4), 2.0)
    det = DetectorResponse(g["det_e"], g["det_theta"], g["det_table"])
    geos = {name: ConeGeometry(50.0, 80.0, 10, 14, 1.5, 1.5, det_channel_offset=0.4, use_curved_detector=curved)
            for name, curved in (("flat", False), ("curved", True))}
    return g, library, grid_q, det, geos


@pytest.mark.parametrize("name", ["flat", "curved"])
def test_oracle_image_and_primary_match_reference(name):
    from citrus_gb300.scatter_image import panel_direction_set
    from oracle import image as oimage
    from oracle import physics
    g, library, grid_q, det, geos = _image_setup()
    geo, angle = geos[name], 0.8
    grid_c = grid_q.coarsen(2)
    rho = g["rho"]
    rho_c = rho.reshape(2, 3, 2, 3, 2, 2, 2).mean(axis=(2, 4, 6))
    mu_c = np.einsum("mg,mijk->gijk", library.mu_t, rho_c)
    phi = physics.uncollided_fluence(library, rho, grid_q, geo, angle)
    assert rel_err(phi, g[f"{name}_phi"]) < 1e-12
    cone = panel_direction_set(geo, angle, (3, 6), max_polar_angle=grid_c)
    np.testing.assert_allclose(cone.omega, g[f"{name}_cone_omega"], atol=1e-13)
    np.testing.assert_allclose(cone.cell_width, g[f"{name}_cone_width"], rtol=1e-10, atol=1e-13)
    img = oimage.combined_image(library, rho, phi, grid_q, 2, g["T"], 2, geo, angle, cone.omega, cone.weight,
                                cone.cell_width, mu_c, det)
    assert rel_err(img["fluence"], g[f"{name}_fluence"]) < 1e-11
    assert rel_err(img["planar_fluence"], g[f"{name}_planar"]) < 1e-11
    assert rel_err(img["signal_per_group"], g[f"{name}_signal_pg"]) < 1e-11
    assert rel_err(img["signal"], g[f"{name}_signal_only"]) < 1e-11
    prim = oimage.primary(library, rho, grid_q, geo, angle, det)
    assert rel_err(prim["signal"], g[f"{name}_primary_signal"]) < 1e-12
    assert rel_err(prim["fluence"], g[f"{name}_primary_fluence"]) < 1e-12


# ---- the reference's own regression anchor and the single-view workload ---------------------------------------------

def test_pre_quadrature_fixture_reproduces_the_reference_golden_case():
    """The fixture's solve (the reference's float64 CPU path run on the stored inputs) reproduces the reference's
    committed regression case ``synthetic_cpu`` at its own tolerance, 1e-10: the inputs are pinned."""
    g = golden("pre_quadrature_synthetic")
    check_regression_case(g["scatter_signal"], g["primary_signal"], g["si_iterations"], float(g["si_history"][-1]),
                          g, "synthetic_cpu", 1e-10)


def test_seven_material_synthetic_library_matches_reference():
    from citrus_gb300.cross_sections import synthetic_library
    g = golden("pre_quadrature_synthetic")
    lib = synthetic_library(4, 5, num_materials=7)
    for k in ("group_edges", "group_energy", "spectrum_fraction", "mu_t", "mu_pe", "mu_s_l", "eta_grid", "mu_s_eta",
              "fine_energy", "fine_mu_t", "fine_weight", "fine_group", "nominal_density"):
        np.testing.assert_allclose(getattr(lib, k), g[f"lib_{k}"], rtol=0, atol=1e-15)
    assert lib.materials == tuple(str(m) for m in g["lib_materials"])


def test_single_view_workload_densities_match_the_fixture():
    from citrus_gb300.workloads import single_view
    np.testing.assert_array_equal(single_view().rho, golden("config1_view")["rho"])


# ---- the library's on-disk format ------------------------------------------------------------------------------------

def test_library_file_written_by_the_reference_loads():
    from citrus_gb300.cross_sections import MultigroupLibrary, synthetic_library
    from conftest import GOLDEN
    lib = MultigroupLibrary.load(str(GOLDEN / "reference_library.pt"))
    ours = synthetic_library(3, 2, num_eta=21, num_fine_per_group=2)
    for k in MultigroupLibrary._FIELDS + ("nominal_density",):  # torch and numpy linspace differ in the last bit
        np.testing.assert_allclose(getattr(lib, k), getattr(ours, k), rtol=1e-15, atol=1e-16)
    assert lib.materials == ("water", "bone_cortical_icrp")


def test_library_file_written_here_has_the_reference_format(tmp_path):
    """save() writes what the reference's MultigroupLibrary.load reads: the same keys, tensor dtypes and shapes as a
    file written by the reference's own save, and the same values; load() reads it back unchanged."""
    import torch
    from citrus_gb300.cross_sections import MultigroupLibrary
    from conftest import GOLDEN
    reference = torch.load(str(GOLDEN / "reference_library.pt"), weights_only=True)
    lib = MultigroupLibrary.load(str(GOLDEN / "reference_library.pt"))
    lib.save(str(tmp_path / "lib.pt"))
    ours = torch.load(str(tmp_path / "lib.pt"), weights_only=True)
    assert set(ours) == set(reference)
    for k, v in reference.items():
        if isinstance(v, torch.Tensor):
            assert ours[k].dtype == v.dtype and ours[k].shape == v.shape and torch.equal(ours[k], v), k
        else:
            assert ours[k] == v, k
    again = MultigroupLibrary.load(str(tmp_path / "lib.pt"))
    for k in MultigroupLibrary._FIELDS:
        np.testing.assert_array_equal(getattr(again, k), getattr(lib, k))


def test_library_file_errors(tmp_path):
    import torch
    from citrus_gb300.cross_sections import MultigroupLibrary
    from conftest import GOLDEN
    fields = torch.load(str(GOLDEN / "reference_library.pt"), weights_only=True)
    del fields["mu_pe"]
    torch.save(fields, str(tmp_path / "missing.pt"))
    with pytest.raises(KeyError):
        MultigroupLibrary.load(str(tmp_path / "missing.pt"))
    fields = torch.load(str(GOLDEN / "reference_library.pt"), weights_only=True)
    fields["eta_map"] = torch.linspace(1.0, 0.0, 9, dtype=torch.float64)
    torch.save(fields, str(tmp_path / "adaptive.pt"))
    with pytest.raises(ValueError):
        MultigroupLibrary.load(str(tmp_path / "adaptive.pt"))
