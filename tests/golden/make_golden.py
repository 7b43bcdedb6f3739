"""Generate the golden fixtures of the test suite by running the reference itself (cabouman/citrus v0.28.0).

Run in a checkout beside the reference, with CITRUS_REFERENCE set to its root (the directory that holds ``citrus/``
and ``tests/data/``). The reference imports xraylib at module level for element tables only; ``_shims/xraylib.py``
stands in for it (the synthetic library used here never reads those tables). Every fixture is small, float64, and
produced by the reference's own float64 CPU path; the script is deterministic (seeded).

    python tests/golden/make_golden.py [case ...]
"""

from __future__ import annotations

import math
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REFERENCE = os.environ.get("CITRUS_REFERENCE")
if not REFERENCE:
    sys.exit("set CITRUS_REFERENCE to the root of a cabouman/citrus v0.28.0 checkout")
sys.path[:0] = [str(HERE / "_shims"), REFERENCE]

import torch  # noqa: E402

F64 = torch.float64
CASES = {}


def case(fn):
    CASES[fn.__name__] = fn
    return fn


def save(name, **arrays):
    out = {}
    for k, v in arrays.items():
        out[k] = v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else np.asarray(v)
    np.savez_compressed(HERE / f"{name}.npz", **out)
    size = (HERE / f"{name}.npz").stat().st_size
    print(f"{name}.npz: {len(out)} arrays, {size / 1024:.1f} KiB")


@case
def sweep_small():
    """Reference sweep (PyTorch path, float64) of a random direction-dependent source on an anisotropic grid."""
    from citrus.scatter_solver.angular_quadrature import product_quadrature
    from citrus.scatter_solver.geometry import Grid
    from citrus.scatter_solver.transport_sweep import make_sweep_context, sweep

    g = torch.Generator().manual_seed(1234)
    grid = Grid((3, 4, 5), 0.7, 1.3 / 0.7, 0.9 / 0.7)
    quadrature = product_quadrature(4, 8, dtype=F64)
    L, G = 2, 3
    ctx = make_sweep_context(grid, quadrature, L, device="cpu", dtype=F64, backend="torch")
    mu = torch.rand(G, *grid.shape, generator=g, dtype=F64) * 1.5 + 0.1
    src = torch.randn(ctx.num_directions, G, 4, *grid.shape, generator=g, dtype=F64)
    phi, psi = sweep(ctx, mu, lambda idx: src.index_select(0, idx), direction_chunk=3, return_psi=True)
    save("sweep_small", shape=np.array(grid.shape), deltas=np.array(grid.deltas), L=L, mu=mu, source=src,
         omega=ctx.quadrature.omega, weight=ctx.quadrature.weight, permutation=ctx.permutation, phi=phi, psi=psi,
         c=ctx.c, plane_offsets=ctx.plan.plane_offsets, octant=ctx.plan.octant, cell=ctx.plan.cell,
         upstream=ctx.plan.upstream)


@case
def quadrature_tables():
    """Sweep product sets, harmonics and a cone set with cell widths."""
    from citrus.scatter_solver.angular_quadrature import (hemisphere_quadrature, product_quadrature,
                                                          real_spherical_harmonics)

    arrays = {}
    for p, a, L in ((4, 12, 3), (6, 20, 5), (10, 24, 7)):
        q = product_quadrature(p, a, dtype=F64)
        arrays[f"omega_{p}x{a}"] = q.omega
        arrays[f"weight_{p}x{a}"] = q.weight
        arrays[f"Y_{p}x{a}_L{L}"] = real_spherical_harmonics(L, q.omega)
    cone = hemisphere_quadrature([0.3, -0.9, 0.1], 8, 16, 0.4, dtype=F64, tangent_axes=((0.9, 0.3, 0.0),
                                                                                         (0.0, 0.0, 1.0)))
    arrays.update(cone_omega=cone.omega, cone_weight=cone.weight, cone_width=cone.cell_width)
    save("quadrature_tables", **arrays)


@case
def scatter_moments_small():
    """Scattering-source moments with and without the LD axis (angular_quadrature.scatter_source_moments)."""
    from citrus.scatter_solver.angular_quadrature import scatter_source_moments

    g = torch.Generator().manual_seed(77)
    G, L, spatial = 3, 2, (3, 4, 5)
    transfer = torch.rand(G, G, L + 2, *spatial, generator=g, dtype=F64)
    transfer[1, 0] = 0.0
    phi4 = torch.randn(G, (L + 1) ** 2, 4, *spatial, generator=g, dtype=F64)
    phi1 = torch.randn(G, (L + 1) ** 2, *spatial, generator=g, dtype=F64)
    save("scatter_moments_small", transfer=transfer, phi4=phi4, phi1=phi1,
         T4=scatter_source_moments(transfer, phi4), T1=scatter_source_moments(transfer, phi1))


@case
def siddon_small():
    """The five Siddon ray operations of the reference (PyTorch path, float64) on a small anisotropic grid, with a flat
    and a curved panel."""
    from citrus.scatter_solver.geometry import ConeGeometry, Grid
    from citrus.scatter_solver.ray_tracing import SiddonProjectors

    g = torch.Generator().manual_seed(99)
    grid = Grid((6, 7, 5), 1.1, 0.9, 1.3, recon_slice_offset=0.4)
    vol = torch.rand(2, *grid.shape, generator=g, dtype=F64)
    proj = SiddonProjectors(backend="torch")
    arrays = dict(volume=vol)
    omegas = torch.nn.functional.normalize(torch.randn(5, 3, generator=g, dtype=F64), dim=-1)
    points = (torch.rand(20, 3, generator=g, dtype=F64) - 0.5) * 14.0
    arrays.update(omegas=omegas, points=points)
    for name, curved in (("flat", False), ("curved", True)):
        geo = ConeGeometry(30.0, 45.0, 5, 7, 1.7, 1.9, det_row_offset=0.3, det_channel_offset=-0.2,
                           use_curved_detector=curved)
        angle = 0.7
        arrays[f"{name}_upstream"] = proj.upstream_cumulative(vol, grid, geo, angle)
        arrays[f"{name}_to_points"] = proj.upstream_to_points(vol, grid, geo, angle, points)
        arrays[f"{name}_primary"] = proj.primary_project(vol, grid, geo, angle)
        arrays[f"{name}_primary_n2"] = proj.primary_project(vol, grid, geo, angle, samples_per_pixel_axis=2)
        down = proj.downstream_cumulative(vol, grid, geo, angle, omegas)
        arrays[f"{name}_downstream"] = down
        arrays[f"{name}_oblique"] = proj.oblique_project(vol, grid, geo, angle, omegas)
        arrays[f"{name}_pixels"] = geo.pixel_centers(angle, dtype=F64)
    save("siddon_small", **arrays)


def small_spectral_library():
    """A three-group Klein-Nishina library from citrus_gb300 (its fields are plain arrays; the reference reads them)."""
    sys.path.insert(0, str(HERE.parent.parent))
    from citrus_gb300.cross_sections import BONE, WATER, spectral_library
    from citrus_gb300.workloads import bremsstrahlung_spectrum
    return spectral_library(np.linspace(120.0, 40.0, 4), bremsstrahlung_spectrum(seed=3), [WATER, BONE], 3,
                            num_eta=101, fine_per_group=4)


def reference_library(lib):
    """The reference's MultigroupLibrary holding the same float64 tables."""
    from citrus.scatter_solver.cross_sections import MultigroupLibrary
    t = lambda a: torch.as_tensor(np.asarray(a), dtype=F64)  # noqa: E731
    return MultigroupLibrary(group_edges=t(lib.group_edges), group_energy=t(lib.group_energy),
                             spectrum_fraction=t(lib.spectrum_fraction), mu_t=t(lib.mu_t), mu_pe=t(lib.mu_pe),
                             mu_s_l=t(lib.mu_s_l), eta_grid=t(lib.eta_grid), mu_s_eta=t(lib.mu_s_eta),
                             fine_energy=t(lib.fine_energy), fine_mu_t=t(lib.fine_mu_t),
                             fine_weight=t(lib.fine_weight), fine_group=torch.as_tensor(lib.fine_group),
                             materials=tuple(lib.materials), nominal_density=t(lib.nominal_density))


@case
def uncollided_small():
    """Uncollided fluence, first-collision source, sampling correction and LD moments (q = 2) of the reference on a
    small grid with the synthetic two-material library, flat and curved panels."""
    from citrus.scatter_solver.angular_quadrature import product_quadrature
    from citrus.scatter_solver.cross_sections import synthetic_library
    from citrus.scatter_solver.geometry import ConeGeometry, Grid
    from citrus.scatter_solver.ray_tracing import SiddonProjectors
    from citrus.scatter_solver.source import SourceModel
    from citrus.scatter_solver.uncollided import (DENSE, first_collision_moments_at_directions,
                                                  first_collision_sampling_correction,
                                                  first_collision_source_at_directions, uncollided_fluence)

    g = torch.Generator().manual_seed(5)
    library = reference_library(small_spectral_library())
    grid = Grid((4, 4, 6), 1.5)
    rho = torch.rand(2, *grid.shape, generator=g, dtype=F64) * torch.tensor([1.0, 1.8], dtype=F64)[:, None, None, None]
    q = product_quadrature(4, 8, dtype=F64)
    arrays = dict(rho=rho, omega=q.omega, weight=q.weight)
    for name, curved in (("flat", False), ("curved", True)):
        geo = ConeGeometry(40.0, 60.0, 30, 40, 1.0, 1.0, use_curved_detector=curved)
        angle = 0.3
        phi = uncollided_fluence(library, rho, grid, geo, angle, SourceModel(), SiddonProjectors(backend="torch"))
        src = first_collision_source_at_directions(library, rho, phi, grid, geo, angle, q.omega[::4], pairs=DENSE)
        corr = first_collision_sampling_correction(library, rho, phi, grid, geo, angle, q.omega, q.weight, pairs=DENSE)
        mom = first_collision_moments_at_directions(library, rho, phi, grid, geo, angle, q.omega[::4], corr, 2,
                                                    pairs=DENSE)
        arrays.update({f"{name}_phi": phi, f"{name}_source": src, f"{name}_scale": corr.scale,
                       f"{name}_beta": corr.beta, f"{name}_moments": mom})
    save("uncollided_small", **arrays)


def scintillator_table():
    """A synthetic energy-integrating detector table D(E, theta) = E (1 - exp(-mu(E) t / cos theta))."""
    e = np.linspace(10.0, 150.0, 57)
    th = np.radians(np.linspace(0.0, 89.5, 46))
    mu = 0.9 * (e / 60.0) ** -2.5 + 0.1
    return e, th, e[:, None] * (-np.expm1(-mu[:, None] * 4.51 * 0.06 / np.cos(th)[None, :]))


@case
def image_small():
    """The reference's collapsed-cone image (full and signal-only) and primary of one view, flat and curved panels,
    with the three-group Klein-Nishina library and a synthetic scintillator response."""
    from citrus.scatter_solver.angular_quadrature import scatter_source_moments
    from citrus.scatter_solver.cross_sections import mu_t_volume, transfer_moments_volume
    from citrus.scatter_solver.detector import DetectorResponse, no_grid
    from citrus.scatter_solver.geometry import ConeGeometry, Grid
    from citrus.scatter_solver.ray_tracing import SiddonProjectors
    from citrus.scatter_solver.scatter_image import (combined_scatter_image, make_direction_context,
                                                     panel_direction_set, primary_image)
    from citrus.scatter_solver.source import SourceModel
    from citrus.scatter_solver.uncollided import DENSE, uncollided_fluence

    g = torch.Generator().manual_seed(21)
    library = reference_library(small_spectral_library())
    L = 2
    grid_q = Grid((6, 6, 4), 2.0)
    q = 2
    grid_c = grid_q.coarsen(q)
    rho = torch.rand(2, *grid_q.shape, generator=g, dtype=F64) * torch.tensor([1.0, 0.5], dtype=F64)[:, None, None,
                                                                                                         None]
    rho_c = rho.reshape(2, 3, 2, 3, 2, 2, 2).mean(dim=(2, 4, 6))
    mu_c = mu_t_volume(library, rho_c)
    phi_coll = torch.rand(library.num_groups, (L + 1) ** 2, *grid_c.shape, generator=g, dtype=F64) * 1e-4
    T = scatter_source_moments(transfer_moments_volume(library, rho_c)[:, :, :L + 1], phi_coll)
    e, th, table = scintillator_table()
    det = DetectorResponse(torch.as_tensor(e), torch.as_tensor(th), torch.as_tensor(table))
    arrays = dict(rho=rho, T=T, det_e=e, det_theta=th, det_table=table)
    for name, curved in (("flat", False), ("curved", True)):
        geo = ConeGeometry(50.0, 80.0, 10, 14, 1.5, 1.5, det_channel_offset=0.4, use_curved_detector=curved)
        angle = 0.8
        proj = SiddonProjectors(backend="torch")
        phi = uncollided_fluence(library, rho, grid_q, geo, angle, SourceModel(), proj)
        cone = panel_direction_set(geo, angle, (3, 6), max_polar_angle=grid_c, dtype=F64)
        grid_response = no_grid()
        ctx = make_direction_context(cone, geo, angle, det, grid_response, library, "cpu", F64, chunk=5)
        full = combined_scatter_image(library, rho, phi, grid_q, q, T, L, geo, angle, cone, mu_c, proj, det,
                                      grid_response, ctx, pairs=DENSE, grid_coarse=grid_c)
        sig = combined_scatter_image(library, rho, phi, grid_q, q, T, L, geo, angle, cone, mu_c, proj, det,
                                     grid_response, ctx, pairs=DENSE, grid_coarse=grid_c,
                                     signal_only=True)["signal"]
        prim = primary_image(library, rho, grid_q, geo, angle, SourceModel(), proj, det, grid_response)
        arrays.update({f"{name}_phi": phi, f"{name}_cone_omega": cone.omega, f"{name}_cone_weight": cone.weight,
                       f"{name}_cone_width": cone.cell_width, f"{name}_fluence": full["fluence"],
                       f"{name}_planar": full["planar_fluence"], f"{name}_signal_pg": full["signal_per_group"],
                       f"{name}_signal": full["signal"], f"{name}_signal_only": sig,
                       f"{name}_primary_signal": prim["signal"], f"{name}_primary_fluence": prim["fluence"]})
    save("image_small", **arrays)


STEP_CONFIG = dict(num_groups=3, legendre_order=2, num_polar=4, num_azimuthal=8, transport_cell_cm=2.0,
                   quadrature_point_spacing_cm=1.0, cone_num_polar=3, cone_num_azimuthal=6, direction_chunk=4,
                   source_iteration_tolerance=1e-4, max_source_iterations=40)


@case
def citrus_step_small():
    """Two CITRUS scatter steps of one view (citrus_view_step with the primary) and a converged solve_view of the
    reference's ScatterSolver, float64 CPU, flat and curved panels."""
    from citrus.citrus import CitrusState, citrus_view_step
    from citrus.scatter_solver.config import SolverConfig
    from citrus.scatter_solver.detector import DetectorResponse, no_grid
    from citrus.scatter_solver.geometry import ConeGeometry, Grid
    from citrus.scatter_solver.ray_tracing import SiddonProjectors
    from citrus.scatter_solver.scatter_solver import ScatterSolver

    g = torch.Generator().manual_seed(31)
    library = reference_library(small_spectral_library())
    grid = Grid((8, 8, 6), 1.0)
    rho = torch.zeros(2, *grid.shape, dtype=F64)
    rho[0] = 0.9 + 0.2 * torch.rand(*grid.shape, generator=g, dtype=F64)
    rho[1, 2:5, 3:6, 1:4] = 1.85
    rho[0, 2:5, 3:6, 1:4] = 0.0
    e, th, table = scintillator_table()
    det = DetectorResponse(torch.as_tensor(e), torch.as_tensor(th), torch.as_tensor(table))
    config = SolverConfig(**STEP_CONFIG)
    arrays = dict(rho=rho, det_e=e, det_theta=th, det_table=table)
    for name, curved in (("flat", False), ("curved", True)):
        geo = ConeGeometry(40.0, 60.0, 12, 16, 1.2, 1.2, use_curved_detector=curved)
        solver = ScatterSolver(library, config, geo, SiddonProjectors(backend="torch"), det, no_grid(),
                               device="cpu", dtype=F64)
        fields = solver.material_fields(rho, grid)
        angle = 0.6
        state = CitrusState()
        for step in (1, 2):
            scatter, primary, state = citrus_view_step(solver, state, fields, angle, primary=True)
            arrays[f"{name}_step{step}_scatter"] = scatter
            arrays[f"{name}_step{step}_collided"] = state.collided_moments
            arrays[f"{name}_step{step}_change"] = np.asarray(state.history[-1])
        arrays[f"{name}_primary"] = primary
        result = solver.solve_view(rho, grid, angle, signal_only=True)
        arrays[f"{name}_solve_scatter"] = result.scatter_signal
        arrays[f"{name}_solve_primary"] = result.primary["signal"]
        arrays[f"{name}_solve_iterations"] = np.asarray(result.source_iteration_result.num_iterations)
        arrays[f"{name}_solve_history"] = np.asarray(result.source_iteration_result.history)
        arrays[f"{name}_mu_t_coarse"] = fields.mu_t_coarse
        arrays[f"{name}_rho_coarse"] = fields.rho_coarse
    save("citrus_step_small", **arrays)




@case
def density_model():
    """The reference's interpolating density model (float32 maps of a seeded attenuation volume from below 0 to above
    the densest material) for a three-material library, with its effective energy, mass attenuations and order."""
    sys.path.insert(0, str(HERE.parent.parent))
    from citrus_gb300.cross_sections import AVOGADRO, BONE, WATER, MaterialModel, spectral_library
    from citrus_gb300.workloads import bremsstrahlung_spectrum
    from citrus.utilities import (attenuation_to_densities, attenuation_to_density, effective_energy,
                                  mass_attenuation_at, material_order)
    soft = MaterialModel("soft_tissue", AVOGADRO * 0.549, 0.0185, 0.0115, 1.04)
    lib = spectral_library(np.linspace(120.0, 40.0, 4), bremsstrahlung_spectrum(seed=3), [WATER, BONE, soft], 1,
                           num_eta=21, fine_per_group=4)
    ref = reference_library(lib)
    g = torch.Generator().manual_seed(11)
    X = (torch.rand(6, 7, 5, generator=g) * 1.4 - 0.2).to(torch.float32)
    e = effective_energy(ref)
    rho = attenuation_to_densities(ref, X)
    single = torch.stack([attenuation_to_density(ref, X, m) for m in range(3)])
    X50 = X * 0.7
    rho50 = attenuation_to_densities(ref, X50, 50.0)
    save("density_model", X=X, rho=rho, single=single, X50=X50, rho50=rho50, energy=np.array(e),
         mass=mass_attenuation_at(ref, e), order=np.array(material_order(ref)),
         lib_fine_energy=lib.fine_energy, lib_fine_mu_t=lib.fine_mu_t, lib_fine_weight=lib.fine_weight,
         lib_nominal=lib.nominal_density)


def _block_means(a: np.ndarray, b: int) -> np.ndarray:
    """Means over b x b x b blocks of the last three axes."""
    *lead, R, C, S = a.shape
    return a.reshape(*lead, R // b, b, C // b, b, S // b, b).mean(axis=(-5, -3, -1))


@case
def config1_view():
    """The reference's CITRUS scatter step of the single-view workload (32^3 cells of 0.5 cm, one 60 keV group, P3,
    4 x 12 sweep directions, cone 16 x 32, flat 64 x 64 panel of 0.4 cm pixels at 150 cm, ideal counting detector):
    ``citrus_view_step(primary=True, sweeps=1)`` from a cold start and a second step, float64 CPU. Stored: the
    inputs' densities, both steps' scatter images and changes, the primary, the scalar-flux LD moments of the
    collided accumulator element-wise (float32) and the cell means of all 16 moments over 2^3-cell blocks."""
    sys.path.insert(0, str(HERE.parent.parent))
    from citrus_gb300.workloads import single_view
    from citrus.citrus import CitrusState, citrus_view_step
    from citrus.scatter_solver.config import SolverConfig
    from citrus.scatter_solver.detector import ideal_counting_response, no_grid
    from citrus.scatter_solver.geometry import ConeGeometry, Grid
    from citrus.scatter_solver.ray_tracing import SiddonProjectors
    from citrus.scatter_solver.scatter_solver import ScatterSolver

    w = single_view()
    library = reference_library(w.library)
    g = w.geometry
    geo = ConeGeometry(g.source_iso_dist, g.source_detector_dist, g.num_det_rows, g.num_det_channels,
                       g.delta_det_row, g.delta_det_channel)
    grid = Grid(w.grid.shape, w.grid.delta_voxel)
    config = SolverConfig(num_groups=1, legendre_order=w.legendre_order, num_polar=w.num_polar,
                          num_azimuthal=w.num_azimuthal, transport_cell_cm=w.transport_cell_cm,
                          quadrature_point_spacing_cm=0.5, cone_num_polar=w.cone_num_polar,
                          cone_num_azimuthal=w.cone_num_azimuthal, direction_chunk=6)
    solver = ScatterSolver(library, config, geo, SiddonProjectors(backend="torch"), ideal_counting_response(),
                           no_grid(), device="cpu", dtype=F64)
    rho = torch.as_tensor(w.rho, dtype=F64)
    fields = solver.material_fields(rho, grid)
    state = CitrusState()
    arrays = dict(rho=rho)
    for step in (1, 2):
        scatter, primary, state = citrus_view_step(solver, state, fields, 0.0, primary=True)
        phi = state.collided_moments.numpy()                                   # [G, N_sh, 4, R, C, S]
        arrays[f"step{step}_scatter"] = scatter
        arrays[f"step{step}_change"] = np.asarray(state.history[-1])
        arrays[f"step{step}_scalar"] = phi[:, 0].astype(np.float32)
        arrays[f"step{step}_means_b2"] = _block_means(phi[:, :, 0], 2).astype(np.float32)
        arrays[f"step{step}_norms"] = np.sqrt((phi ** 2).sum(axis=(0, 2, 3, 4, 5)))
    arrays["primary"] = primary
    save("config1_view", **arrays)


@case
def pre_quadrature_synthetic():
    """The reference's regression anchor of ``solve_view`` (its ``tests/data/pre_quadrature_reference.json``, cases
    ``synthetic_cpu`` and ``synthetic_cuda``, checked by its ``tests/test_quadrature_grid.py``) with the inputs that
    produce it: the seven-material synthetic library (G = 4, L = 5), the WLAB phantom on the 2 cm grid (10 x 16 x 20),
    the CsI scintillator response, 4 cm cells (q = 2), the fine uncollided trace, view 0.4 rad. Also stored: the full
    float64 images of the same solve run now by the reference."""
    import json
    from citrus.scatter_solver.config import SolverConfig
    from citrus.scatter_solver.cross_sections import synthetic_library
    from citrus.scatter_solver.detector import csi_response, no_grid
    from citrus.scatter_solver.geometry import Grid
    from citrus.scatter_solver.ray_tracing import SiddonProjectors
    from citrus.scatter_solver.scatter_solver import ScatterSolver
    from citrus.utilities import wlab_geometry, wlab_phantom

    grid = Grid((10, 16, 20), 2.0)
    config = SolverConfig(num_groups=4, legendre_order=3, num_polar=4, num_azimuthal=8, cone_num_polar=8,
                          cone_num_azimuthal=16, transport_cell_cm=4.0, quadrature_point_spacing_cm=2.0,
                          source_iteration_tolerance=1e-4, max_source_iterations=40, direction_chunk=8,
                          uncollided_trace_grid="fine")
    library = synthetic_library(config.num_groups, 5, num_materials=7)
    det = csi_response()
    geo = wlab_geometry()
    solver = ScatterSolver(library, config, geo, SiddonProjectors(backend="torch"), det, no_grid(), device="cpu",
                           dtype=F64)
    rho = wlab_phantom(grid, dtype=F64)
    r = solver.solve_view(rho, grid, 0.4)
    cases = json.loads(Path(REFERENCE, "tests", "data", "pre_quadrature_reference.json").read_text())["cases"]
    arrays = dict(rho=rho, det_e=det.energy_kev, det_theta=det.theta_rad, det_table=det.response,
                  geometry=np.array([geo.source_iso_dist, geo.source_detector_dist, geo.num_det_rows,
                                     geo.num_det_channels, geo.delta_det_row, geo.delta_det_channel]),
                  scatter_signal=r.scatter_signal, primary_signal=r.primary["signal"],
                  si_iterations=np.asarray(r.source_iteration_result.num_iterations),
                  si_history=np.asarray(r.source_iteration_result.history))
    for k in ("group_edges", "group_energy", "spectrum_fraction", "mu_t", "mu_pe", "mu_s_l", "eta_grid", "mu_s_eta",
              "fine_energy", "fine_mu_t", "fine_weight", "fine_group", "nominal_density"):
        arrays[f"lib_{k}"] = getattr(library, k)
    arrays["lib_materials"] = np.array(library.materials)
    for name in ("synthetic_cpu", "synthetic_cuda"):
        c = cases[name]
        arrays[f"{name}_image_shape"] = np.array(c["image_shape"])
        for k in ("scatter_signal_blocks", "primary_signal_blocks", "scatter_signal_sum", "primary_signal_sum",
                  "si_iterations", "si_final_change"):
            arrays[f"{name}_{k}"] = np.asarray(c[k], dtype=np.float64)
    save("pre_quadrature_synthetic", **arrays)


@case
def citrus_step_sweeps():
    """Two CITRUS steps of one view with ``sweeps=2`` (``accumulator_update_operator``: the second sweep applies K to
    the last change of the accumulator) from a cold start, on the problem of ``citrus_step_small`` (flat panel),
    float64 CPU."""
    from citrus.citrus import CitrusState, citrus_view_step
    from citrus.scatter_solver.config import SolverConfig
    from citrus.scatter_solver.detector import DetectorResponse, no_grid
    from citrus.scatter_solver.geometry import ConeGeometry, Grid
    from citrus.scatter_solver.ray_tracing import SiddonProjectors
    from citrus.scatter_solver.scatter_solver import ScatterSolver

    g = torch.Generator().manual_seed(31)
    library = reference_library(small_spectral_library())
    grid = Grid((8, 8, 6), 1.0)
    rho = torch.zeros(2, *grid.shape, dtype=F64)
    rho[0] = 0.9 + 0.2 * torch.rand(*grid.shape, generator=g, dtype=F64)
    rho[1, 2:5, 3:6, 1:4] = 1.85
    rho[0, 2:5, 3:6, 1:4] = 0.0
    e, th, table = scintillator_table()
    det = DetectorResponse(torch.as_tensor(e), torch.as_tensor(th), torch.as_tensor(table))
    geo = ConeGeometry(40.0, 60.0, 12, 16, 1.2, 1.2)
    solver = ScatterSolver(library, SolverConfig(**STEP_CONFIG), geo, SiddonProjectors(backend="torch"), det,
                           no_grid(), device="cpu", dtype=F64)
    fields = solver.material_fields(rho, grid)
    state = CitrusState()
    arrays = dict(rho=rho)
    for step in (1, 2):
        scatter, _, state = citrus_view_step(solver, state, fields, 0.6, primary=False, sweeps=2)
        arrays[f"step{step}_scatter"] = scatter
        arrays[f"step{step}_collided"] = state.collided_moments
        arrays[f"step{step}_change"] = np.asarray(state.history[-1])
    save("citrus_step_sweeps", **arrays)


@case
def state_store_codec():
    """The reference's per-view accumulator store (``citrus.StateStore``, host location, float32 arithmetic) on a
    seeded accumulator [G=3, N=16, 4, 4, 5, 6] with moments of decreasing size, one (group, moment) plane holding a
    NaN cell and one all zero: the decoded accumulator and the stored float16 values."""
    from citrus.citrus import StateStore
    g = torch.Generator().manual_seed(8)
    shape = (3, 16, 4, 4, 5, 6)
    phi = (1e-6 * torch.randn(shape, generator=g, dtype=torch.float64)
           * torch.logspace(0, -3, 16, dtype=torch.float64)[None, :, None, None, None, None]).float()
    phi[1, 2, 0, 1, 2, 3] = float("nan")
    phi[2, 5] = 0.0
    store = StateStore(1, shape, "cpu", location="cpu")
    store.put(0, phi)
    save("state_store_codec", phi=phi, decoded=store.get(0), stored=store._data[0].float(), scale=store._scale[0])


def _filter_mass_attenuation(e):
    """A synthetic aluminium-like total mass attenuation in cm^2/g (the photon data is not part of the fixtures)."""
    e = np.asarray(e, dtype=np.float64)
    return 0.16 + 4.0 * (e / 30.0) ** -2.8


@case
def grid_and_source():
    """The reference's anti-scatter grid and source model on the scatter-step path: the focused 1-D grid table (its
    geometric septum-shadow model with its own lead attenuation), grid angles and transmissions for flat and curved
    panels (septa along the channels and the rows, focused, unfocused and at a shorter focal distance, crossed), the
    collapsed-cone image behind the grid for the seven panel/septa routes of its own scatter-image test, and the
    uncollided fluence and primary with an emission profile, an off-focal table and a beam filter. The filter's mass
    attenuation is the synthetic ``_filter_mass_attenuation`` (patched into the reference's fine-energy lookup, since
    the photon data is not read here)."""
    from dataclasses import replace
    import citrus.scatter_solver.source as ref_source
    from citrus.scatter_solver.angular_quadrature import scatter_source_moments
    from citrus.scatter_solver.cross_sections import Material, mu_t_volume, transfer_moments_volume
    from citrus.scatter_solver.detector import (DetectorResponse, focused_1d_grid, grid_angles,
                                                lead_mass_attenuation)
    from citrus.scatter_solver.geometry import ConeGeometry, Grid
    from citrus.scatter_solver.ray_tracing import SiddonProjectors
    from citrus.scatter_solver.scatter_image import (combined_scatter_image, make_direction_context,
                                                     panel_direction_set, primary_image)
    from citrus.scatter_solver.source import SourceModel, bowtie_emission_profile
    from citrus.scatter_solver.uncollided import DENSE, uncollided_fluence

    g = torch.Generator().manual_seed(31)
    energies = np.arange(10.0, 150.1, 5.0)
    grid = focused_1d_grid(energies=energies)
    arrays = dict(grid_energy=grid.energy_kev, grid_theta1=grid.theta1_rad, grid_theta2=grid.theta2_rad,
                  grid_table=grid.transmission, grid_focal=np.array(grid.focal_distance_cm),
                  lead_mu=lead_mass_attenuation(energies))
    # grid angles and transmissions
    omegas = torch.nn.functional.normalize(torch.randn(6, 3, generator=g, dtype=F64), dim=-1)
    arrays["angles_omega"] = omegas
    e_query = torch.tensor([18.0, 47.5, 93.2, 140.0], dtype=F64)
    arrays["angles_energy"] = e_query
    for curved in (False, True):
        geo = ConeGeometry(100.0, 150.0, 5, 7, 4.0, 4.0, det_row_offset=1.0, use_curved_detector=curved)
        pix = geo.pixel_centers(0.9, dtype=F64)
        pre = "curved" if curved else "flat"
        # the primary directions turned away from the normal in both panel axes, so every angle is nonzero
        for septa in ("channels", "rows"):
            for focal, fname in ((None, "default"), (math.inf, "unfocused"), (120.0, "f120")):
                t1, t2 = grid_angles(omegas, pix, geo, 0.9, focal, septa)
                arrays[f"angles_{pre}_{septa}_{fname}_theta1"] = t1
                arrays[f"angles_{pre}_{septa}_{fname}_theta2"] = t2
            sep = replace(grid, septa_along=septa)
            arrays[f"transmission_{pre}_{septa}"] = sep.transmission_at(e_query, omegas, pix, geo, 0.9)
        crossed = replace(grid, crossed=replace(grid, septa_along="rows"))
        arrays[f"transmission_{pre}_crossed"] = crossed.transmission_at(e_query, omegas, pix, geo, 0.9)
    # the image behind the grid (the scatter-image test's routes, on the small image setup)
    library = reference_library(small_spectral_library())
    L = 2
    grid_q = Grid((6, 6, 4), 2.0)
    q = 2
    grid_c = grid_q.coarsen(q)
    rho = torch.rand(2, *grid_q.shape, generator=g, dtype=F64) * torch.tensor([1.0, 0.5], dtype=F64)[:, None, None,
                                                                                                         None]
    rho_c = rho.reshape(2, 3, 2, 3, 2, 2, 2).mean(dim=(2, 4, 6))
    mu_c = mu_t_volume(library, rho_c)
    phi_coll = torch.rand(library.num_groups, (L + 1) ** 2, *grid_c.shape, generator=g, dtype=F64) * 1e-4
    T = scatter_source_moments(transfer_moments_volume(library, rho_c)[:, :, :L + 1], phi_coll)
    e, th, table = scintillator_table()
    det = DetectorResponse(torch.as_tensor(e), torch.as_tensor(th), torch.as_tensor(table))
    arrays.update(image_rho=rho, image_T=T)
    along_rows = replace(grid, septa_along="rows")
    crossed = replace(grid, crossed=along_rows)
    routes = {"flat_rows": (False, grid), "flat_channels": (False, along_rows), "flat_crossed": (False, crossed),
              "curved_rows": (True, along_rows), "curved_pixel": (True, grid), "curved_crossed": (True, crossed)}
    proj = SiddonProjectors(backend="torch")
    for name, (curved, grid_response) in routes.items():
        geo = ConeGeometry(50.0, 80.0, 10, 14, 1.5, 1.5, det_channel_offset=0.4, use_curved_detector=curved)
        angle = 0.8
        phi = uncollided_fluence(library, rho, grid_q, geo, angle, SourceModel(), proj)
        cone = panel_direction_set(geo, angle, (3, 6), max_polar_angle=grid_c, dtype=F64)
        ctx = make_direction_context(cone, geo, angle, det, grid_response, library, "cpu", F64, chunk=5)
        full = combined_scatter_image(library, rho, phi, grid_q, q, T, L, geo, angle, cone, mu_c, proj, det,
                                      grid_response, ctx, pairs=DENSE, grid_coarse=grid_c)
        sig = combined_scatter_image(library, rho, phi, grid_q, q, T, L, geo, angle, cone, mu_c, proj, det,
                                     grid_response, ctx, pairs=DENSE, grid_coarse=grid_c,
                                     signal_only=True)["signal"]
        prim = primary_image(library, rho, grid_q, geo, angle, SourceModel(), proj, det, grid_response)
        arrays.update({f"image_{name}_phi": phi, f"image_{name}_signal_pg": full["signal_per_group"],
                       f"image_{name}_signal": full["signal"], f"image_{name}_signal_only": sig,
                       f"image_{name}_fluence": full["fluence"], f"image_{name}_primary": prim["signal"]})
        if name == "flat_rows":
            arrays.update(image_cone_omega=cone.omega, image_cone_weight=cone.weight, image_cone_width=cone.cell_width)
    # the responses averaged over each group's fine energies (SolverConfig.group_averaged_responses)
    from citrus.scatter_solver.detector import group_averaged_responses
    avg_det, avg_grid = group_averaged_responses(det, crossed, library)
    arrays.update(avg_det_energy=avg_det.energy_kev, avg_det_table=avg_det.response,
                  avg_grid_energy=avg_grid.energy_kev, avg_grid_table=avg_grid.transmission,
                  avg_crossed_energy=avg_grid.crossed.energy_kev, avg_crossed_table=avg_grid.crossed.transmission)
    # the source model: emission profile, off-focal table and beam filter
    filter_material = Material("filter", 2.7, "Al")
    ref_source._fine_attenuation = lambda energies, key, definition: torch.as_tensor(
        _filter_mass_attenuation(energies.detach().cpu().numpy()), dtype=key[4]).to(key[3])
    arrays["filter_mu"] = _filter_mass_attenuation(library.fine_energy)
    for curved in (False, True):
        pre = "curved" if curved else "flat"
        geo = ConeGeometry(50.0, 80.0, 10, 14, 1.5, 1.5, det_channel_offset=0.4, use_curved_detector=curved)
        profile = bowtie_emission_profile(geo, 0.3)
        profile = profile * (1.0 + 0.05 * torch.arange(10, dtype=F64))[:, None]
        thickness = 0.1 + 0.02 * torch.arange(14, dtype=F64) ** 1.5
        source = SourceModel(emission_profile=profile, field_margin_channels_cm=0.5, field_margin_rows_cm=0.25,
                             off_focal_distance_cm=[0.0, 1.0, 3.0], off_focal_fraction=[0.3, 0.1, 0.02],
                             filter_material=filter_material, filter_thickness_cm=thickness)
        arrays.update({f"source_{pre}_profile": profile, f"source_{pre}_thickness": thickness})
        big = Grid((8, 10, 6), 3.0)  # wider than the field, so points see the margins and the off-focal table
        rho_b = torch.rand(2, *big.shape, generator=g, dtype=F64) * torch.tensor([1.0, 0.4], dtype=F64)[:, None,
                                                                                                          None, None]
        arrays[f"source_{pre}_rho"] = rho_b
        arrays[f"source_{pre}_phi"] = uncollided_fluence(library, rho_b, big, geo, 0.8, source, proj)
        d = big.center_coordinates(dtype=F64).reshape(-1, 3) - torch.tensor(geo.source_position(0.8), dtype=F64)
        arrays[f"source_{pre}_b"] = source.angular_weight(d, geo, 0.8)
        arrays[f"source_{pre}_filter_path"] = source.filter_path(d, geo, 0.8)
        prim = primary_image(library, rho_b, big, geo, 0.8, source, proj, det, grid)
        arrays[f"source_{pre}_primary"] = prim["signal"]
        arrays[f"source_{pre}_primary_fluence"] = prim["fluence"]
        # 2 x 2 sub-rays per pixel: the fine-energy transmission (filter included) averaged over the sub-pixels
        prim2 = primary_image(library, rho_b, big, geo, 0.8, source, proj, det, grid, samples_per_pixel_axis=2)
        arrays[f"source_{pre}_primary_n2"] = prim2["signal"]
    save("grid_and_source", **arrays)


@case
def library_file():
    """A library written by the reference's own ``MultigroupLibrary.save`` (``torch.save`` of a dict of every field),
    the two-material synthetic library with G = 3, L = 2, 21 eta nodes: the on-disk format ``load`` reads."""
    from citrus.scatter_solver.cross_sections import synthetic_library
    synthetic_library(3, 2, num_eta=21, num_fine_per_group=2).save(str(HERE / "reference_library.pt"))
    print(f"reference_library.pt: {(HERE / 'reference_library.pt').stat().st_size / 1024:.1f} KiB")


if __name__ == "__main__":
    names = sys.argv[1:] or list(CASES)
    for n in names:
        CASES[n]()
