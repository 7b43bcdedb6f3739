"""The per-view CITRUS step and the converged view solve on sm_103a against the reference's own results
(``citrus_view_step`` twice, with the primary, and ``solve_view``), flat and curved panels."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import golden, rel_err
from citrus_gb300.citrus_step import CitrusState, citrus_view_step
from citrus_gb300.geometry import ConeGeometry, Grid
from citrus_gb300.responses import DetectorResponse, no_grid
from citrus_gb300.scatter_solver import ScatterSolver, SolverConfig
from test_oracle_golden import _uncollided_setup

pytestmark = pytest.mark.gpu
STEP_CONFIG = dict(num_groups=3, legendre_order=2, num_polar=4, num_azimuthal=8, transport_cell_cm=2.0,
                   quadrature_point_spacing_cm=1.0, cone_num_polar=3, cone_num_azimuthal=6, direction_chunk=4,
                   source_iteration_tolerance=1e-4, max_source_iterations=40)


def _solver(name, device, **overrides):
    g = golden("citrus_step_small")
    library, _, _ = _uncollided_setup()
    det = DetectorResponse(g["det_e"], g["det_theta"], g["det_table"])
    geo = ConeGeometry(40.0, 60.0, 12, 16, 1.2, 1.2, use_curved_detector=name == "curved")
    return g, ScatterSolver(library, SolverConfig(**dict(STEP_CONFIG, **overrides)), geo, detector=det,
                            grid_response=no_grid(), device=device)


@pytest.mark.parametrize("name", ["flat", "curved"])
def test_citrus_view_steps_match_reference(cuda_device, name):
    g, solver = _solver(name, cuda_device)
    grid = Grid((8, 8, 6), 1.0)
    rho = torch.as_tensor(g["rho"], dtype=torch.float32, device=cuda_device)
    fields = solver.material_fields(rho, grid)
    assert rel_err(fields.rho_coarse, g[f"{name}_rho_coarse"]) < 1e-6
    assert rel_err(fields.mu_t_coarse, g[f"{name}_mu_t_coarse"]) < 1e-6
    state = CitrusState()
    for step in (1, 2):
        scatter, primary, state = citrus_view_step(solver, state, fields, 0.6, primary=True)
        assert rel_err(state.collided_moments, g[f"{name}_step{step}_collided"]) < 1e-4
        assert rel_err(scatter, g[f"{name}_step{step}_scatter"]) < 1e-4
        assert abs(state.history[-1] - float(g[f"{name}_step{step}_change"])) < 1e-4
    assert rel_err(primary, g[f"{name}_primary"]) < 2e-6


@pytest.mark.parametrize("name", ["flat", "curved"])
def test_solve_view_matches_reference(cuda_device, name):
    g, solver = _solver(name, cuda_device)
    grid = Grid((8, 8, 6), 1.0)
    rho = torch.as_tensor(g["rho"], dtype=torch.float32, device=cuda_device)
    result = solver.solve_view(rho, grid, 0.6, signal_only=True)
    assert result.source_iteration_result.num_iterations == int(g[f"{name}_solve_iterations"])
    np.testing.assert_allclose(result.source_iteration_result.history, g[f"{name}_solve_history"], rtol=1e-3,
                               atol=1e-6)
    assert rel_err(result.scatter_signal, g[f"{name}_solve_scatter"]) < 1e-4
    assert rel_err(result.primary["signal"], g[f"{name}_solve_primary"]) < 2e-6


@pytest.mark.parametrize("name", ["flat", "curved"])
def test_bf16x3_moment_products_keep_the_step_and_spr_within_bounds(cuda_device, name):
    """The mixed-precision step (tensor-core bfloat16 hi/lo spherical-harmonic products) against the reference's
    float64 step: collided moments and scatter signal within 2e-4, the scatter-to-primary ratio within 0.5 %."""
    g, solver = _solver(name, cuda_device, moment_precision="bf16x3")
    grid = Grid((8, 8, 6), 1.0)
    rho = torch.as_tensor(g["rho"], dtype=torch.float32, device=cuda_device)
    fields = solver.material_fields(rho, grid)
    state = CitrusState()
    for step in (1, 2):
        scatter, primary, state = citrus_view_step(solver, state, fields, 0.6, primary=True)
        assert rel_err(state.collided_moments, g[f"{name}_step{step}_collided"]) < 2e-4
        assert rel_err(scatter, g[f"{name}_step{step}_scatter"]) < 2e-4
    p = primary.detach().cpu().double().numpy()
    mask = p > 1e-3 * p.max()
    spr = scatter.detach().cpu().double().numpy()[mask] / p[mask]
    spr_ref = g[f"{name}_step2_scatter"][mask] / g[f"{name}_primary"][mask]
    assert np.abs(spr / spr_ref - 1.0).max() < 5e-3


@pytest.mark.parametrize("name", ["flat", "curved"])
def test_primary_signals_of_all_views(cuda_device, name):
    from citrus_gb300.citrus_step import primary_signals
    g, solver = _solver(name, cuda_device)
    grid = Grid((8, 8, 6), 1.0)
    rho = torch.as_tensor(g["rho"], dtype=torch.float32, device=cuda_device)
    fields = solver.material_fields(rho, grid)
    angles = [0.6, 1.3, 2.9]
    signals = primary_signals(solver, fields, angles)
    assert rel_err(signals[0], g[f"{name}_primary"]) < 2e-6
    for v, a in enumerate(angles):
        assert torch.equal(signals[v], solver.primary(fields, a)["signal"])
    planar = primary_signals(solver, fields, angles, quantity="planar_fluence")
    assert torch.allclose(planar[1], solver.primary(fields, 1.3)["planar_fluence"].sum(0))
    with pytest.raises(ValueError):
        primary_signals(solver, fields, angles, quantity="counts")


def test_citrus_view_steps_with_two_sweeps_match_reference(cuda_device):
    """``sweeps=2`` (the second sweep applies K to the accumulator's last change, reference ``citrus.py:192-247``):
    two steps from a cold start against the reference's float64 run."""
    ref = golden("citrus_step_sweeps")
    _, solver = _solver("flat", cuda_device)
    grid = Grid((8, 8, 6), 1.0)
    rho = torch.as_tensor(ref["rho"], dtype=torch.float32, device=cuda_device)
    fields = solver.material_fields(rho, grid)
    state = CitrusState()
    for step in (1, 2):
        scatter, primary, state = citrus_view_step(solver, state, fields, 0.6, primary=False, sweeps=2)
        assert primary is None
        assert rel_err(state.collided_moments, ref[f"step{step}_collided"]) < 1e-4
        assert rel_err(scatter, ref[f"step{step}_scatter"]) < 1e-4
        assert abs(state.history[-1] - float(ref[f"step{step}_change"])) < 1e-4
    with pytest.raises(ValueError):
        citrus_view_step(solver, state, fields, 0.6, sweeps=0)
