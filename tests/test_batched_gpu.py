"""Batched accumulator sweeps (several views per persistent sweep launch) equal the per-view CITRUS steps."""

from __future__ import annotations

import pytest
import torch

from conftest import rel_err
from citrus_gb300.batched import GraphedOuterIteration, batched_view_steps
from citrus_gb300.citrus_step import CitrusState, citrus_view_step
from citrus_gb300.geometry import Grid
from test_citrus_step_gpu import _solver

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["flat", "curved"])
def test_batched_steps_equal_per_view_steps(cuda_device, name):
    g, solver = _solver(name, cuda_device)
    grid = Grid((8, 8, 6), 1.0)
    fields = solver.material_fields(torch.as_tensor(g["rho"], dtype=torch.float32, device=cuda_device), grid)
    angles = [0.3, 1.7, 4.0]
    single = [CitrusState() for _ in angles]
    batched = [CitrusState() for _ in angles]
    for _ in range(2):
        ref = []
        for v, a in enumerate(angles):
            s, _, single[v] = citrus_view_step(solver, single[v], fields, a, primary=False)
            ref.append(s)
        signals, _, batched = batched_view_steps(solver, batched, fields, angles, batch=2)
        for v in range(len(angles)):
            assert rel_err(signals[v], ref[v]) < 1e-6
            assert rel_err(batched[v].collided_moments, single[v].collided_moments) < 1e-6
            assert abs(batched[v].history[-1] - single[v].history[-1]) < 1e-6


@pytest.mark.parametrize("name", ["flat", "curved"])
def test_one_point_per_cell_batched_steps_equal_per_view_steps(cuda_device, name):
    """One point per transport cell: the warm batched steps form the sweep source in one pass from the first-collision
    means (citrus_first_collision_means, citrus_source_expansion_first); the per-view steps write the moment
    quadruples and accumulate the expansion over them. Same states and signals."""
    g, solver = _solver(name, cuda_device, quadrature_point_spacing_cm=2.0)
    grid = Grid((8, 8, 6), 1.0)
    fields = solver.material_fields(torch.as_tensor(g["rho"], dtype=torch.float32, device=cuda_device), grid)
    assert fields.q == 1
    angles = [0.3, 1.7, 4.0]
    single = [CitrusState() for _ in angles]
    batched = [CitrusState() for _ in angles]
    for _ in range(3):
        ref = []
        for v, a in enumerate(angles):
            s, _, single[v] = citrus_view_step(solver, single[v], fields, a, primary=False)
            ref.append(s)
        signals, _, batched = batched_view_steps(solver, batched, fields, angles, batch=2)
        for v in range(len(angles)):
            assert rel_err(signals[v], ref[v]) < 1e-6
            assert rel_err(batched[v].collided_moments, single[v].collided_moments) < 1e-6
            assert abs(batched[v].history[-1] - single[v].history[-1]) < 1e-6


def test_first_collision_means_are_the_moments_first_components(cuda_device):
    """With one point per cell the first-collision LD moments are (mean, 0, 0, 0); citrus_first_collision_means gives
    the means alone, read from the same cached source values."""
    g, solver = _solver("curved", cuda_device, quadrature_point_spacing_cm=2.0)
    fields = solver.material_fields(torch.as_tensor(g["rho"], dtype=torch.float32, device=cuda_device),
                                    Grid((8, 8, 6), 1.0))
    assert fields.q == 1
    ctx = solver.sweep_context(fields.grid_coarse)
    uc = solver.uncollided_fluence(fields, 0.9)
    first = solver.first_collision_moment_source(fields, 0.9, uc, ctx)
    assert first.means is not None
    index = torch.arange(ctx.omega.shape[0], device=cuda_device)
    quads = first(index)
    means = first.means(index)
    assert tuple(means.shape) == tuple(quads.shape[:1]) + (ctx.num_cells, solver.num_groups)
    assert float(quads[..., 1:].abs().max()) == 0.0
    assert rel_err(means, quads[..., 0].reshape(means.shape)) < 1e-6


@pytest.mark.parametrize("name", ["flat", "curved"])
def test_graphed_outer_iterations_equal_batched_steps(cuda_device, name):
    """The outer iteration recorded into a CUDA graph (accumulators updated in place) gives the eager batched steps'
    results on every replay, including after the densities change."""
    g, solver = _solver(name, cuda_device)
    grid = Grid((8, 8, 6), 1.0)
    rho = torch.as_tensor(g["rho"], dtype=torch.float32, device=cuda_device)
    angles = [0.3, 1.7, 4.0]
    graphed = GraphedOuterIteration(solver, grid, angles, batch=2)
    eager = [CitrusState() for _ in angles]
    for step in range(5):
        rho_step = rho * (1.0 + 0.05 * step)          # the densities move between outer iterations
        signals, states = graphed.step(rho_step)
        fields = solver.material_fields(rho_step, grid)
        ref, _, eager = batched_view_steps(solver, eager, fields, angles, batch=2)
        for v in range(len(angles)):
            assert rel_err(signals[v], ref[v]) < 1e-6, (step, v)
            assert rel_err(states[v].collided_moments, eager[v].collided_moments) < 1e-6, (step, v)
            assert abs(states[v].history[-1] - eager[v].history[-1]) < 1e-6
    assert graphed.replays == 3
