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


def test_graphed_outer_iteration_seeded_with_accumulators(cuda_device):
    """GraphedOuterIteration.seed starts every view from given accumulators (as the learned proposal does): seeded
    with the accumulators of an eager cold step, its next steps (the first eager, the rest replayed from the graph)
    equal the eager batched steps that follow that cold step."""
    g, solver = _solver("flat", cuda_device)
    grid = Grid((8, 8, 6), 1.0)
    rho = torch.as_tensor(g["rho"], dtype=torch.float32, device=cuda_device)
    angles = [0.3, 1.7, 4.0]
    fields = solver.material_fields(rho, grid)
    _, _, eager = batched_view_steps(solver, [CitrusState() for _ in angles], fields, angles, batch=2)
    graphed = GraphedOuterIteration(solver, grid, angles, batch=2)
    graphed.seed(rho, [s.collided_moments.clone() for s in eager])
    for step in range(3):
        signals, states = graphed.step(rho)
        ref, _, eager = batched_view_steps(solver, eager, fields, angles, batch=2)
        for v in range(len(angles)):
            assert rel_err(signals[v], ref[v]) < 1e-6, (step, v)
            assert rel_err(states[v].collided_moments, eager[v].collided_moments) < 1e-6, (step, v)
    assert graphed.replays == 2
    with pytest.raises(ValueError):
        graphed.seed(rho, [eager[0].collided_moments])


@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_direction_chunks_of_the_batched_step(cuda_device, monkeypatch, precision):
    """A store budget that forces direction chunks (1 and 3 directions per octant of the 4 x 8 set's 4) gives the
    unchunked batched steps' signals and accumulators to rounding (the moment product accumulates over the chunks;
    in bf16x3 each chunk's product carries the split's own ~1e-5), cold and warm."""
    import citrus_gb300.batched as batched
    g, solver = _solver("curved", cuda_device, moment_precision=precision)
    grid = Grid((8, 8, 6), 1.0)
    fields = solver.material_fields(torch.as_tensor(g["rho"], dtype=torch.float32, device=cuda_device), grid)
    angles = [0.3, 1.7, 4.0]
    ctx = solver.sweep_context(fields.grid_coarse)
    per_direction = 8 * ctx.num_cells * 4 * solver.num_groups * 4
    runs = []
    for budget in (batched.SWEEP_STORE_BUDGET_BYTES, per_direction, 3 * per_direction):
        monkeypatch.setattr(batched, "SWEEP_STORE_BUDGET_BYTES", budget)
        states = [CitrusState() for _ in angles]
        out = []
        for _ in range(2):
            signals, _, states = batched_view_steps(solver, states, fields, angles, batch=2)
            out.append((signals.clone(), [s.collided_moments.clone() for s in states]))
        runs.append(out)
    assert batched.direction_chunk(ctx.num_cells, solver.num_groups, ctx.directions_per_octant,
                                   per_direction) == 1
    tol = 1e-6 if precision == "fp32" else 2e-5   # bf16x3: the hi/lo split's ~1e-5, chunk partials added in float32
    for other in runs[1:]:
        for (sa, aa), (sb, ab) in zip(runs[0], other):
            assert rel_err(sb, sa) < tol
            for x, y in zip(ab, aa):
                assert rel_err(x, y) < tol
