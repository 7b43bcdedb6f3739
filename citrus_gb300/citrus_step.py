"""The per-view CITRUS scatter step and its operators (mirrors ``citrus/citrus.py:70-366``).

Every outer iteration of the CITRUS loop advances each view's collided-fluence accumulator ``Phi`` by one transport
sweep, ``Phi_new = phi^(1) + K Phi`` (the first-collision source and the scattering source of ``Phi`` transported
together: the first-collision moments are written into the sweep's store and the scattering source is added to them
by one accumulating small-K product), and projects the last-collided source onto the panel (signal only).
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np
import torch
from torch import Tensor

from .scatter_image import primary_from_path_lengths, primary_path_lengths
from .scatter_solver import MaterialFields, ScatterSolver
from .uncollided import present_materials


@dataclass
class CitrusState:
    """Caller-owned state of one view (reference ``citrus.py:70-87``)."""

    angle: Optional[float] = None
    collided_moments: Optional[Tensor] = None
    cone_quadrature: Optional[object] = None
    num_steps: int = 0
    history: list = field(default_factory=list)


def _fields(solver: ScatterSolver, rho, grid, fields: Optional[MaterialFields]) -> MaterialFields:
    return solver.material_fields(rho, grid) if fields is None else fields


def _check_count(name: str, count) -> None:
    if isinstance(count, bool) or not isinstance(count, (int, np.integer)) or count < 1:
        raise ValueError(f"{name} must be an integer >= 1, got {count!r}")


def uncollided_operator(solver: ScatterSolver, rho, grid, angle: float, fields: Optional[MaterialFields] = None):
    """G_1: the uncollided fluence at the quadrature points (reference ``citrus.py:106-124``)."""
    return solver.uncollided_fluence(_fields(solver, rho, grid, fields), angle)


def first_collision_operator(solver: ScatterSolver, rho, grid, angle: float, phi_uncollided: Tensor,
                             fields: Optional[MaterialFields] = None) -> Tensor:
    """phi^(1): one sweep of the first-collision source (reference ``citrus.py:127-147``)."""
    fields = _fields(solver, rho, grid, fields)
    return solver.transport_sweep(fields, solver.first_collision_moment_source(fields, angle, phi_uncollided))


def _check_accumulator(solver: ScatterSolver, fields: MaterialFields, collided: Tensor) -> None:
    ctx = solver.sweep_context(fields.grid_coarse)
    expected = (solver.num_groups, ctx.num_moments, 4, *fields.grid_coarse.shape)
    if tuple(collided.shape) != expected:
        raise ValueError(f"collided_moments must be {expected}, got {tuple(collided.shape)}")


def multiple_collision_operator(solver: ScatterSolver, rho, grid, angle: float, collided_moments: Optional[Tensor],
                                fields: Optional[MaterialFields] = None) -> Tensor:
    """K Phi: one sweep of the scattering source of Phi (reference ``citrus.py:166-194``)."""
    fields = _fields(solver, rho, grid, fields)
    ctx = solver.sweep_context(fields.grid_coarse)
    if collided_moments is None:
        return torch.zeros(solver.num_groups, ctx.num_moments, 4, *fields.grid_coarse.shape, device=solver.device)
    _check_accumulator(solver, fields, collided_moments)
    return solver.transport_sweep(fields, solver.scatter_moment_source(fields, collided_moments.to(solver.device),
                                                                       ctx))


def accumulator_update_operator(solver: ScatterSolver, rho, grid, angle: float, phi_uncollided: Tensor,
                                collided_moments: Optional[Tensor], fields: Optional[MaterialFields] = None, *,
                                sweeps: int = 1) -> Tensor:
    """Phi_new = phi^(1) + K Phi in one sweep; every further sweep adds K (Phi_new - Phi_old)
    (reference ``citrus.py:192-247``)."""
    _check_count("sweeps", sweeps)
    fields = _fields(solver, rho, grid, fields)
    ctx = solver.sweep_context(fields.grid_coarse)
    first = solver.first_collision_moment_source(fields, angle, phi_uncollided, ctx)
    if collided_moments is None:
        previous = None
        collided = solver.transport_sweep(fields, first)
    else:
        _check_accumulator(solver, fields, collided_moments)
        previous = collided_moments.to(solver.device)
        scatter = solver.scatter_moment_source(fields, previous, ctx)
        # one point per cell: the first-collision moments are (mean, 0, 0, 0), and their means go into the
        # expansion's single pass over the store instead of a write of the quadruples and an accumulating pass
        fused = getattr(first, "means", None) is not None and getattr(scatter, "with_means", None) is not None

        def summed_source(direction_index: Tensor, out: Optional[Tensor] = None) -> Tensor:
            if fused and out is not None:
                return scatter.with_means(direction_index, first.means(direction_index), out)
            src = first(direction_index, out)                              # cell-major, into the sweep's store
            return scatter(direction_index, out=src, accumulate=True)      # one accumulating small-K product

        summed_source.cell_major = True  # type: ignore[attr-defined]
        collided = solver.transport_sweep(fields, summed_source)
    for _ in range(int(sweeps) - 1):
        change = collided if previous is None else collided - previous
        source = solver.scatter_moment_source(fields, change, ctx)
        previous = collided
        collided = solver.transport_sweep(fields, source).add_(previous)
    return collided


def project_scatter(solver: ScatterSolver, rho, grid, angle: float, phi_uncollided: Tensor, collided_moments: Tensor,
                    fields: Optional[MaterialFields] = None, quadrature=None, signal_only: bool = False) -> dict:
    """Total scatter image of one view in one collapsed-cone pass (reference ``citrus.py:250-282``)."""
    fields = _fields(solver, rho, grid, fields)
    T = solver.multiple_collision_source_moments(fields, collided_moments.to(solver.device))
    return solver.scatter_image(fields, angle, phi_uncollided, T, quadrature, signal_only=signal_only)


def citrus_view_step(solver: ScatterSolver, state: CitrusState, fields: MaterialFields, angle: float, *,
                     primary: bool = True, sweeps: int = 1) -> tuple:
    """One CITRUS scatter step of one view (reference ``citrus.py:320-366``).

    Returns (scatter signal [Rd, Cd], primary signal [Rd, Cd] or None, new state).
    """
    if state.angle is not None and abs(float(state.angle) - float(angle)) > 1e-12:
        raise ValueError(f"state belongs to angle {state.angle}, got {angle}")
    grid = fields.grid_fine
    cone = state.cone_quadrature if state.cone_quadrature is not None else solver.cone_quadrature(grid, angle)
    phi_uc = uncollided_operator(solver, None, grid, angle, fields)
    new = accumulator_update_operator(solver, None, grid, angle, phi_uc, state.collided_moments, fields,
                                      sweeps=sweeps)
    scatter = project_scatter(solver, None, grid, angle, phi_uc, new, fields, cone, signal_only=True)["signal"]
    del phi_uc
    primary_signal = solver.primary(fields, angle)["signal"] if primary else None
    if state.collided_moments is None:
        norm = float(torch.linalg.vector_norm(new[:, 0, 0]))
        change = 1.0 if norm > 0 else 0.0
    else:
        prev = state.collided_moments[:, 0, 0].to(new)
        norm, diff = torch.stack([torch.linalg.vector_norm(new[:, 0, 0]),
                                  torch.linalg.vector_norm(new[:, 0, 0] - prev)]).tolist()
        change = diff / norm if norm > 0 else 0.0
    new_state = CitrusState(angle=float(angle), collided_moments=new, cone_quadrature=cone,
                            num_steps=state.num_steps + 1, history=state.history + [change])
    return scatter, primary_signal, new_state


def citrus_step(solver: ScatterSolver, state: CitrusState, rho, grid, angle: float,
                fields: Optional[MaterialFields] = None) -> tuple:
    """One CITRUS scatter step of one view from the densities (reference ``citrus.py:285-317``)."""
    return citrus_view_step(solver, state, _fields(solver, rho, grid, fields), angle)


def primary_signals(solver: ScatterSolver, fields: MaterialFields, angles, out: Optional[Tensor] = None,
                    quantity: str = "signal") -> Tensor:
    """Primary signal (or planar fluence summed over the groups) of every view, ``[V, Rd, Cd]`` (reference
    ``citrus.py:369-458``).

    The reference projects the material maps with the reconstruction's MBIRTORCH projector, which is not part of this
    package; here the path lengths are the Siddon line integrals from the focal spot to the pixel centres through the
    fine-grid density maps (``GB300Projectors.primary_project``), one launch per view over the materials present, and
    ``primary_from_path_lengths`` turns them into the primary of each view, as the reference does.
    """
    if quantity not in ("signal", "planar_fluence"):
        raise ValueError(f"quantity must be 'signal' or 'planar_fluence', got {quantity!r}")
    angle_array = np.asarray(angles, dtype=np.float64).reshape(-1)
    Rd, Cd = solver.geometry.image_shape
    if out is None:
        out = torch.empty((angle_array.size, Rd, Cd), device=solver.device, dtype=torch.float32)
    elif tuple(out.shape) != (angle_array.size, Rd, Cd):
        raise ValueError(f"out must be [{angle_array.size}, {Rd}, {Cd}], got {tuple(out.shape)}")
    rho = fields.rho_fine
    present = present_materials(rho)                                   # once for all views
    traced = (rho if present is None else rho[list(present)]).contiguous()
    for v, angle in enumerate(angle_array):
        path = primary_path_lengths(solver.projectors, traced, fields.grid_fine, solver.geometry, float(angle),
                                    solver.primary_samples_per_pixel_axis)
        image = primary_from_path_lengths(solver.library, path, present, solver.geometry, float(angle), solver.source,
                                          *solver.responses())
        out[v] = image["signal"] if quantity == "signal" else image["planar_fluence"].sum(0)
    return out
