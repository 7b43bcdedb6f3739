"""The scatter step of many views with their accumulator sweeps batched (several views per sweep launch).

Within an outer iteration every view sweeps the same transport grid with the same attenuation, so the sweeps of a
batch of views run as ONE persistent wavefront launch over a ``[B, 8, D8, N, 4G]`` store (the plane barriers are paid
once per batch instead of once per view), their scattering sources are expanded by one batched small-K product and
their moments accumulated by another. The uncollided fluence, first-collision source and image stay per view (each
view has its own focal spot and cone). Results equal the per-view ``citrus_view_step`` to float rounding
(``tests/test_batched_gpu.py``).
"""

from __future__ import annotations

from typing import Optional, Sequence

import torch

from . import kernels
from .citrus_step import CitrusState, project_scatter
from .scatter_solver import MaterialFields, ScatterSolver


def batched_view_steps(solver: ScatterSolver, states: Sequence[CitrusState], fields: MaterialFields,
                       angles: Sequence[float], batch: int = 4, primary: bool = False) -> tuple:
    """One CITRUS scatter step of every view, ``batch`` views per sweep launch.

    Returns (scatter signals [V, Rd, Cd], primary signals [V, Rd, Cd] or None, new states).
    """
    ctx = solver.sweep_context(fields.grid_coarse)
    precision = solver.config.moment_precision
    G, N, N_sh, D8 = solver.num_groups, ctx.num_cells, ctx.num_moments, ctx.directions_per_octant
    Q = 4 * G
    J = N * Q
    shape = tuple(ctx.shape)
    device = solver.device
    Rd, Cd = solver.geometry.image_shape
    V = len(angles)
    signals = torch.empty(V, Rd, Cd, device=device)
    primaries = torch.empty(V, Rd, Cd, device=device) if primary else None
    new_states = list(states)
    index = ctx.direction_indices(0, D8)
    Y = ctx.Y.index_select(0, index).contiguous()                  # [8 D8, N_sh]
    Yw_t = ctx.Y_weighted.index_select(0, index).t().contiguous()  # [N_sh, 8 D8]
    mu_cells = fields.mu_t_coarse.reshape(G, N).t().contiguous()
    syncs, norms, pending = [], [], []
    for b0 in range(0, V, batch):
        views = list(range(b0, min(V, b0 + batch)))
        B = len(views)
        store = torch.empty(B, 8, D8, N, Q, device=device)
        phi_uc = []
        for j, v in enumerate(views):
            if states[v].angle is not None and abs(float(states[v].angle) - float(angles[v])) > 1e-12:
                raise ValueError(f"state {v} belongs to angle {states[v].angle}, got {angles[v]}")
            uc = solver.uncollided_fluence(fields, float(angles[v]))
            first = solver.first_collision_moment_source(fields, float(angles[v]), uc, ctx)
            first(index, out=store[j].view((8 * D8,) + shape + (G, 4)))
            phi_uc.append(uc)
        previous = [states[v].collided_moments for v in views]
        if any(p is not None for p in previous):
            T_all = torch.zeros(B, N_sh, J, device=device)
            for j, p in enumerate(previous):
                if p is not None:
                    kernels.scattering_moments(fields.mu_s_l_coarse, p, "cell_major",
                                               out=T_all[j].view((N_sh,) + shape + (G, 4)))
            kernels.small_k_gemm(Y, T_all, store.view(B, 8 * D8, J), accumulate=True, precision=precision)
            del T_all
        syncs.append(kernels.sweep_planes(ctx.flat_index, store, mu_cells, ctx.c, method="persistent"))
        moments = torch.empty(B, N_sh, J, device=device)
        kernels.small_k_gemm(Yw_t, store.view(B, 8 * D8, J), moments, precision=precision)
        del store
        for j, v in enumerate(views):
            new = moments[j].view(N_sh, N, G, 4).permute(2, 0, 3, 1).reshape(G, N_sh, 4, *shape)
            cone = states[v].cone_quadrature if states[v].cone_quadrature is not None else \
                solver.cone_quadrature(fields.grid_fine, float(angles[v]))
            signals[v] = project_scatter(solver, None, fields.grid_fine, float(angles[v]), phi_uc[j], new, fields,
                                         cone, signal_only=True)["signal"]
            if primary:
                primaries[v] = solver.primary(fields, float(angles[v]))["signal"]
            prev = previous[j]
            norm = torch.linalg.vector_norm(new[:, 0, 0])
            diff = norm if prev is None else torch.linalg.vector_norm(new[:, 0, 0] - prev[:, 0, 0])
            norms.append(torch.stack([norm, diff]))
            pending.append((v, new, cone, prev is None))
    # one read-back for every view's change norm and the sweeps' barrier words, after all launches are queued
    if syncs and bool(torch.stack([w[2] for w in syncs]).ne(0).any()):
        raise kernels._lib.CitrusKernelError("batched sweep: a grid-barrier wait of the persistent sweep ran out")
    values = torch.stack(norms).tolist() if norms else []
    for (v, new, cone, cold), (norm, diff) in zip(pending, values):
        change = (1.0 if norm > 0 else 0.0) if cold else (diff / norm if norm > 0 else 0.0)
        new_states[v] = CitrusState(angle=float(angles[v]), collided_moments=new, cone_quadrature=cone,
                                    num_steps=states[v].num_steps + 1, history=states[v].history + [change])
    return signals, primaries, new_states
