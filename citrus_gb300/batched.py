"""The scatter step of many views with their accumulator sweeps batched (several views per sweep launch), and the
whole outer iteration captured once into a CUDA graph and replayed.

Within an outer iteration every view sweeps the same transport grid with the same attenuation, so the sweeps of a
batch of views run as ONE persistent wavefront launch over a ``[B, 8, D8, N, 4G]`` store (the plane barriers are paid
once per batch instead of once per view), their scattering sources are expanded by one batched small-K product and
their moments accumulated by another. The uncollided fluence, first-collision source and image stay per view (each
view has its own focal spot and cone). Results equal the per-view ``citrus_view_step`` to float rounding
(``tests/test_batched_gpu.py``).

:class:`GraphedOuterIteration` keeps every view's accumulator in one ``[V, N_sh, N 4G]`` store that each step updates
in place (a view's scattering moments are read from it before the new moments are written over it), so the launches
of one outer iteration, about 400 per view, are recorded once into a CUDA graph and replayed for every further
iteration with no host work per view.
"""

from __future__ import annotations

from dataclasses import replace
from typing import Optional, Sequence

import torch
from torch import Tensor

from . import kernels
from .citrus_step import CitrusState, project_scatter
from .scatter_solver import MaterialFields, ScatterSolver


def _check_states(states: Sequence[CitrusState], angles: Sequence[float]) -> None:
    for v, (state, angle) in enumerate(zip(states, angles)):
        if state.angle is not None and abs(float(state.angle) - float(angle)) > 1e-12:
            raise ValueError(f"state {v} belongs to angle {state.angle}, got {angle}")


def sweep_launch_config(solver: ScatterSolver, fields: MaterialFields, views: int, batch: int) -> tuple:
    """(views per sweep launch, form of the sweep threads): the autotuner's choice for this grid, with ``batch``
    views when it is positive."""
    from .autotune import sweep_config

    ctx = solver.sweep_context(fields.grid_coarse)
    G = solver.num_groups
    mu_cells = fields.mu_t_coarse.reshape(G, ctx.num_cells).t().contiguous()
    tuned_views, form = sweep_config(ctx, mu_cells, G, views)
    return (min(int(batch), max(1, views)) if batch > 0 else tuned_views), form


def resolve_batch(solver: ScatterSolver, fields: MaterialFields, views: int, batch: int) -> int:
    """Views per sweep launch: ``batch`` when positive, else the autotuner's choice for this grid."""
    return sweep_launch_config(solver, fields, views, batch)[0]


def _launch_views(solver: ScatterSolver, states: Sequence[CitrusState], fields: MaterialFields,
                  angles: Sequence[float], batch: int, primary: bool, store_out: Optional[Tensor],
                  signals: Tensor, cones: list) -> tuple:
    """Queue the step of every view; no host read-back. Returns (primaries, new accumulators, [V, 2] norms of the new
    scalar flux and of its change, [batches, 4] sweep barrier words)."""
    ctx = solver.sweep_context(fields.grid_coarse)
    precision = solver.config.moment_precision
    G, N, N_sh, D8 = solver.num_groups, ctx.num_cells, ctx.num_moments, ctx.directions_per_octant
    Q = 4 * G
    J = N * Q
    shape = tuple(ctx.shape)
    device = solver.device
    Rd, Cd = solver.geometry.image_shape
    V = len(angles)
    primaries = torch.empty(V, Rd, Cd, device=device) if primary else None
    index = ctx.direction_indices(0, D8)
    Y = ctx.Y.index_select(0, index).contiguous()                  # [8 D8, N_sh]
    Yw_t = ctx.Y_weighted.index_select(0, index).t().contiguous()  # [N_sh, 8 D8]
    mu_cells = fields.mu_t_coarse.reshape(G, N).t().contiguous()
    syncs, norms, accumulators = [], [], []
    batch, form = sweep_launch_config(solver, fields, V, batch)
    for b0 in range(0, V, batch):
        views = list(range(b0, min(V, b0 + batch)))
        B = len(views)
        store = torch.empty(B, 8, D8, N, Q, device=device)
        phi_uc, firsts = [], []
        for v in views:
            uc = solver.uncollided_fluence(fields, float(angles[v]))
            firsts.append(solver.first_collision_moment_source(fields, float(angles[v]), uc, ctx))
            phi_uc.append(uc)
        previous = [states[v].collided_moments for v in views]
        # the previous scalar flux, kept for the change norm before an in-place store overwrites it
        previous_scalar = [None if p is None else p[:, 0, 0].clone() for p in previous]
        warm = any(p is not None for p in previous)
        # with one point per cell the first-collision moments are (mean, 0, 0, 0): their means go into the float32
        # source expansion's output pass instead of being written into the store and read back by it (in either
        # moment precision: the single pass moves less than half the bytes of the two, whichever form the product takes)
        fused = warm and N_sh <= 64 and all(f.means is not None for f in firsts)
        if fused:
            means = torch.empty(B, 8 * D8, N * G, device=device)
            for j, first in enumerate(firsts):
                first.means(index, out=means[j])
        else:
            for j, first in enumerate(firsts):
                first(index, out=store[j].view((8 * D8,) + shape + (G, 4)))
        if warm:
            T_all = torch.zeros(B, N_sh, J, device=device)
            for j, p in enumerate(previous):
                if p is not None:
                    kernels.scattering_moments(fields.mu_s_l_coarse, p, "cell_major",
                                               out=T_all[j].view((N_sh,) + shape + (G, 4)))
            if fused:
                kernels.source_expansion_first(Y, T_all, store.view(B, 8 * D8, J), means, precision=precision)
                del means
            else:
                kernels.small_k_gemm(Y, T_all, store.view(B, 8 * D8, J), accumulate=True, precision=precision)
            del T_all
        syncs.append(kernels.sweep_chunk(ctx, store, mu_cells, ctx.c, form))
        moments = torch.empty(B, N_sh, J, device=device) if store_out is None else store_out[b0:b0 + B]
        kernels.small_k_gemm(Yw_t, store.view(B, 8 * D8, J), moments, precision=precision)
        del store
        for j, v in enumerate(views):
            new = moments[j].view(N_sh, N, G, 4).permute(2, 0, 3, 1).reshape(G, N_sh, 4, *shape)
            signals[v] = project_scatter(solver, None, fields.grid_fine, float(angles[v]), phi_uc[j], new, fields,
                                         cones[v], signal_only=True)["signal"]
            if primary:
                primaries[v] = solver.primary(fields, float(angles[v]))["signal"]
            norm = torch.linalg.vector_norm(new[:, 0, 0])
            prev = previous_scalar[j]
            diff = norm if prev is None else torch.linalg.vector_norm(new[:, 0, 0] - prev)
            norms.append(torch.stack([norm, diff]))
            accumulators.append(new)
    sync_words = torch.stack([s for s in syncs]) if syncs else torch.zeros(0, 4, dtype=torch.int32, device=device)
    return primaries, accumulators, torch.stack(norms), sync_words


def _finish(states: Sequence[CitrusState], angles: Sequence[float], cones: list, accumulators: list,
            norms: Tensor, sync_words: Tensor) -> list:
    """One read-back for every view's change norm and the sweeps' barrier words; the new states."""
    if sync_words.numel() and bool(sync_words[:, 2].ne(0).any()):
        raise kernels._lib.CitrusKernelError("batched sweep: a grid-barrier wait of the persistent sweep ran out")
    values = norms.tolist()
    new_states = []
    for v, (norm, diff) in enumerate(values):
        cold = states[v].collided_moments is None
        change = (1.0 if norm > 0 else 0.0) if cold else (diff / norm if norm > 0 else 0.0)
        new_states.append(CitrusState(angle=float(angles[v]), collided_moments=accumulators[v],
                                      cone_quadrature=cones[v], num_steps=states[v].num_steps + 1,
                                      history=states[v].history + [change]))
    return new_states


def _cones(solver: ScatterSolver, states: Sequence[CitrusState], fields: MaterialFields,
           angles: Sequence[float]) -> list:
    return [s.cone_quadrature if s.cone_quadrature is not None else solver.cone_quadrature(fields.grid_fine, float(a))
            for s, a in zip(states, angles)]


def batched_view_steps(solver: ScatterSolver, states: Sequence[CitrusState], fields: MaterialFields,
                       angles: Sequence[float], batch: int = 4, primary: bool = False) -> tuple:
    """One CITRUS scatter step of every view, ``batch`` views per sweep launch (0: the autotuner's choice).

    Returns (scatter signals [V, Rd, Cd], primary signals [V, Rd, Cd] or None, new states).
    """
    _check_states(states, angles)
    Rd, Cd = solver.geometry.image_shape
    signals = torch.empty(len(angles), Rd, Cd, device=solver.device)
    cones = _cones(solver, states, fields, angles)
    primaries, accumulators, norms, sync_words = _launch_views(solver, states, fields, angles, batch, primary, None,
                                                               signals, cones)
    return signals, primaries, _finish(states, angles, cones, accumulators, norms, sync_words)


class GraphedOuterIteration:
    """Every view's scatter step of one outer iteration, replayed from a CUDA graph.

    The first ``step`` runs the cold start eagerly into a ``[V, N_sh, N 4G]`` accumulator store; the second runs the
    warm step eagerly in place (every lazily built table and context now exists) and then records it into a CUDA
    graph; every further ``step`` refreshes the material fields into the graph's static field tensors and replays the
    graph, which reads each view's accumulator from the store and writes the new one over it. A change of the traced
    materials re-records the graph.

    ``step`` returns (signals [V, Rd, Cd], states): the signals tensor is the graph's output buffer, overwritten by the
    next replay (copy it to keep it); the states' accumulators are views of the store, updated in place likewise.
    """

    def __init__(self, solver: ScatterSolver, grid_fine, angles: Sequence[float], batch: int = 4) -> None:
        self.solver, self.grid, self.batch = solver, grid_fine, int(batch)
        self.angles = [float(a) for a in angles]
        # every view's direction context must stay cached: the graph reads the tables it holds
        solver.direction_context_cache_size = max(solver.direction_context_cache_size, len(self.angles))
        self.states = [CitrusState() for _ in self.angles]
        self.store: Optional[Tensor] = None
        self.fields: Optional[MaterialFields] = None
        self.graph: Optional[torch.cuda.CUDAGraph] = None
        self.replays = 0
        Rd, Cd = solver.geometry.image_shape
        self.signals = torch.empty(len(self.angles), Rd, Cd, device=solver.device)

    def _refresh_fields(self, rho: Tensor) -> bool:
        """Copy the fields of ``rho`` into the static ones; False when the traced materials changed."""
        fresh = self.solver.material_fields(rho, self.grid)
        if self.fields is None or fresh.traced_materials != self.fields.traced_materials:
            self.fields = fresh
            return False
        f = self.fields
        for name in ("rho_fine", "rho_coarse", "rho_quadrature", "mu_t_coarse", "mu_s_l_coarse"):
            dst, src = getattr(f, name), getattr(fresh, name)
            if dst.data_ptr() != src.data_ptr():
                dst.copy_(src)
        return True

    def _eager(self) -> None:
        cones = _cones(self.solver, self.states, self.fields, self.angles)
        _, accumulators, norms, sync_words = _launch_views(self.solver, self.states, self.fields, self.angles,
                                                           self.batch, False, self.store, self.signals, cones)
        self.states = _finish(self.states, self.angles, cones, accumulators, norms, sync_words)

    def _capture(self) -> None:
        cones = _cones(self.solver, self.states, self.fields, self.angles)
        # the graph reads the accumulators from the store, where the warm states' views already point
        warm = [replace(s) for s in self.states]
        self.graph = torch.cuda.CUDAGraph()
        stream = torch.cuda.Stream(self.solver.device)
        stream.wait_stream(torch.cuda.current_stream(self.solver.device))
        with torch.cuda.stream(stream), torch.cuda.graph(self.graph, stream=stream):
            _, self._accumulators, self._norms, self._sync_words = _launch_views(
                self.solver, warm, self.fields, self.angles, self.batch, False, self.store, self.signals, cones)
        torch.cuda.current_stream(self.solver.device).wait_stream(stream)
        self._cones = cones

    def step(self, rho: Tensor) -> tuple:
        """One outer iteration's scatter step of every view from fine densities ``rho`` [M, R, C, S]."""
        solver = self.solver
        same_materials = self._refresh_fields(rho)
        if self.store is None:
            ctx = solver.sweep_context(self.fields.grid_coarse)
            self.store = torch.empty(len(self.angles), ctx.num_moments, ctx.num_cells * 4 * solver.num_groups,
                                     device=solver.device)
        if self.graph is None or not same_materials:
            self.graph = None
            warm = all(s.collided_moments is not None for s in self.states)
            self._eager()
            if warm:
                self._capture()
            return self.signals, self.states
        self.graph.replay()
        self.replays += 1
        self.states = _finish(self.states, self.angles, self._cones, self._accumulators, self._norms,
                              self._sync_words)
        return self.signals, self.states
