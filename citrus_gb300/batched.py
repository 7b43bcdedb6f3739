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


SWEEP_STORE_BUDGET_BYTES = 40 * 2 ** 30   # the store of one view's chunk: 8 x directions x N x 4G floats


def direction_chunk(num_cells: int, num_groups: int, directions_per_octant: int,
                    budget: Optional[int] = None) -> int:
    """Directions per octant swept together in one view's chunk: all of them when the store fits ``budget``
    (``SWEEP_STORE_BUDGET_BYTES`` when None) and the sweep's 32-bit lane positions (8 N dc G float4 below 2^31),
    else as many as do."""
    budget = SWEEP_STORE_BUDGET_BYTES if budget is None else int(budget)
    per_direction = 8 * num_cells * 4 * num_groups * 4
    lanes = (2 ** 31 - 1) // (8 * num_cells * num_groups)
    return max(1, min(directions_per_octant, budget // per_direction, lanes))


def sweep_launch_config(solver: ScatterSolver, fields: MaterialFields, views: int, batch: int) -> tuple:
    """(views per sweep launch, form of the sweep threads, directions per octant per chunk): the autotuner's choice
    for this grid and chunk, with ``batch`` views when it is positive."""
    from .autotune import sweep_config

    ctx = solver.sweep_context(fields.grid_coarse)
    G = solver.num_groups
    dc = direction_chunk(ctx.num_cells, G, ctx.directions_per_octant)
    mu_cells = fields.mu_t_coarse.reshape(G, ctx.num_cells).t().contiguous()
    tuned_views, form = sweep_config(ctx, mu_cells, G, views, dc=dc)
    chosen = min(int(batch), max(1, views)) if batch > 0 else tuned_views
    return min(chosen, views_that_fit(ctx, G, dc, solver.device)), form, dc


def views_that_fit(ctx, num_groups: int, dc: int, device, share: float = 0.6) -> int:
    """Views per sweep launch whose working set fits ``share`` of the free device memory: per view its scattering
    moments and new accumulator (N_sh x N x 4G floats each), the chunk's store (8 x dc x N x 4G) and first-collision
    means (8 x dc x N x G)."""
    N, J = ctx.num_cells, ctx.num_cells * 4 * num_groups
    per_view = 4 * (2 * ctx.num_moments * J + 8 * dc * J + 8 * dc * N * num_groups)
    if torch.cuda.is_current_stream_capturing():
        return 1 << 30
    free, _ = torch.cuda.mem_get_info(device)
    # memory the caching allocator holds but no tensor uses counts as free: the count then does not depend on what
    # the previous step left cached, and the views per launch (and the products' tuned shapes) stay the same
    free += torch.cuda.memory_reserved(device) - torch.cuda.memory_allocated(device)
    return max(1, int(share * free) // per_view)


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
    mu_cells = fields.mu_t_coarse.reshape(G, N).t().contiguous()
    syncs, norms, accumulators = [], [], []
    batch, form, dc = sweep_launch_config(solver, fields, V, batch)
    for b0 in range(0, V, batch):
        views = list(range(b0, min(V, b0 + batch)))
        B = len(views)
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
        T_all = None
        if warm:  # the scattering moments of every view, formed before any chunk overwrites an accumulator
            T_all = torch.zeros(B, N_sh, J, device=device)
            for j, p in enumerate(previous):
                if p is not None:
                    kernels.scattering_moments(fields.mu_s_l_coarse, p, "cell_major",
                                               out=T_all[j].view((N_sh,) + shape + (G, 4)))
        moments = torch.empty(B, N_sh, J, device=device) if store_out is None else store_out[b0:b0 + B]
        for d0 in range(0, D8, dc):   # direction chunks (one, unless a view's store outgrows the budget)
            d1 = min(D8, d0 + dc)
            k = d1 - d0
            index = ctx.direction_indices(d0, d1)
            Y = ctx.Y.index_select(0, index).contiguous()                  # [8 k, N_sh]
            Yw_t = ctx.Y_weighted.index_select(0, index).t().contiguous()  # [N_sh, 8 k]
            store = torch.empty(B, 8, k, N, Q, device=device)
            if fused:
                means = torch.empty(B, 8 * k, N * G, device=device)
                for j, first in enumerate(firsts):
                    first.means(index, out=means[j])
                kernels.source_expansion_first(Y, T_all, store.view(B, 8 * k, J), means, precision=precision)
                del means
            else:
                for j, first in enumerate(firsts):
                    first(index, out=store[j].view((8 * k,) + shape + (G, 4)))
                if warm:
                    kernels.small_k_gemm(Y, T_all, store.view(B, 8 * k, J), accumulate=True, precision=precision)
            c = ctx.c if k == D8 else ctx.c[:, d0:d1].contiguous()
            syncs.append(kernels.sweep_chunk(ctx, store, mu_cells, c, form))
            kernels.small_k_gemm(Yw_t, store.view(B, 8 * k, J), moments, accumulate=d0 > 0, precision=precision)
            del store
        del T_all
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

    def seed(self, rho: Tensor, accumulators: Sequence[Tensor]) -> None:
        """Start every view from a given accumulator ``[G, N_sh, 4, Rc, Cc, Sc]`` (the learned proposal, say)
        instead of the cold start: the accumulators are copied into the store, and the next ``step`` runs warm (and
        records the graph)."""
        if len(accumulators) != len(self.angles):
            raise ValueError(f"need one accumulator per view ({len(self.angles)}), got {len(accumulators)}")
        self._refresh_fields(rho)
        ctx = self.solver.sweep_context(self.fields.grid_coarse)
        G, N_sh, shape = self.solver.num_groups, ctx.num_moments, ctx.shape
        if self.store is None:
            self.store = torch.empty(len(self.angles), N_sh, ctx.num_cells * 4 * G, device=self.solver.device)
        self.graph = None
        for v, acc in enumerate(accumulators):
            view = self.store[v].view(N_sh, *shape, G, 4).permute(4, 0, 5, 1, 2, 3)   # [G, N_sh, 4, Rc, Cc, Sc]
            if tuple(acc.shape) != tuple(view.shape):
                raise ValueError(f"accumulator {v} must be {tuple(view.shape)}, got {tuple(acc.shape)}")
            view.copy_(acc)
            self.states[v] = CitrusState(angle=self.angles[v], collided_moments=view)

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
