"""Linear-discontinuous discrete-ordinates sweep of all directions and groups with vacuum boundaries.

Mirrors ``citrus/scatter_solver/transport_sweep.py`` and ``wavefront.py``: the quadrature is reordered by octant
(direction ``m = octant * D8 + d``), the 8 octants are swept together one diagonal wavefront plane at a time, and the
result is ``phi[g, n, k, cell] = sum_m w_m Y_n(Omega_m) psi_m[g, k, cell]``, a ``[G, N_sh, 4, R, C, S]`` view of
cell-major storage ``[N_sh, R, C, S, G, 4]``. Per direction chunk the sweep fills the chunk's store
``[8, Dc, N, 4G]`` with the source (cell-major), solves it in place (``kernels.sweep_planes``: one persistent
cooperative launch by default) and accumulates the moments with ``kernels.small_k_gemm``.
"""

from __future__ import annotations

import inspect
from dataclasses import dataclass
from typing import Callable, Optional

import numpy as np
import torch
from torch import Tensor

from . import kernels
from .geometry import Grid
from .quadrature import Quadrature, SphericalHarmonicBasis, spherical_harmonic_basis, to_device

SourceFunction = Callable[..., Tensor]

OCTANT_SIGNS = np.array([[1 if not (o & 4) else -1, 1 if not (o & 2) else -1, 1 if not (o & 1) else -1]
                         for o in range(8)], dtype=np.int64)


@dataclass(frozen=True, eq=False)
class SweepPlan:
    """Wavefront ordering of all 8 octants of a grid (reference ``wavefront.py:22-125``), numpy int64.

    Entries of plane p are ``plane_offsets[p]:plane_offsets[p+1]``; within a plane they are grouped by octant.
    ``upstream[e, a]`` is the flat index of the upstream neighbour along x, y, z, or -1 for vacuum.
    """

    shape: tuple
    num_planes: int
    plane_offsets: np.ndarray
    octant: np.ndarray
    cell: np.ndarray
    upstream: np.ndarray

    @property
    def num_cells(self) -> int:
        return int(np.prod(self.shape))


def build_sweep_plan(shape) -> SweepPlan:
    """Plane-sorted (octant, cell, upstream) entries: plane of cell (i, j, k) in octant o is i' + j' + k' with each
    index reflected where the octant's direction component is negative."""
    R, C, S = (int(v) for v in shape)
    i, j, k = (a.reshape(-1) for a in np.meshgrid(np.arange(R), np.arange(C), np.arange(S), indexing="ij"))
    flat = (i * C + j) * S + k
    n = flat.size
    octs, cells, ups, planes = [], [], [], []
    for o in range(8):
        sx, sy, sz = OCTANT_SIGNS[o]
        px = j if sx > 0 else C - 1 - j
        py = i if sy > 0 else R - 1 - i
        pz = k if sz > 0 else S - 1 - k
        nj, ni, nk = j - sx, i - sy, k - sz
        ux = np.where((nj >= 0) & (nj < C), (i * C + nj) * S + k, -1)
        uy = np.where((ni >= 0) & (ni < R), (ni * C + j) * S + k, -1)
        uz = np.where((nk >= 0) & (nk < S), (i * C + j) * S + nk, -1)
        octs.append(np.full(n, o, dtype=np.int64))
        cells.append(flat)
        ups.append(np.stack([ux, uy, uz], axis=1))
        planes.append(px + py + pz)
    octant, cell, upstream, plane = (np.concatenate(a) for a in (octs, cells, ups, planes))
    order = np.argsort(plane * 8 + octant, kind="stable")
    octant, cell, upstream, plane = octant[order], cell[order], upstream[order], plane[order]
    num_planes = R + C + S - 2
    offsets = np.zeros(num_planes + 1, dtype=np.int64)
    offsets[1:] = np.cumsum(np.bincount(plane, minlength=num_planes))
    return SweepPlan((R, C, S), num_planes, offsets, octant, cell, upstream)


@dataclass(frozen=True, eq=False)
class TiledPlan:
    """The entries of a sweep plan in tile-diagonal order (no counterpart in the reference, whose plan is one launch
    per plane): in each octant's sweep frame the cells are cut into tiles of ``tile``^3; a task is one tile of one
    octant, the tasks of a diagonal (equal sums of tile coordinates) are independent, and within a task the entries run
    by sub-plane (equal sums of in-tile coordinates).

    Attributes:
        octant, cell, upstream: the entries (as in ``SweepPlan``), ordered by task and sub-plane.
        sub_offsets: [tasks, num_sub + 1] entry range of each sub-plane of each task.
        diagonal_offsets: [num_diagonals + 1] task range of each diagonal.
    """

    shape: tuple
    tile: int
    num_sub: int
    octant: np.ndarray
    cell: np.ndarray
    upstream: np.ndarray
    sub_offsets: np.ndarray
    diagonal_offsets: np.ndarray

    @property
    def num_diagonals(self) -> int:
        return int(self.diagonal_offsets.size - 1)

    @property
    def num_tasks(self) -> int:
        return int(self.sub_offsets.shape[0])


def build_tiled_plan(shape, tile: int) -> TiledPlan:
    """The plan's entries in tile-diagonal order: a cell's octant-frame coordinates (as in ``build_sweep_plan``) split
    into tile coordinates (the diagonal is their sum) and in-tile coordinates (the sub-plane is their sum); every
    upstream neighbour of a cell is on the same sub-plane minus one of its tile or on an earlier diagonal."""
    R, C, S = (int(v) for v in shape)
    T = int(tile)
    if T < 1:
        raise ValueError("tile must be >= 1")
    i, j, k = (a.reshape(-1) for a in np.meshgrid(np.arange(R), np.arange(C), np.arange(S), indexing="ij"))
    flat = (i * C + j) * S + k
    n = flat.size
    nt = [-(-C // T), -(-R // T), -(-S // T)]                      # tiles along x (cols), y (rows), z (slices)
    num_sub = 3 * T - 2
    octs, cells, ups, keys, subs, diags = [], [], [], [], [], []
    for o in range(8):
        sx, sy, sz = OCTANT_SIGNS[o]
        px = j if sx > 0 else C - 1 - j
        py = i if sy > 0 else R - 1 - i
        pz = k if sz > 0 else S - 1 - k
        nj, ni, nk = j - sx, i - sy, k - sz
        ux = np.where((nj >= 0) & (nj < C), (i * C + nj) * S + k, -1)
        uy = np.where((ni >= 0) & (ni < R), (ni * C + j) * S + k, -1)
        uz = np.where((nk >= 0) & (nk < S), (i * C + j) * S + nk, -1)
        tx, ty, tz = px // T, py // T, pz // T
        diag = tx + ty + tz
        keys.append(((diag * 8 + o) * nt[0] + tx) * nt[1] * nt[2] + ty * nt[2] + tz)
        subs.append(px % T + py % T + pz % T)
        diags.append(diag)
        octs.append(np.full(n, o, dtype=np.int64))
        cells.append(flat)
        ups.append(np.stack([ux, uy, uz], axis=1))
    key, sub, diag, octant, cell, upstream = (np.concatenate(a) for a in (keys, subs, diags, octs, cells, ups))
    task_keys, task = np.unique(key, return_inverse=True)          # ascending key: diagonals in order
    order = np.lexsort((cell, sub, task))
    octant, cell, upstream, sub, task = octant[order], cell[order], upstream[order], sub[order], task[order]
    num_tasks = task_keys.size
    counts = np.bincount(task * num_sub + sub, minlength=num_tasks * num_sub).reshape(num_tasks, num_sub)
    sub_offsets = np.zeros((num_tasks, num_sub + 1), dtype=np.int64)
    sub_offsets[:, 1:] = np.cumsum(counts, axis=1)
    sub_offsets += np.concatenate([[0], np.cumsum(counts.sum(1))[:-1]])[:, None]
    task_diag = np.zeros(num_tasks, dtype=np.int64)
    task_diag[task] = diag[order]
    num_diagonals = int(task_diag.max()) + 1
    diagonal_offsets = np.zeros(num_diagonals + 1, dtype=np.int64)
    diagonal_offsets[1:] = np.cumsum(np.bincount(task_diag, minlength=num_diagonals))
    return TiledPlan((R, C, S), T, num_sub, octant, cell, upstream, sub_offsets, diagonal_offsets)


@dataclass(frozen=True, eq=False)
class SweepContext:
    """Everything the sweep needs that depends only on the grid and the quadrature (reference
    ``transport_sweep.py:77-153``); device tables are float32 / int32 on ``device``."""

    shape: tuple
    deltas: tuple
    L: int
    plan: SweepPlan
    quadrature: Quadrature
    permutation: np.ndarray
    basis: SphericalHarmonicBasis
    directions_per_octant: int
    c: Tensor
    s: Tensor
    Y: Tensor
    Y_weighted: Tensor
    flat_index: kernels.FlatPlaneIndex
    device: torch.device
    omega: Tensor = None       # [8 D8, 3] float32 directions of the reordered quadrature
    weight: Tensor = None      # [8 D8] float32 weights

    @property
    def num_cells(self) -> int:
        return self.shape[0] * self.shape[1] * self.shape[2]

    def tiled_index(self, tile: int) -> kernels.TiledIndex:
        """The entry tables in tile-diagonal order for tiles of ``tile``^3 cells (built once per tile size)."""
        cache = self.__dict__.setdefault("_tiled", {})
        index = cache.get(int(tile))
        if index is None:
            plan = build_tiled_plan(self.shape, int(tile))
            up = np.where(plan.upstream < 0, self.num_cells, plan.upstream)
            dev = lambda a: torch.as_tensor(np.ascontiguousarray(a).astype(np.int32)).to(self.device)  # noqa: E731
            index = kernels.TiledIndex(tile=int(tile), num_sub=plan.num_sub, octant=dev(plan.octant),
                                       cell=dev(plan.cell), upstream=dev(up.reshape(-1)),
                                       sub_offsets=dev(plan.sub_offsets), diagonal_offsets=dev(plan.diagonal_offsets))
            cache[int(tile)] = index
        return index

    @property
    def num_planes(self) -> int:
        return self.plan.num_planes

    @property
    def num_directions(self) -> int:
        return 8 * self.directions_per_octant

    @property
    def num_moments(self) -> int:
        return (self.L + 1) ** 2

    def direction_indices(self, start: int, stop: int) -> Tensor:
        """Octant-major reordered indices of the per-octant chunk ``start <= d < stop``: ``o * D8 + d``."""
        d = torch.arange(start, stop, dtype=torch.int64, device=self.device)
        o = torch.arange(8, dtype=torch.int64, device=self.device)
        return (o[:, None] * self.directions_per_octant + d[None, :]).reshape(-1)


def make_sweep_context(grid: Grid, quadrature: Quadrature, L: int, device) -> SweepContext:
    """Sweep context of a grid and a quadrature (reference ``transport_sweep.py:156-235``)."""
    D8 = quadrature.directions_per_octant
    if D8 is None or D8 < 1:
        raise ValueError("the quadrature must hold the same (non-zero) number of directions in every octant")
    if L < 0:
        raise ValueError("L must be >= 0")
    device = torch.device(device)
    permutation = quadrature.by_octant()
    reordered = quadrature.reordered(permutation)
    if not np.array_equal(reordered.octant, np.repeat(np.arange(8), D8)):
        raise RuntimeError("octant reordering failed")
    basis = spherical_harmonic_basis(L, reordered)
    deltas = tuple(float(v) for v in grid.deltas)
    omega = reordered.omega.reshape(8, D8, 3)
    c = np.abs(omega) / np.asarray(deltas)
    s = np.where(omega < 0, -1.0, 1.0)
    if not np.array_equal(s.astype(np.int64), np.broadcast_to(OCTANT_SIGNS[:, None, :], (8, D8, 3))):
        raise RuntimeError("direction signs disagree with the sweep plan's octant signs")
    plan = build_sweep_plan(grid.shape)
    N = plan.num_cells
    upstream = np.where(plan.upstream < 0, N, plan.upstream)
    flat = kernels.FlatPlaneIndex(
        octant=torch.as_tensor(plan.octant.astype(np.int32)).to(device),
        cell=torch.as_tensor(plan.cell.astype(np.int32)).to(device),
        upstream=torch.as_tensor(upstream.astype(np.int32).reshape(-1)).to(device),
        offsets=tuple(int(v) for v in plan.plane_offsets),
        offsets_host=torch.as_tensor(plan.plane_offsets.astype(np.int64)),
        offsets_device=torch.as_tensor(plan.plane_offsets.astype(np.int32)).to(device))
    return SweepContext(shape=tuple(grid.shape), deltas=deltas, L=int(L), plan=plan, quadrature=reordered,
                        permutation=permutation, basis=basis, directions_per_octant=D8, c=to_device(c, device),
                        s=to_device(s, device), Y=to_device(basis.Y, device),
                        Y_weighted=to_device(basis.Y_weighted, device), flat_index=flat, device=device,
                        omega=torch.as_tensor(reordered.omega, dtype=torch.float32).to(device),
                        weight=torch.as_tensor(reordered.weight, dtype=torch.float32).to(device))


def source_function_accepts_out(source_function) -> bool:
    try:
        p = inspect.signature(source_function).parameters.get("out")
    except (TypeError, ValueError):
        return False
    return p is not None and p.kind in (inspect.Parameter.POSITIONAL_OR_KEYWORD, inspect.Parameter.KEYWORD_ONLY)


def source_is_cell_major(source_function) -> bool:
    return bool(getattr(source_function, "cell_major", False))


def _fill_source(ctx: SweepContext, source_function, d0: int, d1: int, G: int, out: Tensor) -> None:
    """Evaluate the chunk's source once for all ``8 dc`` directions and store it cell-major in ``out``
    (reference ``transport_sweep.py:408-450``)."""
    chunk = d1 - d0
    N = ctx.num_cells
    index = ctx.direction_indices(d0, d1)
    if source_is_cell_major(source_function):
        cell_major = out.view((8 * chunk,) + tuple(ctx.shape) + (G, 4))
        result = source_function(index, out=cell_major)
        if result.data_ptr() != cell_major.data_ptr() or tuple(result.shape) != tuple(cell_major.shape):
            raise ValueError("a cell-major source function must write its [Dsel, R, C, S, G, 4] moments into `out`")
        return
    expected = (8 * chunk, G, 4) + tuple(ctx.shape)
    result = source_function(index)
    if tuple(result.shape) != expected:
        raise ValueError(f"source_function returned shape {tuple(result.shape)}, expected {expected}")
    out.view(8 * chunk, N, 4 * G).copy_(result.reshape(8 * chunk, 4 * G, N).transpose(1, 2))


def sweep(ctx: SweepContext, mu_t: Tensor, source_function, direction_chunk: Optional[int] = None,
          return_psi: bool = False, method: str = "persistent", check: bool = True, precision: str = "fp32"):
    """Sweep every direction and group (reference ``transport_sweep.py:457-537``).

    Args:
        ctx: sweep context.
        mu_t: [G, R, C, S] float32 CUDA total attenuation in 1/cm.
        source_function: ``source(direction_index [Dsel], out=..)`` writing cell-major moments
            ``[Dsel, R, C, S, G, 4]`` into ``out`` (``cell_major = True``), or returning ``[Dsel, G, 4, R, C, S]``.
        direction_chunk: directions per octant swept together (None: all D8).
        return_psi: also return the angular fluence ``[M, G, 4, R, C, S]`` (tests).
        method: plane driver of ``kernels.sweep_planes``.
        check: read back the barrier words and raise on a timeout (one host synchronization per sweep).
        precision: arithmetic of the moment accumulation ``Yw^T psi`` (``kernels.small_k_gemm``).

    Returns:
        phi ``[G, N_sh, 4, R, C, S]`` (a view of cell-major storage), or (phi, psi).
    """
    if mu_t.dim() != 4 or tuple(mu_t.shape[1:]) != tuple(ctx.shape):
        raise ValueError(f"mu_t must be [G, {ctx.shape}], got {tuple(mu_t.shape)}")
    kernels._check_cuda_f32("mu_t", mu_t, contiguous=False)
    G = int(mu_t.shape[0])
    Q = 4 * G
    N = ctx.num_cells
    D8 = ctx.directions_per_octant
    Dc = D8 if direction_chunk is None else max(1, min(int(direction_chunk), D8))
    device = mu_t.device
    mu_cells = mu_t.reshape(G, N).t().contiguous()
    moments = torch.empty(ctx.num_moments, N * Q, device=device, dtype=torch.float32)
    psi_out = torch.zeros(ctx.num_directions, G, 4, N, device=device) if return_psi else None
    syncs = []
    first = True
    for d0 in range(0, D8, Dc):
        d1 = min(d0 + Dc, D8)
        chunk = d1 - d0
        index = ctx.direction_indices(d0, d1)
        c = ctx.c[:, d0:d1].contiguous()
        store = torch.empty(8, chunk, N, Q, device=device, dtype=torch.float32)
        _fill_source(ctx, source_function, d0, d1, G, store)
        sync = kernels.sweep_planes(ctx.flat_index, store, mu_cells, c, method=method)
        if sync is not None:
            syncs.append(sync)
        weights = ctx.Y_weighted.index_select(0, index).t().contiguous()  # [N_sh, 8 dc]
        kernels.small_k_gemm(weights, store.view(8 * chunk, N * Q), moments, accumulate=not first,
                             precision=precision)
        first = False
        if psi_out is not None:
            psi_out[index] = store.view(8 * chunk, N, Q).permute(0, 2, 1).reshape(8 * chunk, G, 4, N)
    if check and syncs:
        if bool(torch.stack([s[2] for s in syncs]).ne(0).any()):
            raise kernels._lib.CitrusKernelError("sweep: a grid-barrier wait of the persistent sweep ran out")
    phi = moments.view(ctx.num_moments, N, G, 4).permute(2, 0, 3, 1).reshape(G, ctx.num_moments, 4, *ctx.shape)
    if psi_out is not None:
        return phi, psi_out.view(ctx.num_directions, G, 4, *ctx.shape)
    return phi
