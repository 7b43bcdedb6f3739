"""Python face of the sm_103a kernels, with the names, arguments and errors of the reference's kernel modules.

Each function validates its tensors on the host (float32, CUDA, contiguous where required, matching shapes; a
``ValueError`` otherwise, as in ``citrus/scatter_solver/kernels/*.py``) and then calls one C-ABI entry point of
``libcitrus_gb300.so`` on the current stream. There is no other implementation behind them: on a machine without the
library or without CUDA the calls raise.
"""

from __future__ import annotations

import math
from dataclasses import dataclass
from typing import Optional

import torch
from torch import Tensor

from . import _lib

LAYOUTS = ("contiguous", "moment_major", "cell_major")
DEFAULT_BARRIER_TIMEOUT_NS = 2_000_000_000


def kernels_usable(device) -> tuple:
    """(usable, reason) for ``device``: a CUDA device and a loadable library of the current ABI; never raises."""
    device = torch.device(device)
    if device.type != "cuda":
        return False, "not a CUDA device"
    if not torch.cuda.is_available():
        return False, "CUDA is not available"
    try:
        version = _lib.library().citrus_abi_version()
    except Exception as e:  # noqa: BLE001
        return False, f"library unavailable ({type(e).__name__}: {e})"
    return True, f"libcitrus_gb300 ABI {version} on {torch.cuda.get_device_name(device)}"


def _check_cuda_f32(name: str, t: Tensor, contiguous: bool = True) -> None:
    if not isinstance(t, Tensor) or t.device.type != "cuda" or t.dtype != torch.float32:
        raise ValueError(f"{name} must be a float32 CUDA tensor")
    if contiguous and not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")


# =====================================================================================================================
# transport sweep
# =====================================================================================================================

@dataclass(frozen=True, eq=False)
class FlatPlaneIndex:
    """Plane-sorted int32 entry tables of a sweep plan on the sweep device (reference ``sweep_kernels.py:44-78``).

    Attributes:
        octant: [E] octant code of each entry (E = 8 N), sorted by plane.
        cell: [E] flat cell index.
        upstream: [E * 3] upstream neighbour along x, y, z, N for vacuum.
        offsets: num_planes + 1 host ints.
        offsets_host: the offsets as an int64 CPU tensor (for the per-plane launches).
        offsets_device: the offsets as an int32 device tensor (for the persistent launch).
    """

    octant: Tensor
    cell: Tensor
    upstream: Tensor
    offsets: tuple
    offsets_host: Tensor
    offsets_device: Tensor

    @property
    def num_planes(self) -> int:
        return len(self.offsets) - 1


@dataclass(frozen=True)
class TiledIndex:
    """A sweep plan's int32 entry tables in tile-diagonal order on the sweep device (``transport_sweep.TiledPlan``).

    Attributes:
        tile: tile edge T in cells.
        num_sub: sub-planes per tile, 3 T - 2.
        octant, cell, upstream: the entries ([E], [E], [E * 3] with N for vacuum) by task and sub-plane.
        sub_offsets: [tasks, num_sub + 1] entry ranges of the tasks' sub-planes.
        diagonal_offsets: [num_diagonals + 1] task ranges of the diagonals.
    """

    tile: int
    num_sub: int
    octant: Tensor
    cell: Tensor
    upstream: Tensor
    sub_offsets: Tensor
    diagonal_offsets: Tensor

    @property
    def num_diagonals(self) -> int:
        return int(self.diagonal_offsets.numel() - 1)


@dataclass(frozen=True)
class SweepForm:
    """How an accumulator sweep runs: ``tile`` 0 is the plane wavefront (one grid barrier per plane) with the thread
    form ``thread_form`` of ``sweep_planes``; a tile edge T > 0 is the tiled schedule (``sweep_tiled``: one grid barrier
    per tile diagonal) with ``dirs_per_block`` directions per task and thread form 1 or 2."""

    thread_form: int = 1
    tile: int = 0
    dirs_per_block: int = 1


def sweep_tiled(index: TiledIndex, store: Tensor, mu_cells: Tensor, c: Tensor, *, dirs_per_block: int = 1,
                thread_form: int = 1, sync: Optional[Tensor] = None, max_blocks: int = 0,
                timeout_ns: int = DEFAULT_BARRIER_TIMEOUT_NS, skip_block: int = -1) -> Tensor:
    """Sweep one direction chunk in place with the tiled schedule: the same store as ``sweep_planes``, bit for bit.

    Args:
        index: the tile-diagonal entry tables of the grid.
        store, mu_cells, c: as ``sweep_planes``.
        dirs_per_block: directions of a chunk that one block sweeps through a tile (1 to Dc).
        thread_form: 1 (one view at a time, four blocks per SM) or 2 (the loads of two views before their solves).
        sync, max_blocks, timeout_ns, skip_block: as the persistent launch of ``sweep_planes``.

    Returns:
        The sync words (``sync[2] != 0`` means a barrier wait ran out).
    """
    views, Dc, N, G = _sweep_shape(store, mu_cells, c)
    if index.octant.numel() != 8 * N:
        raise ValueError("the tiled index does not belong to this grid")
    if not 1 <= int(dirs_per_block) <= Dc:
        raise ValueError(f"dirs_per_block must be in [1, {Dc}], got {dirs_per_block}")
    if sync is None:
        sync = torch.empty(4, dtype=torch.int32, device=store.device)
    _lib.call("citrus_sweep_tiled", store.data_ptr(), mu_cells.data_ptr(), c.data_ptr(), index.octant.data_ptr(),
              index.cell.data_ptr(), index.upstream.data_ptr(), index.diagonal_offsets.data_ptr(),
              index.sub_offsets.data_ptr(), index.num_diagonals, index.num_sub, N, G, Dc, views,
              int(dirs_per_block), sync.data_ptr(), int(max_blocks), int(thread_form), int(timeout_ns),
              int(skip_block), _lib.stream_handle(store.device))
    return sync


def _sweep_shape(store: Tensor, mu_cells: Tensor, c: Tensor) -> tuple:
    """(views, Dc, N, G) of a sweep store, after the checks of ``sweep_planes``."""
    if store.dim() == 4:
        views, (_, Dc, N, Q) = 1, store.shape
    elif store.dim() == 5:
        views, _, Dc, N, Q = store.shape
    else:
        raise ValueError(f"store must be [8, Dc, N, 4G] or [V, 8, Dc, N, 4G], got {tuple(store.shape)}")
    if store.shape[-4] != 8 or Q % 4:
        raise ValueError(f"store must be [.., 8, Dc, N, 4G], got {tuple(store.shape)}")
    G = Q // 4
    _check_cuda_f32("store", store)
    _check_cuda_f32("mu_cells", mu_cells)
    _check_cuda_f32("c", c)
    if tuple(mu_cells.shape) != (N, G):
        raise ValueError(f"mu_cells must be [{N}, {G}], got {tuple(mu_cells.shape)}")
    if tuple(c.shape) != (8, Dc, 3):
        raise ValueError(f"c must be [8, {Dc}, 3], got {tuple(c.shape)}")
    return int(views), int(Dc), int(N), int(G)


def sweep_planes(index: FlatPlaneIndex, store: Tensor, mu_cells: Tensor, c: Tensor, *, method: str = "persistent",
                 sync: Optional[Tensor] = None, max_blocks: int = 0,
                 timeout_ns: int = DEFAULT_BARRIER_TIMEOUT_NS, skip_block: int = -1,
                 thread_form: int = 0) -> Optional[Tensor]:
    """Sweep one direction chunk in place (reference ``sweep_kernels.py:265-290``).

    Args:
        index: the plane-sorted entry tables.
        store: [8, Dc, N, 4G] or [V, 8, Dc, N, 4G] float32 contiguous source moments, overwritten with the
            angular-fluence moments (V views sharing ``mu_cells``).
        mu_cells: [N, G] float32 contiguous total attenuation per cell in 1/cm.
        c: [8, Dc, 3] float32 contiguous ``|Omega_a| / Delta_a`` of the chunk directions.
        method: "persistent" (one cooperative launch, grid barrier between planes) or "planes" (one launch per plane).
        sync: [4] int32 device scratch of the persistent launch; allocated when None.
        max_blocks: cap on the persistent grid (0: as many blocks as fit).
        timeout_ns: bound of every barrier wait of the persistent launch.
        skip_block: test hook forcing a barrier timeout (-1 in normal use).
        thread_form: the form of the persistent launch's threads, each of which solves its lane (entry,
            direction, group) in every view: 2 or 4 views loaded before they are solved, or one view at a time with
            registers capped for 5 (1), 6 (3) or 4 (5) blocks per SM (0: 1).

    Returns:
        The sync words of the persistent launch (``sync[2] != 0`` means a barrier wait ran out), or None.
    """
    views, Dc, N, G = _sweep_shape(store, mu_cells, c)
    if index.octant.numel() != 8 * N:
        raise ValueError("the plane index does not belong to this grid")
    stream = _lib.stream_handle(store.device)
    if method == "planes":
        _lib.call("citrus_sweep_planes", store.data_ptr(), mu_cells.data_ptr(), c.data_ptr(), index.octant.data_ptr(),
                  index.cell.data_ptr(), index.upstream.data_ptr(), index.offsets_host.data_ptr(), index.num_planes,
                  N, G, Dc, views, stream)
        return None
    if method != "persistent":
        raise ValueError(f"method must be 'persistent' or 'planes', got {method!r}")
    if sync is None:
        sync = torch.empty(4, dtype=torch.int32, device=store.device)
    _lib.call("citrus_sweep_persistent_config", store.data_ptr(), mu_cells.data_ptr(), c.data_ptr(),
              index.octant.data_ptr(), index.cell.data_ptr(), index.upstream.data_ptr(), index.offsets_device.data_ptr(),
              index.num_planes, N, G, Dc, views, sync.data_ptr(), int(max_blocks), int(thread_form),
              int(timeout_ns), int(skip_block), stream)
    return sync


def sweep_chunk(ctx, store: Tensor, mu_cells: Tensor, c: Tensor, form: SweepForm, **kwargs) -> Optional[Tensor]:
    """Sweep a chunk in the form ``form``: the plane wavefront of ``sweep_planes`` (persistent) or the tiled schedule
    of ``sweep_tiled`` on the context's tables (``ctx.flat_index`` / ``ctx.tiled_index(T)``)."""
    if form.tile > 0:
        return sweep_tiled(ctx.tiled_index(form.tile), store, mu_cells, c, dirs_per_block=min(form.dirs_per_block,
                           int(c.shape[1])), thread_form=form.thread_form, **kwargs)
    return sweep_planes(ctx.flat_index, store, mu_cells, c, method="persistent", thread_form=form.thread_form,
                        **kwargs)


# =====================================================================================================================
# small-K products
# =====================================================================================================================

def source_expansion_first(A: Tensor, B: Tensor, C: Tensor, F: Tensor, precision: str = "fp32",
                           error_word: Optional[Tensor] = None) -> Tensor:
    """``C[b] = A @ B[b]`` plus the LD quadruples ``(F[b], 0, 0, 0)``: the source of an accumulator sweep (the
    expansion ``Y @ T`` of ``transport_sweep.py:524`` added to first-collision moments of one point per cell, given by
    their means) in one pass that writes C without reading it. In "fp32" the float32 CUDA-core product gives the same
    values as writing the quadruples into C and accumulating ``small_k_gemm(A, B, C)`` over them; in "bf16x3" the
    product runs on the tcgen05 tensor cores with the bfloat16 hi/lo split (``small_k_gemm``'s mixed precision) and
    the means are added in its epilogue, 128 rows of A per launch (``error_word`` as in ``small_k_gemm``).

    Args:
        A: [M, K] float32 contiguous, K <= 64.
        B: [batch, K, J] float32 contiguous, J a multiple of 4.
        C: [batch, M, J] float32 contiguous output.
        F: [batch, M, J // 4] float32 contiguous means.
        precision: "fp32" or "bf16x3".
    """
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {PRECISIONS}, got {precision!r}")
    for name, t in (("A", A), ("B", B), ("C", C), ("F", F)):
        _check_cuda_f32(name, t)
    if A.dim() != 2 or B.dim() != 3 or C.dim() != 3 or F.dim() != 3:
        raise ValueError("A must be [M, K], B [batch, K, J], C [batch, M, J], F [batch, M, J / 4]")
    M, K = A.shape
    batch, _, J = B.shape
    if tuple(B.shape) != (batch, K, J) or tuple(C.shape) != (batch, M, J) or tuple(F.shape) != (batch, M, J // 4):
        raise ValueError(f"shapes A {tuple(A.shape)}, B {tuple(B.shape)}, C {tuple(C.shape)}, F {tuple(F.shape)} "
                         "do not chain")
    if J % 4 or K > 64:
        raise ValueError("J must be a multiple of 4 and K at most 64")
    stream = _lib.stream_handle(C.device)
    if precision == "bf16x3":
        err = None if error_word is None else error_word.data_ptr()
        for r0 in range(0, M, 128):
            rows = min(128, M - r0)
            _lib.call("citrus_source_expansion_first_bf16x3", A[r0:].data_ptr(), K, B.data_ptr(), J,
                      C.data_ptr() + 4 * r0 * J, J, F.data_ptr() + 4 * r0 * (J // 4), J // 4, rows, K, J, batch,
                      K * J, M * J, M * (J // 4), err, stream)
        return C
    _lib.call("citrus_source_expansion_first", A.data_ptr(), K, B.data_ptr(), J, C.data_ptr(), J, F.data_ptr(),
              J // 4, M, K, J, batch, K * J, M * J, M * (J // 4), stream)
    return C


PRECISIONS = ("fp32", "bf16x3")


def small_k_gemm(A: Tensor, B: Tensor, C: Tensor, accumulate: bool = False, precision: str = "fp32",
                 error_word: Optional[Tensor] = None, tensor_cores_only: bool = False) -> Tensor:
    """``C (=|+=) A @ B`` for A [M, K] and B, C [.., K or M, J] row-major 2-D (or batched 3-D) views.

    B and C may be strided views whose last axis is contiguous. ``precision`` "fp32" multiplies in float32 on the CUDA
    cores; "bf16x3" runs the tcgen05 tensor-core product, which splits both operands into bfloat16 high and low
    parts and accumulates A_hi B_hi + A_hi B_lo + A_lo B_hi in float32 (``error_word``, an int32 device tensor,
    becomes non-zero if a wait for the tensor cores ran out); ``tensor_cores_only`` only checks that the precision
    asks for it.
    """
    if precision not in PRECISIONS:
        raise ValueError(f"precision must be one of {PRECISIONS}, got {precision!r}")
    _check_cuda_f32("A", A, contiguous=False)
    _check_cuda_f32("B", B, contiguous=False)
    _check_cuda_f32("C", C, contiguous=False)
    if A.dim() != 2 or A.stride(1) != 1:
        raise ValueError("A must be a 2-D row-major matrix")
    if B.dim() == 2:
        B, C = B[None], C[None]
    if B.dim() != 3 or C.dim() != 3 or B.shape[0] != C.shape[0]:
        raise ValueError("B and C must be 2-D matrices or equal batches of them")
    M, K = A.shape
    batch, KB, J = B.shape
    if KB != K or tuple(C.shape) != (batch, M, J):
        raise ValueError(f"shape mismatch: A {tuple(A.shape)}, B {tuple(B.shape)}, C {tuple(C.shape)}")
    if B.stride(2) != 1 or C.stride(2) != 1:
        raise ValueError("B and C need a contiguous last axis")
    sb, sc = (B.stride(0), C.stride(0)) if batch > 1 else (0, 0)
    stream = _lib.stream_handle(A.device)
    err = None if error_word is None else error_word.data_ptr()

    def tensor_cores(out: Tensor, ld_out: int, s_out: int) -> None:
        # at most 128 rows and 128 inner terms per call; inner dimensions above 64 go in steps of 64 (partial sums
        # added), which keeps the split operands of a CTA small enough for three per SM
        step = K if K <= 64 else 64
        for r0 in range(0, M, 128):
            rows = min(128, M - r0)
            for k0 in range(0, K, step):
                inner = min(step, K - k0)
                _lib.call("citrus_small_k_gemm_bf16x3", A[r0:, k0:].data_ptr(), A.stride(0),
                          B[:, k0:].data_ptr(), B.stride(1), out.data_ptr() + 4 * r0 * ld_out, ld_out, rows, inner,
                          J, batch, sb, s_out, int(bool(accumulate) or k0 > 0), err, stream)

    if tensor_cores_only and precision != "bf16x3":
        raise ValueError("tensor_cores_only needs precision='bf16x3'")
    if precision == "bf16x3":   # the mixed precision: every spherical-harmonic product on the tensor cores
        tensor_cores(C, C.stride(1), sc)
        return C
    from .autotune import small_k_gemm_config

    # the kernel: the autotuner's choice for this shape among the float32 forms
    variant, tile = small_k_gemm_config(A, B, C, M, K, J, batch, sb, sc, accumulate)
    _lib.call("citrus_small_k_gemm_config", A.data_ptr(), A.stride(0), B.data_ptr(), B.stride(1), C.data_ptr(),
              C.stride(1), M, K, J, batch, sb, sc, int(bool(accumulate)), int(variant), int(tile), stream)
    return C


# =====================================================================================================================
# scattering moments
# =====================================================================================================================

def cell_major_view(storage: Tensor, num_spatial: int) -> Tensor:
    """The ``[G, N, (4), *spatial]`` view of cell-major storage ``[N, *spatial, G, (4)]``."""
    g = num_spatial + 1
    spatial_axes = list(range(1, num_spatial + 1))
    if storage.dim() == num_spatial + 3:
        return storage.permute(g, 0, g + 1, *spatial_axes)
    return storage.permute(g, 0, *spatial_axes)


def _merged_stride(t: Tensor, first: int) -> Optional[int]:
    sizes, strides = t.shape[first:], t.stride()[first:]
    kept = [(n, s) for n, s in zip(sizes, strides) if n != 1]
    if not kept:
        return 1
    for (n0, s0), (n1, s1) in zip(kept, kept[1:]):
        if s0 != s1 * n1:
            return None
    return kept[-1][1]


def scattering_moments(transfer: Tensor, phi: Tensor, layout: str = "contiguous",
                       out: Optional[Tensor] = None) -> Tensor:
    """Scattering-source moments ``T[g, n] = sum_g' transfer[g', g, l(n)] phi[g', n]`` (reference
    ``scattering_kernels.py:206-252``), in a new tensor of the requested storage.

    Args:
        transfer: [G_in, G_out, L_x+1, *spatial] Legendre transfer moments in 1/cm.
        phi: [G_in, N, *rest] moments, rest = spatial or (4, *spatial), any strides.
        layout: "contiguous" ([G_out, N, *rest]), "moment_major" ([N, G_out, *rest]) or "cell_major"
            ([N, *spatial, G_out, (4)], the sweep's storage).
        out: storage of the requested layout to write into (``[N, *spatial, G_out, (4)]`` for "cell_major"), or
            None to allocate it.

    Returns:
        [G_out, N, *rest] view of the requested storage.
    """
    if layout not in LAYOUTS:
        raise ValueError(f"layout must be one of {LAYOUTS}, got {layout!r}")
    _check_cuda_f32("transfer", transfer, contiguous=False)
    _check_cuda_f32("phi", phi, contiguous=False)
    G_in, G_out, num_legendre = (int(v) for v in transfer.shape[:3])
    spatial = tuple(int(v) for v in transfer.shape[3:])
    N = int(phi.shape[1])
    rest = tuple(int(v) for v in phi.shape[2:])
    if phi.shape[0] != G_in:
        raise ValueError(f"phi has {phi.shape[0]} groups, transfer has {G_in}")
    L = math.isqrt(N) - 1
    if (L + 1) ** 2 != N or L + 1 > num_legendre:
        raise ValueError(f"phi has {N} moments, not (L+1)^2 with L < {num_legendre}")
    has_k = rest != spatial
    if has_k and (len(rest) != len(spatial) + 1 or rest[0] != 4 or rest[1:] != spatial):
        raise ValueError(f"phi trailing shape {rest} must be spatial {spatial} or (4, *spatial)")
    X = math.prod(spatial)
    transfer = transfer.contiguous()
    ps_x = _merged_stride(phi, phi.dim() - len(spatial))
    if ps_x is None:
        phi = phi.contiguous()
        ps_x = 1
    if layout != "cell_major" and out is not None:
        raise ValueError("out is supported for the cell_major layout")
    if layout == "contiguous":
        out = torch.empty((G_out, N) + rest, device=phi.device, dtype=phi.dtype)
    elif layout == "moment_major":
        out = torch.empty((N, G_out) + rest, device=phi.device, dtype=phi.dtype).movedim(0, 1)
    else:
        shape = (N,) + spatial + (G_out,) + ((4,) if has_k else ())
        if out is not None:
            if tuple(out.shape) != shape or not out.is_contiguous() or out.dtype != torch.float32:
                raise ValueError(f"out must be contiguous float32 cell-major storage {shape}")
            storage = out
        else:
            storage = torch.empty(shape, device=phi.device, dtype=phi.dtype)
        out = cell_major_view(storage, len(spatial))
    os_x = _merged_stride(out, out.dim() - len(spatial))
    if X == 0:
        return out
    _lib.call("citrus_scattering_moments", transfer.data_ptr(), phi.data_ptr(), out.data_ptr(), G_in, G_out,
              num_legendre, N, 4 if has_k else 1, X, phi.stride(0), phi.stride(1), phi.stride(2) if has_k else 0,
              ps_x, out.stride(0), out.stride(1), out.stride(2) if has_k else 0, os_x,
              _lib.stream_handle(phi.device))
    return out
