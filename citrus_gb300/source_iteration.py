"""Source iteration over collision order and the scattering source (mirrors
``citrus/scatter_solver/source_iteration.py``).

``scatter_moments`` forms ``T[g, n] = sum_g' mu_s_l[g', g, l(n)] phi[g', n]`` in the sweep's cell-major storage
(``kernels.scattering_moments``), ``scatter_source_function`` expands it at the sweep directions with one small-K
product per chunk (``kernels.small_k_gemm``, written straight into the sweep's store or added to it), and
``source_iteration`` sweeps collision orders until ``||phi_n|| / ||phi_total||`` of the scalar-flux cell means drops
below the tolerance.
"""

from __future__ import annotations

from dataclasses import dataclass, field
from typing import Callable, Optional

import torch
from torch import Tensor

from . import kernels
from .transport_sweep import SweepContext, sweep


@dataclass
class SourceIterationResult:
    """phi_total [G, N_sh, 4, R, C, S], the number of sweeps, the relative changes and norms, the convergence flag
    (reference ``source_iteration.py:28-46``)."""

    phi_total: Tensor
    num_iterations: int
    history: list = field(default_factory=list)
    phi_norms: list = field(default_factory=list)
    converged: bool = False


def scatter_moments(mu_s_l_volume: Tensor, phi: Tensor) -> Tensor:
    """T of ``phi`` as a ``[G_out, N, *rest]`` view of cell-major storage (reference ``source_iteration.py:49-62``)."""
    return kernels.scattering_moments(mu_s_l_volume, phi, "cell_major")


def scatter_source_function(ctx: SweepContext, T: Tensor, precision: str = "fp32"):
    """Source function of the scattering source with moments T (reference ``source_iteration.py:65-106``); the
    expansion ``Y @ T`` runs in ``precision`` (``kernels.small_k_gemm``).

    The callable ``source(direction_index, out=None, accumulate=False)`` returns cell-major
    ``[Dsel, R, C, S, G, 4]`` moments ``sum_n Y[d, n] T[:, n]``, written into (or added to) ``out``.
    """
    if T.shape[1] != ctx.num_moments:
        raise ValueError(f"T has {T.shape[1]} spherical-harmonic moments, context has {ctx.num_moments}")
    if T.dim() != 6 or T.shape[2] != 4 or tuple(T.shape[3:]) != tuple(ctx.shape):
        raise ValueError(f"T must be [G, {ctx.num_moments}, 4, {ctx.shape}], got {tuple(T.shape)}")
    G, num_moments = int(T.shape[0]), int(T.shape[1])
    spatial = tuple(T.shape[3:])
    matrix = T.permute(1, 3, 4, 5, 0, 2).contiguous().view(num_moments, -1)  # no copy for cell-major storage

    def source(direction_index: Tensor, out: Optional[Tensor] = None, accumulate: bool = False) -> Tensor:
        Y_sel = ctx.Y.index_select(0, direction_index.to(ctx.Y.device)).contiguous()
        if out is None:
            out = torch.empty((Y_sel.shape[0],) + spatial + (G, 4), device=T.device, dtype=T.dtype)
            accumulate = False
        kernels.small_k_gemm(Y_sel, matrix, out.view(Y_sel.shape[0], -1), accumulate=accumulate,
                             precision=precision)
        return out

    def with_means(direction_index: Tensor, means: Tensor, out: Tensor) -> Tensor:
        """``out`` = the same expansion plus the LD quadruples ``(means, 0, 0, 0)`` (means ``[Dsel, R, C, S, G]``)
        in one pass that writes ``out`` without reading it (in the moment precision)."""
        Y_sel = ctx.Y.index_select(0, direction_index.to(ctx.Y.device)).contiguous()
        D = Y_sel.shape[0]
        kernels.source_expansion_first(Y_sel, matrix.unsqueeze(0), out.view(1, D, -1), means.reshape(1, D, -1),
                                       precision=precision)
        return out

    source.cell_major = True  # type: ignore[attr-defined]
    source.with_means = with_means if num_moments <= 64 else None  # type: ignore[attr-defined]
    return source


def multiple_collision_source_moments(mu_s_l_volume_coarse: Tensor, phi_total: Tensor) -> Tensor:
    """Cell-mean moments T of the multiple-collision source, a ``[G, N_sh, R, C, S]`` view of cell-major storage
    (reference ``scatter_solver.py:899-910``)."""
    return kernels.scattering_moments(mu_s_l_volume_coarse, phi_total[:, :, 0], "cell_major")


def _scalar_norms(*phis: Tensor) -> list:
    return torch.stack([torch.linalg.vector_norm(phi[:, 0, 0]) for phi in phis]).tolist()


def source_iteration(ctx: SweepContext, mu_t_coarse: Tensor, mu_s_l_volume_coarse: Tensor,
                     first_collision_source_function, tolerance: float, max_iterations: int,
                     direction_chunk: Optional[int] = None,
                     callback: Optional[Callable] = None, precision: str = "fp32") -> SourceIterationResult:
    """Collision-order iteration from the first-collision source (reference ``source_iteration.py:138-204``)."""
    if max_iterations < 1:
        raise ValueError("max_iterations must be >= 1")
    phi_total: Optional[Tensor] = None
    history, norms = [], []
    converged = False
    source_function = first_collision_source_function
    n = 0
    for n in range(1, max_iterations + 1):
        phi_n = sweep(ctx, mu_t_coarse, source_function, direction_chunk=direction_chunk, precision=precision)
        source_function = None
        if phi_total is None:
            phi_total = phi_n.clone()
        else:
            phi_total.add_(phi_n)
        norm_n, norm_total = _scalar_norms(phi_n, phi_total)
        relative = norm_n / norm_total if norm_total > 0 else 0.0
        history.append(relative)
        norms.append(norm_n)
        if callback is not None:
            callback(n, phi_n, relative)
        if relative < tolerance:
            converged = True
            break
        if n == max_iterations:
            break
        source_function = scatter_source_function(ctx, scatter_moments(mu_s_l_volume_coarse, phi_n),
                                                  precision=precision)
        del phi_n
    return SourceIterationResult(phi_total=phi_total, num_iterations=n, history=history, phi_norms=norms,
                                 converged=converged)
