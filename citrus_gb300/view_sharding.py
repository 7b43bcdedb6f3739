"""Views of one outer iteration sharded over ranks, one process per GPU.

Within an outer iteration the views are independent given the shared read-only material fields (the reference loops
over them, ``citrus/citrus.py:1914-1935``), so each rank owns a round-robin share of the views and their accumulator
states, computes its views' scatter signals, and one all-gather per outer iteration assembles the ``[V, Rd, Cd]``
signals on every rank. There is no other data-path exchange. The same code runs over NCCL on GPUs and over gloo on CPU
ranks (the tests).
"""

from __future__ import annotations

from typing import Callable, Sequence

import torch
import torch.distributed as dist


def owned_views(num_views: int, rank: int, world_size: int) -> list:
    """Round-robin share of a rank: views rank, rank + W, rank + 2W, ..."""
    if not 0 <= rank < world_size:
        raise ValueError(f"rank {rank} outside [0, {world_size})")
    return list(range(rank, num_views, world_size))


def gather_signals(local: torch.Tensor, num_views: int, group=None) -> torch.Tensor:
    """All-gather the per-rank signals [n_local, Rd, Cd] into [V, Rd, Cd] in view order.

    Every rank pads its share to ceil(V / W) views so the collective moves equal blocks; padding is dropped.
    """
    world = dist.get_world_size(group)
    per_rank = -(-num_views // world)
    Rd, Cd = local.shape[1:]
    padded = torch.zeros(per_rank, Rd, Cd, dtype=local.dtype, device=local.device)
    padded[:local.shape[0]] = local
    blocks = [torch.empty_like(padded) for _ in range(world)]
    dist.all_gather(blocks, padded, group=group)
    out = torch.empty(num_views, Rd, Cd, dtype=local.dtype, device=local.device)
    for r in range(world):
        views = owned_views(num_views, r, world)
        out[views] = blocks[r][:len(views)]
    return out


def sharded_scatter_stage(view_step: Callable[[int, float], torch.Tensor], angles: Sequence[float],
                          image_shape: Sequence[int], device=None, group=None) -> torch.Tensor:
    """Run ``view_step(view_index, angle) -> [Rd, Cd]`` on this rank's views and all-gather every view's signal.

    ``image_shape`` is the panel's (Rd, Cd) and ``device`` the device of the signals (the collective's): a rank
    that owns no view (more ranks than views) joins the all-gather with an empty block of that shape."""
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    mine = owned_views(len(angles), rank, world)
    Rd, Cd = (int(n) for n in image_shape)
    if mine:
        local = torch.stack([view_step(v, float(angles[v])) for v in mine])
        if tuple(local.shape[1:]) != (Rd, Cd):
            raise ValueError(f"view_step returned [{tuple(local.shape[1:])}], expected the panel's [{Rd}, {Cd}]")
    else:
        local = torch.zeros(0, Rd, Cd, device=device)
    return gather_signals(local, len(angles), group)
