"""The plane-wavefront and tile-diagonal plans of the sweep (host tables, no GPU): every (octant, cell) entry once,
and every upstream neighbour of an entry earlier in its schedule."""

from __future__ import annotations

import numpy as np
import pytest

from citrus_gb300.transport_sweep import build_sweep_plan, build_tiled_plan


@pytest.mark.parametrize("shape, tile", [((5, 7, 6), 2), ((8, 8, 8), 4), ((9, 8, 17), 8), ((6, 5, 7), 3),
                                         ((3, 1, 4), 5), ((16, 16, 16), 8)])
def test_tiled_plan_orders_every_upstream_neighbour_first(shape, tile):
    p = build_tiled_plan(shape, tile)
    q = build_sweep_plan(shape)
    N = int(np.prod(shape))
    assert p.num_sub == 3 * tile - 2
    assert p.sub_offsets[0, 0] == 0 and p.sub_offsets[-1, -1] == 8 * N
    assert np.all(p.sub_offsets[1:, 0] == p.sub_offsets[:-1, -1]) and np.all(np.diff(p.sub_offsets, axis=1) >= 0)
    assert p.diagonal_offsets[0] == 0 and p.diagonal_offsets[-1] == p.num_tasks
    # the same entries as the plane plan, each once
    a = np.sort(p.octant * N + p.cell)
    np.testing.assert_array_equal(a, np.sort(q.octant * N + q.cell))
    np.testing.assert_array_equal(a, np.arange(8 * N))
    # every entry's upstream neighbour: the previous sub-plane of its task, or a task on an earlier diagonal
    task = np.repeat(np.arange(p.num_tasks), np.diff(p.sub_offsets[:, [0, -1]], axis=1).ravel())
    sub = np.concatenate([np.repeat(np.arange(p.num_sub), np.diff(row)) for row in p.sub_offsets])
    diag = np.repeat(np.arange(p.num_diagonals), np.diff(p.diagonal_offsets))[task]
    pos = np.empty((8, N), dtype=np.int64)
    pos[p.octant, p.cell] = np.arange(8 * N)
    for axis in range(3):
        up = p.upstream[:, axis]
        has = up >= 0
        me = np.nonzero(has)[0]
        src = pos[p.octant[has], up[has]]
        same = task[src] == task[me]
        assert np.all(np.where(same, sub[src] == sub[me] - 1, diag[src] < diag[me]))
    # the upstream tables agree with the plane plan's, entry by entry
    order = np.argsort(q.octant * N + q.cell)
    mine = np.argsort(p.octant * N + p.cell)
    np.testing.assert_array_equal(p.upstream[mine], q.upstream[order])


def test_tiled_plan_rejects_a_bad_tile():
    with pytest.raises(ValueError):
        build_tiled_plan((4, 4, 4), 0)
