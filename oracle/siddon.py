"""Oracle of the Siddon line integrals and the five ray operations, float64 numpy.

Follows citrus/scatter_solver/ray_tracing.py:141-202 (clip to the box, all plane crossings sorted, segment lengths
times the field at the segment midpoint's voxel) and :405-620 (upstream to voxel centres / points, primary to pixel
centres, downstream to the panel, oblique through pixel centres).
"""

from __future__ import annotations

import math

import numpy as np


def _box(grid):
    lo = np.asarray(grid.lower_corner(), dtype=np.float64)
    delta = np.asarray(grid.deltas, dtype=np.float64)
    n = np.array([grid.num_cols, grid.num_rows, grid.num_slices])
    return lo, lo + delta * n, delta, n


def line_integrals(volume, starts, ends, grid, chunk=4096):
    """[G, R] integrals of volume [G, rows, cols, slices] along starts -> ends ([R, 3]) (ray_tracing.py:141-284)."""
    volume = np.asarray(volume, dtype=np.float64)
    G = volume.shape[0]
    flat = volume.reshape(G, -1).T
    lo, hi, delta, n = _box(grid)
    planes = [lo[a] + delta[a] * np.arange(1, n[a]) for a in range(3)]
    starts = np.asarray(starts, dtype=np.float64).reshape(-1, 3)
    ends = np.asarray(ends, dtype=np.float64).reshape(-1, 3)
    out = np.zeros((G, starts.shape[0]))
    for s in range(0, starts.shape[0], chunk):
        p0, p1 = starts[s:s + chunk], ends[s:s + chunk]
        d = p1 - p0
        nz = d != 0
        inv = 1.0 / np.where(nz, d, 1.0)
        a1, a2 = (lo - p0) * inv, (hi - p0) * inv
        inside = (p0 >= lo) & (p0 <= hi)
        amin = np.where(nz, np.minimum(a1, a2), np.where(inside, -np.inf, np.inf))
        amax = np.where(nz, np.maximum(a1, a2), np.where(inside, np.inf, -np.inf))
        a_lo = np.clip(amin.max(-1), 0.0, None)
        a_hi = np.clip(amax.min(-1), None, 1.0)
        valid = a_hi > a_lo
        a_lo, a_hi = np.where(valid, a_lo, 0.0), np.where(valid, a_hi, 0.0)
        lists = [a_lo[:, None], a_hi[:, None]]
        for a in range(3):
            if planes[a].size == 0:
                continue
            t = (planes[a][None, :] - p0[:, a:a + 1]) * inv[:, a:a + 1]
            t = np.where(nz[:, a:a + 1], t, a_lo[:, None])
            lists.append(np.minimum(np.maximum(t, a_lo[:, None]), a_hi[:, None]))
        alphas = np.sort(np.concatenate(lists, 1), 1)
        seg = alphas[:, 1:] - alphas[:, :-1]
        mid = 0.5 * (alphas[:, 1:] + alphas[:, :-1])
        idx = np.zeros(mid.shape, dtype=np.int64)
        strides = (n[2], n[0] * n[2], 1)
        for a in range(3):
            pos = p0[:, a:a + 1] + mid * d[:, a:a + 1]
            idx += np.clip(np.floor((pos - lo[a]) / delta[a]), 0, n[a] - 1).astype(np.int64) * strides[a]
        length = seg * np.linalg.norm(d, axis=-1, keepdims=True)
        out[:, s:s + chunk] = np.einsum("rpg,rp->gr", flat[idx], length)
    return out


def centers(grid):
    import torch
    x, y, z = grid.axis_coordinates(dtype=torch.float64)
    return np.stack(np.broadcast_arrays(x.double().numpy()[None, :, None], y.double().numpy()[:, None, None],
                                        z.double().numpy()[None, None, :]), -1)


def upstream_to_points(volume, grid, source, points):
    """[G, P] from the focal spot to each point (ray_tracing.py:426-444)."""
    points = np.asarray(points, dtype=np.float64).reshape(-1, 3)
    return line_integrals(volume, np.broadcast_to(np.asarray(source), points.shape), points, grid)


def primary_project(volume, grid, geometry, angle):
    """[G, Rd, Cd] from the focal spot to every pixel centre (ray_tracing.py:447-483)."""
    pixels = geometry.pixel_centers_np(angle)
    tau = upstream_to_points(volume, grid, geometry.source_position(angle), pixels.reshape(-1, 3))
    return tau.reshape(-1, *pixels.shape[:2])


def downstream_cumulative(volume, grid, geometry, angle, omegas):
    """[K, G, R, C, S] from every voxel centre along each direction to the panel (ray_tracing.py:501-545)."""
    volume = np.asarray(volume, dtype=np.float64)
    omegas = np.asarray(omegas, dtype=np.float64).reshape(-1, 3)
    G = volume.shape[0]
    out = np.full((omegas.shape[0], *volume.shape), np.inf)
    n_hat = np.asarray(geometry.panel_axes(angle)[2])
    c = centers(grid).reshape(-1, 3)
    diagonal = math.sqrt(sum(e * e for e in grid.extent)) * (1 + 1e-9) + 1e-9
    for k, w in enumerate(omegas):
        if not (w @ (-n_hat)) > 0:
            continue
        t = np.clip(geometry.panel_distance_along_np(c, w[None, :], angle), 0.0, diagonal)
        out[k] = line_integrals(volume, c, c + t[:, None] * w, grid).reshape(G, *volume.shape[1:])
    return out


def oblique_project(field, grid, geometry, angle, omegas):
    """[K, G, Rd, Cd] through every pixel centre along each direction (ray_tracing.py:572-620)."""
    field = np.asarray(field, dtype=np.float64)
    omegas = np.asarray(omegas, dtype=np.float64).reshape(-1, 3)
    pixels = geometry.pixel_centers_np(angle)
    Rd, Cd = pixels.shape[:2]
    p = pixels.reshape(-1, 3)
    lo = np.asarray(grid.lower_corner())
    center = lo + 0.5 * np.asarray(grid.extent)
    half = 0.5 * math.sqrt(sum(e * e for e in grid.extent)) * (1 + 1e-6) + 1e-6
    out = []
    q = center - p
    for k, w in enumerate(omegas):
        # elementwise, in the reference's order of operations (ray_tracing.py:588-595): the rounding of these
        # endpoints decides whether a line along a face of the box meets it
        w2 = float((w[0] * w[0] + w[1] * w[1]) + w[2] * w[2])
        cp = ((q[:, 0] * w[0] + q[:, 1] * w[1]) + q[:, 2] * w[2]) / w2
        h = half / math.sqrt(w2)
        a = p + (cp - h)[:, None] * w
        b = p + (cp + h)[:, None] * w
        vol = field if field.ndim == 4 else field[k]
        out.append(line_integrals(vol, a, b, grid).reshape(-1, Rd, Cd))
    return np.stack(out)
