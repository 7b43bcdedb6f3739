"""Oracle of the linear-discontinuous wavefront sweep and of the scattering source, float64 numpy.

Follows citrus/scatter_solver/wavefront.py:75-125 (plan), linear_discontinuous_cell.py:14-87 (cell right-hand sides
and closed-form solve), transport_sweep.py:271-357 (plane step with a zero vacuum cell) and :457-537 (chunks and
moment accumulation), angular_quadrature.py:600-677 (scattering moments) and source_iteration.py:65-204.
"""

from __future__ import annotations

import math

import numpy as np

from citrus_gb300.quadrature import degree_of_moment, real_spherical_harmonics

SIGNS = np.array([[1 if not (o & 4) else -1, 1 if not (o & 2) else -1, 1 if not (o & 1) else -1] for o in range(8)],
                 dtype=np.float64)


def plan(shape):
    """(offsets, octant, cell, upstream) of the 8-octant wavefront order (wavefront.py:75-125); vacuum = -1."""
    R, C, S = shape
    i, j, k = (a.reshape(-1) for a in np.meshgrid(np.arange(R), np.arange(C), np.arange(S), indexing="ij"))
    flat = (i * C + j) * S + k
    rows = []
    for o in range(8):
        sx, sy, sz = SIGNS[o].astype(int)
        plane = (j if sx > 0 else C - 1 - j) + (i if sy > 0 else R - 1 - i) + (k if sz > 0 else S - 1 - k)
        ux = np.where((j - sx >= 0) & (j - sx < C), (i * C + j - sx) * S + k, -1)
        uy = np.where((i - sy >= 0) & (i - sy < R), ((i - sy) * C + j) * S + k, -1)
        uz = np.where((k - sz >= 0) & (k - sz < S), (i * C + j) * S + k - sz, -1)
        rows.append((plane, np.full(flat.size, o), flat, np.stack([ux, uy, uz], 1)))
    plane = np.concatenate([r[0] for r in rows])
    octant = np.concatenate([r[1] for r in rows])
    cell = np.concatenate([r[2] for r in rows])
    upstream = np.concatenate([r[3] for r in rows])
    order = np.argsort(plane * 8 + octant, kind="stable")
    counts = np.bincount(plane, minlength=R + C + S - 2)
    offsets = np.concatenate([[0], np.cumsum(counts)])
    return offsets, octant[order], cell[order], upstream[order]


def cell_solve(c, s, mu, src, X, Y, Z):
    """Closed-form LD solve of one cell (linear_discontinuous_cell.py:14-87).

    c, s: [..., 3]; mu: [...]; src, X, Y, Z: [..., 4] (source and the x, y, z upstream neighbours' moments 0, x, y, z).
    Returns psi [..., 4].
    """
    cx, cy, cz = c[..., 0], c[..., 1], c[..., 2]
    sx, sy, sz = s[..., 0], s[..., 1], s[..., 2]
    pbx = X[..., 0] + sx * X[..., 1]
    pby = Y[..., 0] + sy * Y[..., 2]
    pbz = Z[..., 0] + sz * Z[..., 3]
    r0 = src[..., 0] + cx * pbx + cy * pby + cz * pbz
    rx = src[..., 1] - 3 * sx * cx * pbx + cy * Y[..., 1] + cz * Z[..., 1]
    ry = src[..., 2] - 3 * sy * cy * pby + cx * X[..., 2] + cz * Z[..., 2]
    rz = src[..., 3] - 3 * sz * cz * pbz + cx * X[..., 3] + cy * Y[..., 3]
    csum = cx + cy + cz
    dx, dy, dz = 3 * cx + (csum - cx) + mu, 3 * cy + (csum - cy) + mu, 3 * cz + (csum - cz) + mu
    qx, qy, qz = cx / dx, cy / dy, cz / dz
    den = csum + mu + 3 * (cx * qx + cy * qy + cz * qz)
    p0 = (r0 - (sx * qx * rx + sy * qy * ry + sz * qz * rz)) / den
    return np.stack([p0, (rx + 3 * sx * cx * p0) / dx, (ry + 3 * sy * cy * p0) / dy, (rz + 3 * sz * cz * p0) / dz],
                    axis=-1)


def sweep_chunk(shape, c, mu_cells, source):
    """Sweep one chunk plane by plane (transport_sweep.py:271-357).

    c: [8, Dc, 3] |Omega_a| / Delta_a; mu_cells: [N, G]; source: [8, Dc, N, G, 4]. Returns psi [8, Dc, N, G, 4].
    """
    offsets, octant, cell, upstream = plan(shape)
    N = int(np.prod(shape))
    store = np.zeros((8, c.shape[1], N + 1) + source.shape[3:], dtype=np.float64)
    up = np.where(upstream < 0, N, upstream)
    for p in range(len(offsets) - 1):
        sl = slice(offsets[p], offsets[p + 1])
        o, n, u = octant[sl], cell[sl], up[sl]
        cc = c[o][:, :, None, :]                                    # [E, Dc, 1, 3]
        ss = np.broadcast_to(SIGNS[o][:, None, None, :], cc.shape)  # [E, Dc, 1, 3]
        X = store[o, :, u[:, 0]]                                    # [E, Dc, G, 4]
        Y = store[o, :, u[:, 1]]
        Z = store[o, :, u[:, 2]]
        src = source[o, :, n]
        mu = mu_cells[n][:, None, :]                                # [E, 1, G]
        store[o, :, n] = cell_solve(cc, ss, mu, src, X, Y, Z)
    return store[:, :, :N]


def octant_order(omega):
    """Stable permutation grouping directions by octant (angular_quadrature.py:121-129)."""
    neg = (np.asarray(omega) < 0).astype(np.int64)
    return np.argsort(neg[:, 0] * 4 + neg[:, 1] * 2 + neg[:, 2], kind="stable")


def sweep(shape, deltas, omega, weight, L, mu_t, source, direction_chunk=None):
    """Full sweep (transport_sweep.py:457-537).

    omega, weight: the quadrature in octant-reordered order ([M, 3], [M]); mu_t: [G, R, C, S];
    source: [M, G, 4, R, C, S] (reordered order). Returns (phi [G, N_sh, 4, R, C, S], psi [M, G, 4, R, C, S]).
    """
    omega = np.asarray(omega, dtype=np.float64)
    M = omega.shape[0]
    D8 = M // 8
    G = mu_t.shape[0]
    N = int(np.prod(shape))
    Yw = np.asarray(weight)[:, None] * real_spherical_harmonics(L, omega)    # [M, N_sh]
    c_all = (np.abs(omega) / np.asarray(deltas)).reshape(8, D8, 3)
    mu_cells = mu_t.reshape(G, N).T
    src = source.reshape(8, D8, G, 4, N).transpose(0, 1, 4, 2, 3)            # [8, D8, N, G, 4]
    Dc = D8 if direction_chunk is None else min(D8, int(direction_chunk))
    psi = np.empty((8, D8, N, G, 4))
    for d0 in range(0, D8, Dc):
        d1 = min(d0 + Dc, D8)
        psi[:, d0:d1] = sweep_chunk(shape, c_all[:, d0:d1], mu_cells, src[:, d0:d1])
    psi_m = psi.reshape(M, N, G, 4)
    phi = np.einsum("mn,mcgk->gnkc", Yw, psi_m).reshape(G, Yw.shape[1], 4, *shape)
    return phi, psi_m.transpose(0, 2, 3, 1).reshape(M, G, 4, *shape)


def scatter_moments(transfer, phi):
    """T[g, n, ...] = sum_g' transfer[g', g, l(n), ...] phi[g', n, ...] (angular_quadrature.py:600-677).

    transfer: [G_in, G_out, L+1, *spatial]; phi: [G_in, N, *rest] with rest = spatial or (4, *spatial).
    """
    N = phi.shape[1]
    deg = degree_of_moment(math.isqrt(N) - 1)
    rows = transfer[:, :, deg]                           # [G_in, G_out, N, *spatial]
    if phi.ndim == transfer.ndim:                        # the linear-discontinuous axis
        rows = rows[:, :, :, None]
    return np.einsum("ab...,a...->b...", rows, phi)


def scatter_source(Y_selected, T):
    """Source at directions, sum_n Y[d, n] T[:, n] -> [D, G, *rest] (source_iteration.py:65-106)."""
    return np.einsum("dn,gn...->dg...", Y_selected, T)


def source_iteration(shape, deltas, omega, weight, L, mu_t, transfer, first_source, tolerance, max_iterations):
    """Collision-order iteration (source_iteration.py:138-204). first_source: [M, G, 4, R, C, S]."""
    Y = real_spherical_harmonics(L, omega)
    total = None
    history = []
    source = first_source
    n = 0
    for n in range(1, max_iterations + 1):
        phi_n, _ = sweep(shape, deltas, omega, weight, L, mu_t, source)
        total = phi_n.copy() if total is None else total + phi_n
        norm_n = float(np.linalg.norm(phi_n[:, 0, 0]))
        norm_t = float(np.linalg.norm(total[:, 0, 0]))
        rel = norm_n / norm_t if norm_t > 0 else 0.0
        history.append(rel)
        if rel < tolerance or n == max_iterations:
            break
        source = scatter_source(Y, scatter_moments(transfer, phi_n))
    return total, n, history
