"""Oracle of the uncollided fluence and the first-collision source, float64 numpy.

Follows citrus/scatter_solver/uncollided.py:74-349 (primary directions, uncollided fluence from path lengths, the
first-collision source, restriction to LD moments), :357-461 and :538-636 (exact moments, quadrature sums, correction
factors), cross_sections.py:797-883 (group transmission), :905-995 (eta-table interpolation) and source.py:289-382
(focal-spot weight); the source model's off-focal table, emission profile and beam filter through
``oracle/responses.py``.
"""

from __future__ import annotations

import numpy as np

from oracle import responses
from oracle.siddon import centers, upstream_to_points


def primary_directions(grid, geometry, angle):
    """[R, C, S, 3] unit vectors from the focal spot to the point centres."""
    d = centers(grid) - np.asarray(geometry.source_position(angle))
    return d / np.linalg.norm(d, axis=-1, keepdims=True)


def source_weight(geometry, angle, points, margins=(0.0, 0.0)):
    """b(Omega): 1 where the ray from the focal spot through a point meets the collimated field (source.py:289-382)."""
    src = np.asarray(geometry.source_position(angle))
    d = np.asarray(points, dtype=np.float64) - src
    t = geometry.panel_distance_along_np(np.broadcast_to(src, d.shape), d, angle)
    forward = np.isfinite(t) & (t > 0)
    hit = src + np.where(forward, t, 0.0)[..., None] * d
    u, v = geometry.panel_uv_of_points_np(hit, angle)
    hu, hv = geometry.panel_half_extent()
    inside = ((np.abs(u + geometry.det_channel_offset) <= hu + margins[0])
              & (np.abs(v + geometry.det_row_offset) <= hv + margins[1]))
    return (forward & inside).astype(np.float64)


def group_transmission(library, path, materials=None):
    """[G, ...] sum_{e in g} w_e exp(-sum_m mu_m(e) P_m) (cross_sections.py:831-883)."""
    mu = library.fine_mu_t if materials is None else library.fine_mu_t[list(materials)]
    spatial = path.shape[1:]
    tau = np.einsum("me,mp->ep", mu, path.reshape(path.shape[0], -1))
    W = (library.fine_group[None, :] == np.arange(library.num_groups)[:, None]) * library.fine_weight[None, :]
    return (W @ np.exp(-tau)).reshape(library.num_groups, *spatial)


def uncollided_fluence(library, rho, grid, geometry, angle, points=None):
    """[G, *points.shape] (uncollided.py:99-197), all materials traced."""
    pg = grid if points is None else points
    c = centers(pg)
    path = upstream_to_points(rho, grid, geometry.source_position(angle), c.reshape(-1, 3))
    T = group_transmission(library, path)
    d = c - np.asarray(geometry.source_position(angle))
    b = source_weight(geometry, angle, c)
    return T.reshape(-1, *pg.shape) * (b / (d * d).sum(-1))[None]


def uncollided_fluence_with_source(library, rho, grid, geometry, angle, margins=(0.0, 0.0), off_focal=None,
                                   profile=None, thickness=None, filter_density=0.0, filter_mu=None):
    """[G, *grid.shape] uncollided fluence of a source with field margins, an off-focal table, an emission profile
    and a beam filter (uncollided.py:160-197 with source.py:289-430): the filter's path adds filter_mu[e] times it to
    every exponent."""
    c = centers(grid)
    r0 = np.asarray(geometry.source_position(angle))
    d = c - r0
    path = upstream_to_points(rho, grid, geometry.source_position(angle), c.reshape(-1, 3))
    tau = np.einsum("me,mp->ep", library.fine_mu_t, path.reshape(path.shape[0], -1))
    if thickness is not None:
        fp = responses.filter_path(geometry, angle, d.reshape(-1, 3), thickness, filter_density)
        tau = tau + np.asarray(filter_mu)[:, None] * fp[None]
    W = (library.fine_group[None, :] == np.arange(library.num_groups)[:, None]) * library.fine_weight[None, :]
    T = (W @ np.exp(-tau)).reshape(-1, *grid.shape)
    b = responses.source_weight(geometry, angle, d, margins, off_focal, profile)
    return T * (b / (d * d).sum(-1))[None]


def transfer_at(library, rho, eta):
    """[G_in, G_out, ...] per-steradian transfer at cosines eta [...] of densities rho [M, ...]
    (cross_sections.py:905-995, uniform table)."""
    N = library.mu_s_eta.shape[-1]
    eta = np.clip(eta, -1.0, 1.0)
    pos = (eta + 1.0) / 2.0 * (N - 1)
    i0 = np.clip(np.floor(pos).astype(np.int64), 0, N - 2)
    w1 = np.clip(pos - i0, 0.0, 1.0)
    t = library.mu_s_eta                                   # [M, Gi, Go, N]
    v = t[..., i0] + (t[..., i0 + 1] - t[..., i0]) * w1    # [M, Gi, Go, ...]
    return np.einsum("mab...,m...->ab...", v, rho)


def first_collision_source(library, rho, phi_uc, grid, geometry, angle, omegas):
    """[K, G, R, C, S] (uncollided.py:236-271): downscatter only."""
    u = primary_directions(grid, geometry, angle)
    G = phi_uc.shape[0]
    down = np.triu(np.ones((G, G)))
    out = []
    for w in np.asarray(omegas, dtype=np.float64).reshape(-1, 3):
        T = transfer_at(library, rho, u @ w)
        out.append(np.einsum("ab...,ab,a...->b...", T, down, phi_uc))
    return np.stack(out)


def correction(library, rho, phi_uc, grid, geometry, angle, omegas, weights):
    """(scale, beta, I [3, G, ...], E [2, G, ...]) of the sampling correction (uncollided.py:357-461, 538-636)."""
    u = primary_directions(grid, geometry, angle)
    S = first_collision_source(library, rho, phi_uc, grid, geometry, angle, omegas)
    mu = np.einsum("rcsx,kx->krcs", u, np.asarray(omegas, dtype=np.float64).reshape(-1, 3))[:, None]
    w = np.asarray(weights, dtype=np.float64).reshape(-1, 1, 1, 1, 1)
    I = np.stack([(w * S).sum(0), (w * mu * S).sum(0), (w * mu * mu * S).sum(0)])
    G = phi_uc.shape[0]
    E = np.einsum("mabl,ab,m...,a...->lb...", library.mu_s_l[..., :2], np.triu(np.ones((G, G))), rho, phi_uc)
    I0, I1, I2 = I
    E0, E1 = E
    pos = E0 > 0
    c = np.where(pos, E1 / np.where(pos, E0, 1.0), 0.0)
    den = I2 - c * I1
    ok = pos & (np.abs(den) > 1e-12 * np.abs(I0))
    beta = np.clip(np.where(ok, (c * I0 - I1) / np.where(ok, den, 1.0), 0.0), -1.0, 1.0)
    d0 = I0 + beta * I1
    scale = np.where(d0 > 0, E0 / np.where(d0 > 0, d0, 1.0), 1.0)
    return scale, beta, I, E


def restrict_ld(field, f):
    """[..., 4, R/f, C/f, S/f] LD moments (mean, x, y, z slopes) of a refined field (uncollided.py:311-349)."""
    lead = field.shape[:-3]
    R, C, S = (n // f for n in field.shape[-3:])
    x = field.reshape(*lead, R, f, C, f, S, f)
    nl = len(lead)
    ar, ac, asl = nl + 1, nl + 3, nl + 5
    mean = x.mean(axis=(ar, ac, asl))
    if f == 1:
        z = np.zeros_like(mean)
        return np.stack([mean, z, z, z], axis=-4)
    u = (2 * np.arange(f) + 1) / f - 1
    scale = 1.0 / (u * u).mean()

    def slope(axis):
        shape = [1] * x.ndim
        shape[axis] = f
        return (x * u.reshape(shape)).mean(axis=(ar, ac, asl)) * scale

    return np.stack([mean, slope(ac), slope(ar), slope(asl)], axis=-4)


def first_collision_moments(library, rho, phi_uc, grid, geometry, angle, omegas, scale, beta, f):
    """[K, G, 4, Rc, Cc, Sc] LD moments of the corrected source (uncollided.py:464-511)."""
    S = first_collision_source(library, rho, phi_uc, grid, geometry, angle, omegas)
    u = primary_directions(grid, geometry, angle)
    eta = np.einsum("rcsx,kx->krcs", u, np.asarray(omegas, dtype=np.float64).reshape(-1, 3))
    return restrict_ld(S * scale * (1.0 + beta[None] * eta[:, None]), f)
