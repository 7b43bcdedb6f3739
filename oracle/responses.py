"""Oracle of the anti-scatter-grid transmission and the source model's weights, float64 numpy (test infrastructure).

Follows citrus/scatter_solver/detector.py:1077-1143 (grid angles), :730-756 (trilinear table lookup) and
citrus/scatter_solver/source.py:289-430, 484-510 (field weight, off-focal table, emission profile and filter path
interpolated at the ray's panel point). Every quantity is evaluated directly at each (direction, pixel) or point, with
none of the product's factorisations (per direction, per row, per channel, direction part plus pixel part), so it
checks them. Only tests, the smoke check and the bench's CPU leg import it.
"""

from __future__ import annotations

import math

import numpy as np


def _lerp_index(nodes, x):
    nodes = np.asarray(nodes, dtype=np.float64)
    if nodes.size == 1:
        z = np.zeros(np.shape(x), dtype=np.int64)
        return z, z, np.zeros(np.shape(x))
    xc = np.clip(x, nodes[0], nodes[-1])
    hi = np.clip(np.searchsorted(nodes, xc, side="right"), 1, nodes.size - 1)
    lo = hi - 1
    return lo, hi, np.clip((xc - nodes[lo]) / (nodes[hi] - nodes[lo]), 0.0, 1.0)


def table_value(energy_nodes, theta1_nodes, theta2_nodes, table, group_energy, theta1, theta2):
    """[G, ...] trilinear value of a [E, T1, T2] table at the group energies and |theta1|, |theta2|."""
    e0, e1, we = _lerp_index(energy_nodes, np.asarray(group_energy, dtype=np.float64))
    t = table[e0] + (table[e1] - table[e0]) * we[:, None, None]
    a0, a1, w1 = _lerp_index(theta1_nodes, np.abs(theta1))
    b0, b1, w2 = _lerp_index(theta2_nodes, np.abs(theta2))
    low = t[:, a0, b0] * (1 - w2) + t[:, a0, b1] * w2
    high = t[:, a1, b0] * (1 - w2) + t[:, a1, b1] * w2
    return low * (1 - w1) + high * w1


def local_axes(geometry, angle, points):
    """(u, v, n) at panel points: the panel's own on a flat panel, the cylinder's at each point on a curved one."""
    u, v, n = (np.broadcast_to(np.asarray(a, dtype=np.float64), points.shape) for a in geometry.panel_axes(angle))
    if not geometry.use_curved_detector:
        return u, v, n
    h = np.asarray(geometry.source_position(angle)) - points
    h = h - (h * v).sum(-1, keepdims=True) * v
    n = h / np.sqrt((h * h).sum(-1, keepdims=True))
    return np.cross(n, v), v, n


def grid_angles(omega, pixels, geometry, angle, focal_distance, septa_along):
    """[K, Rd, Cd] theta1 and theta2 of directions [K, 3] arriving at pixels [Rd, Cd, 3] (or [Rd, Cd] for one
    direction per pixel, [Rd, Cd, 3])."""
    f = float(geometry.source_detector_dist) if focal_distance is None else float(focal_distance)
    u, v, n = local_axes(geometry, angle, pixels)
    center = np.asarray(geometry.panel_center(angle))
    if math.isinf(f):
        focus = pixels + n  # any point on the normal: theta_f = 0
    elif not geometry.use_curved_detector:
        focus = np.broadcast_to(center + f * n[0, 0], pixels.shape)
    elif septa_along == "channels":
        focus = pixels - ((pixels - center) * v).sum(-1, keepdims=True) * v + f * n
    else:
        focus = pixels + f * n
    across, along = (v, u) if septa_along == "channels" else (u, v)
    omega = np.asarray(omega, dtype=np.float64)
    a = -omega[:, None, None, :] if omega.ndim == 2 else -omega  # [K, 3] directions, or one per pixel
    an = (a * n).sum(-1)
    to_focus = focus - pixels
    theta_f = np.arctan2((to_focus * across).sum(-1), (to_focus * n).sum(-1))
    theta1 = np.arctan2((a * across).sum(-1), an) - (theta_f[None] if omega.ndim == 2 else theta_f)
    theta2 = np.arctan2((a * along).sum(-1), an)
    return theta1, theta2


def grid_transmission(grid, omega, geometry, angle, group_energy):
    """[K, G, Rd, Cd] transmission of a grid (its crossed septa multiply) for directions at every pixel."""
    pixels = geometry.pixel_centers_np(angle)
    out = 1.0
    for septa in ((grid,) if grid.crossed is None else (grid, grid.crossed)):
        t1, t2 = grid_angles(omega, pixels, geometry, angle, septa.focal_distance_cm, septa.septa_along)
        out = out * table_value(septa.energy_kev, septa.theta1_rad, septa.theta2_rad, septa.transmission,
                                group_energy, t1, t2).transpose(1, 0, 2, 3)
    return out


def _panel_uv(geometry, angle, d):
    """Forward flag and panel coordinates of rays from the focal spot along d [..., 3]."""
    r0 = np.asarray(geometry.source_position(angle))
    u_hat, v_hat, n_hat = (np.asarray(a) for a in geometry.panel_axes(angle))
    if geometry.use_curved_detector:
        horizontal = np.sqrt(d[..., 0] ** 2 + d[..., 1] ** 2)
        with np.errstate(divide="ignore"):
            t = np.where(horizontal > 0, geometry.source_detector_dist / horizontal, np.inf)
    else:
        with np.errstate(divide="ignore", invalid="ignore"):
            t = ((np.asarray(geometry.panel_center(angle)) - r0) @ n_hat) / (d @ n_hat)
    forward = np.isfinite(t) & (t > 0)
    e = np.where(forward, t, 0.0)[..., None] * d
    if geometry.use_curved_detector:
        depth = -(e @ n_hat)
        with np.errstate(divide="ignore", invalid="ignore"):
            return forward, geometry.source_detector_dist * np.arctan2(e @ u_hat, depth), \
                geometry.source_detector_dist * (e @ v_hat) / depth
    hit = r0 + e - np.asarray(geometry.panel_center(angle))
    return forward, hit @ u_hat, hit @ v_hat


def _interpolate(img, geometry, u, v):
    rows, channels = geometry.image_shape
    x = np.clip((u + geometry.det_channel_offset) / geometry.delta_det_channel + (channels - 1) / 2, 0, channels - 1)
    y = np.clip((v + geometry.det_row_offset) / geometry.delta_det_row + (rows - 1) / 2, 0, rows - 1)
    c0 = np.clip(np.floor(x).astype(np.int64), 0, max(channels - 2, 0))
    r0 = np.clip(np.floor(y).astype(np.int64), 0, max(rows - 2, 0))
    c1, r1 = np.minimum(c0 + 1, channels - 1), np.minimum(r0 + 1, rows - 1)
    wc, wr = np.clip(x - c0, 0, 1), np.clip(y - r0, 0, 1)
    img = np.broadcast_to(img, (rows, channels)) if img.shape[0] == 1 else img
    return ((img[r0, c0] * (1 - wc) + img[r0, c1] * wc) * (1 - wr) + (img[r1, c0] * (1 - wc) + img[r1, c1] * wc) * wr)


def source_weight(geometry, angle, d, margins=(0.0, 0.0), off_focal=None, profile=None):
    """b(Omega) of rays from the focal spot along d [..., 3]: field weight (off-focal fraction past the field edge)
    times the emission profile at the panel point."""
    forward, u, v = _panel_uv(geometry, angle, d)
    half_u, half_v = geometry.panel_half_extent()
    pu = np.abs(u + geometry.det_channel_offset) - (half_u + margins[0])
    pv = np.abs(v + geometry.det_row_offset) - (half_v + margins[1])
    inside = (pu <= 0) & (pv <= 0)
    w = inside.astype(np.float64)
    if off_focal is not None:
        nodes, values = (np.asarray(a, dtype=np.float64) for a in off_focal)
        dist = np.hypot(np.maximum(pu, 0.0), np.maximum(pv, 0.0))
        frac = np.interp(dist, nodes, values)  # constant below the first node, as the table's first value
        w = np.where(inside, 1.0, np.where(dist > nodes[-1], 0.0, frac))
    w = np.where(forward, w, 0.0)
    if profile is not None:
        w = w * _interpolate(np.asarray(profile, dtype=np.float64), geometry, u, v)
    return w


def filter_path(geometry, angle, d, thickness, density):
    """rho_f t(Omega) of rays from the focal spot along d [..., 3]."""
    _, u, v = _panel_uv(geometry, angle, d)
    t = np.asarray(thickness, dtype=np.float64)
    return _interpolate(t[None] if t.ndim == 1 else t, geometry, u, v) * float(density)
