"""Oracle of the collapsed-cone scatter image and of the primary, float64 numpy.

Follows citrus/scatter_solver/scatter_image.py:542-696 (panel-facing directions and their weights), :829-874
(attenuated emission at the quadrature points), :897-1135 (finite-cone footprint: box blur with the emission-weighted
mean panel height), :1141-1323 (combined image of the first- and multiple-collision sources) and :1419-1471 (primary
from path lengths).
"""

from __future__ import annotations

import dataclasses

import numpy as np

from citrus_gb300.quadrature import real_spherical_harmonics
from oracle import physics, responses, siddon


def box_matrix(N, w):
    """[k, N, N] overlap matrices (scatter_image.py:952-981)."""
    centers = np.arange(N) + 0.5
    half = 0.5 * np.maximum(np.asarray(w, dtype=np.float64), 1e-3)[:, None]
    lo = np.clip(centers[None] - half, 0.0, N)[..., None]
    hi = np.clip(centers[None] + half, 0.0, N)[..., None]
    j = np.arange(N)[None, None, :]
    return np.clip(np.minimum(hi, j + 1.0) - np.maximum(lo, j), 0.0, None) / (hi - lo)


def direction_weights(omega, weight, geometry, angle, detector, group_energy):
    """Kept directions and (fluence [k], planar [k, 1|Cd], signal [k, G, 1|Cd]) weights (scatter_image.py:542-696),
    for an angle-independent grid of transmission 1."""
    n_hat = np.asarray(geometry.panel_axes(angle)[2])
    keep = (omega.astype(np.float32) * (-n_hat).astype(np.float32)).sum(-1) > 0
    omega, weight = omega[keep], weight[keep]
    cos = (omega * (-n_hat)).sum(-1)
    if geometry.use_curved_detector:
        pixels = geometry.pixel_centers_np(angle)
        normals = geometry.local_normals_np(pixels[0], angle)
        cc = np.clip(omega @ (-normals).T, 0.0, 1.0)
        planar = weight[:, None] * cc
        signal = planar[:, None, :] * detector.at(group_energy, np.arccos(cc)).transpose(1, 0, 2)
    else:
        c = (omega * (-n_hat)).sum(-1) / np.linalg.norm(omega, axis=-1)
        theta = np.arccos(np.clip(c, -1.0, 1.0))
        planar = (weight * cos)[:, None]
        signal = (weight * cos)[:, None, None] * detector.at(group_energy, theta).T[:, :, None]
    return keep, weight, planar, signal


def combined_image(library, rho_q, phi_uc, grid_q, q, T, L, geometry, angle, omega_set, weight_set, cell_width_set,
                   mu_t_coarse, detector, footprint=True, grid=None):
    """fluence, planar, signal_per_group [G, Rd, Cd] and signal [Rd, Cd] of one view (scatter_image.py:1141-1323);
    ``grid`` (a GridResponse) weights the signal with its transmission at every direction and pixel, after the
    footprint blur (scatter_image.py:1281-1313)."""
    keep, w, planar_w, signal_w = direction_weights(omega_set, weight_set, geometry, angle, detector,
                                                    library.group_energy)
    omega, cw = omega_set[keep], cell_width_set[keep]
    f = int(q)
    grid_c = grid_q.coarsen(f)
    G = mu_t_coarse.shape[0]
    Rd, Cd = geometry.image_shape
    tau = siddon.downstream_cumulative(mu_t_coarse, grid_c, geometry, angle, omega)         # [k, G, Rc, Cc, Sc]
    Y = real_spherical_harmonics(L, omega)
    S_mc = np.einsum("kn,gn...->kg...", Y, T)                                               # [k, G, Rc, Cc, Sc]
    S_fc = physics.first_collision_source(library, rho_q, phi_uc, grid_q, geometry, angle, omega)
    k = omega.shape[0]
    Rc, Cc, Sc = grid_c.shape
    total = S_fc.reshape(k, G, Rc, f, Cc, f, Sc, f) + S_mc[:, :, :, None, :, None, :, None]
    dx, dy, dz = grid_q.deltas
    ci = np.arange(f) - (f - 1) / 2.0
    off = (omega[:, 1, None, None, None] * (dy * ci)[None, :, None, None]
           + omega[:, 0, None, None, None] * (dx * ci)[None, None, :, None]
           + omega[:, 2, None, None, None] * (dz * ci)[None, None, None, :])[:, None, None, :, None, :, None, :]
    mu_c = mu_t_coarse[None, :, :, None, :, None, :, None]
    depth = np.clip(tau[:, :, :, None, :, None, :, None] - mu_c * off, 0.0, None)
    emission = (total * np.exp(-depth)).reshape(k, G, *grid_q.shape)
    image = siddon.oblique_project(emission, grid_q, geometry, angle, omega)                # [k, G, Rd, Cd]
    if footprint:
        n_hat = np.asarray(geometry.panel_axes(angle)[2])
        pc = np.asarray(geometry.panel_center(angle))
        h = ((siddon.centers(grid_q) - pc) @ n_hat).reshape(-1)
        tot = emission.sum(1).reshape(k, -1)
        lower, extent = grid_q.lower_corner(), grid_q.extent
        corner = [sum((lower[a] + c[a] * extent[a] - pc[a]) * n_hat[a] for a in range(3))
                  for c in [(i, j, kk) for i in (0, 1) for j in (0, 1) for kk in (0, 1)]]
        den = tot.sum(-1)
        hbar = np.where(den > 0, (tot @ h) / np.where(den > 0, den, 1.0), 0.5 * (min(corner) + max(corner)))
        wc = hbar * cw[:, 0] / geometry.delta_det_channel
        wr = hbar * cw[:, 1] / geometry.delta_det_row
        image = np.einsum("kcj,kgrj->kgrc", box_matrix(Cd, wc), image)
        image = np.einsum("krj,kgjc->kgrc", box_matrix(Rd, wr), image)
    fluence = np.einsum("kgrc,k->grc", image, w)
    planar = np.einsum("kgrc,kc->grc", image, np.broadcast_to(planar_w, (k, Cd)))
    signal = np.broadcast_to(signal_w, (k, G, Cd))[:, :, None, :]
    if grid is not None:
        signal = signal * responses.grid_transmission(grid, omega, geometry, angle, library.group_energy)
    signal_pg = np.einsum("kgrc,kgrc->grc", image, np.broadcast_to(signal, image.shape))
    return {"fluence": fluence, "planar_fluence": planar, "signal_per_group": signal_pg, "signal": signal_pg.sum(0)}


def primary(library, rho, grid, geometry, angle, detector):
    """Primary image (scatter_image.py:1419-1471) with an angle-independent unit grid transmission."""
    path = siddon.primary_project(rho, grid, geometry, angle)
    T = physics.group_transmission(library, path)
    pixels = geometry.pixel_centers_np(angle)
    d = pixels - np.asarray(geometry.source_position(angle))
    dist2 = (d * d).sum(-1)
    b = physics.source_weight(geometry, angle, pixels)
    fluence = (b / dist2)[None] * T
    omega_p = d / np.sqrt(dist2)[..., None]
    n = geometry.local_normals_np(pixels, angle)
    theta0 = np.arccos(np.clip((omega_p * (-n)).sum(-1), -1.0, 1.0))
    planar = fluence * np.cos(theta0)
    signal_pg = planar * detector.at(library.group_energy, theta0)
    return {"fluence": fluence, "planar_fluence": planar, "signal_per_group": signal_pg, "signal": signal_pg.sum(0)}


def primary_with_source(library, rho, grid, geometry, angle, detector, n=1, grid_response=None, margins=(0.0, 0.0),
                        off_focal=None, profile=None, thickness=None, filter_density=0.0, filter_mu=None):
    """Primary signal [Rd, Cd] with sub-pixel rays, the source model and an anti-scatter grid
    (scatter_image.py:1395-1471): the fine-energy transmission, the beam filter's path included, averaged over the
    n x n sub-pixels of every pixel; the source weight, the inverse square, the detector response and the grid
    transmission (each set of septa at its own grid angles) at the pixel centres."""
    fine = geometry if n == 1 else dataclasses.replace(
        geometry, num_det_rows=geometry.num_det_rows * n, num_det_channels=geometry.num_det_channels * n,
        delta_det_row=geometry.delta_det_row / n, delta_det_channel=geometry.delta_det_channel / n)
    r0 = np.asarray(geometry.source_position(angle))
    path = siddon.primary_project(rho, grid, fine, angle)                       # [M, Rd n, Cd n]
    tau = np.einsum("me,mrc->erc", library.fine_mu_t, path)
    if thickness is not None:
        fp = responses.filter_path(geometry, angle, fine.pixel_centers_np(angle) - r0, thickness, filter_density)
        tau = tau + np.asarray(filter_mu)[:, None, None] * fp[None]
    W = (library.fine_group[None, :] == np.arange(library.num_groups)[:, None]) * library.fine_weight[None, :]
    T = np.einsum("ge,erc->grc", W, np.exp(-tau))
    Rd, Cd = geometry.image_shape
    T = T.reshape(-1, Rd, n, Cd, n).mean(axis=(2, 4))
    pixels = geometry.pixel_centers_np(angle)
    d = pixels - r0
    dist2 = (d * d).sum(-1)
    b = responses.source_weight(geometry, angle, d, margins, off_focal, profile)
    omega_p = d / np.sqrt(dist2)[..., None]
    normal = geometry.local_normals_np(pixels, angle)
    theta0 = np.arccos(np.clip((omega_p * (-normal)).sum(-1), -1.0, 1.0))
    signal = (b / dist2 * np.cos(theta0))[None] * T * detector.at(library.group_energy, theta0)
    if grid_response is not None:
        for septa in ((grid_response,) if grid_response.crossed is None
                      else (grid_response, grid_response.crossed)):
            t1, t2 = responses.grid_angles(omega_p, pixels, geometry, angle, septa.focal_distance_cm,
                                           septa.septa_along)
            signal = signal * responses.table_value(septa.energy_kev, septa.theta1_rad, septa.theta2_rad,
                                                    septa.transmission, library.group_energy, t1, t2)
    return signal.sum(0)

