"""Detector and anti-scatter-grid responses and the source model of the scatter step.

Mirrors the lookup parts of ``citrus/scatter_solver/detector.py`` and ``source.py`` that the per-view step evaluates:
``DetectorResponse.at`` (bilinear in energy and angle, ``detector.py:197-241``), ``GridResponse`` with the
angle-independent ``no_grid`` table (``detector.py:657-766``), ``detector_angle`` (``:1054-1074``) and the collimated
isotropic point source (``source.py:58-382``: unit emission where the ray from the focal spot meets the field on the
panel). These are host-side float64 tables; the per-pixel and per-direction weights built from them are uploaded once
per view.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .geometry import ConeGeometry


def _bracket(nodes: np.ndarray, x: np.ndarray):
    n = nodes.size
    if n == 1:
        z = np.zeros(np.shape(x), dtype=np.int64)
        return z, z, np.zeros(np.shape(x))
    xc = np.clip(x, nodes[0], nodes[-1])
    i1 = np.clip(np.searchsorted(nodes, xc, side="right"), 1, n - 1)
    i0 = i1 - 1
    w1 = np.clip((xc - nodes[i0]) / (nodes[i1] - nodes[i0]), 0.0, 1.0)
    return i0, i1, w1


@dataclass(frozen=True, eq=False)
class DetectorResponse:
    """D(E, theta0) in keV per incident photon; bilinear, clamped, |theta| used (reference ``detector.py:197-241``)."""

    energy_kev: np.ndarray
    theta_rad: np.ndarray
    response: np.ndarray
    name: str = "detector"

    def at(self, group_energy, theta) -> np.ndarray:
        e = np.asarray(group_energy, dtype=np.float64).reshape(-1)
        ie0, ie1, we = _bracket(self.energy_kev, e)
        it0, it1, wt = _bracket(self.theta_rad, np.abs(np.asarray(theta, dtype=np.float64)))
        table = self.response[ie0] + (self.response[ie1] - self.response[ie0]) * we[:, None]
        a, b = table[:, it0], table[:, it1]
        return a + (b - a) * wt


def ideal_counting_response() -> DetectorResponse:
    """D = 1 per photon: the signal is the photon fluence (reference ``detector.py:294-302``)."""
    return DetectorResponse(np.array([1.0, 1000.0]), np.array([0.0, math.pi / 2]), np.ones((2, 2)), "ideal counting")


def energy_weighted_response() -> DetectorResponse:
    """D = E per photon in keV (reference ``detector.py:305-315``)."""
    e = np.array([1.0, 1000.0])
    return DetectorResponse(e, np.array([0.0, math.pi / 2]), np.repeat(e[:, None], 2, 1), "ideal energy weighted")


@dataclass(frozen=True, eq=False)
class GridResponse:
    """Anti-scatter-grid transmission G(E, theta1, theta2) (reference ``detector.py:657-756``). Only tables that do not
    depend on the angles are evaluated on this path (``no_grid``); the septa geometry is out of scope."""

    energy_kev: np.ndarray
    theta1_rad: np.ndarray
    theta2_rad: np.ndarray
    transmission: np.ndarray
    name: str = "grid"

    @property
    def depends_on_angles(self) -> bool:
        t = self.transmission
        return not bool(np.all(t == t[:, :1, :1]))

    def at_energy(self, group_energy) -> np.ndarray:
        """[G] transmission of an angle-independent table."""
        if self.depends_on_angles:
            raise NotImplementedError("angle-dependent anti-scatter grids are not supported on this path")
        e = np.asarray(group_energy, dtype=np.float64).reshape(-1)
        i0, i1, w = _bracket(self.energy_kev, e)
        col = self.transmission[:, 0, 0]
        return col[i0] + (col[i1] - col[i0]) * w


def no_grid() -> GridResponse:
    """Transmission 1 everywhere (reference ``detector.py:758-766``)."""
    e = np.array([1.0, 1000.0])
    t = np.array([0.0, math.pi / 2])
    return GridResponse(e, t, t.copy(), np.ones((2, 2, 2)), "no grid")


def detector_angle(omega: np.ndarray, geometry: ConeGeometry, angle: float, pixel_positions=None) -> np.ndarray:
    """Angle between photon directions and the inward panel normal (local normal on a curved panel when pixel
    positions are given) (reference ``detector.py:1054-1074``)."""
    omega = np.asarray(omega, dtype=np.float64)
    n = np.asarray(geometry.panel_axes(angle)[2])
    if geometry.use_curved_detector and pixel_positions is not None:
        n = geometry.local_normals_np(pixel_positions, angle)
    c = (omega * (-n)).sum(-1) / np.linalg.norm(omega, axis=-1)
    return np.arccos(np.clip(c, -1.0, 1.0))


@dataclass(frozen=True)
class SourceModel:
    """Isotropic point source collimated to the panel plus field margins (reference ``source.py:58-382``, without an
    emission profile, off-focal table or beam filter)."""

    field_margin_channels_cm: float = 0.0
    field_margin_rows_cm: float = 0.0

    def field_args(self, geometry: ConeGeometry, angle: float) -> list:
        """The 23 doubles of ``citrus_source_weight``."""
        u_hat, v_hat, n_hat = geometry.panel_axes(angle)
        half_u, half_v = geometry.panel_half_extent()
        return [1.0 if geometry.use_curved_detector else 0.0, *geometry.source_position(angle),
                *geometry.panel_center(angle), *u_hat, *v_hat, *n_hat, float(geometry.source_detector_dist),
                float(geometry.det_channel_offset), float(geometry.det_row_offset), half_u, half_v,
                float(self.field_margin_channels_cm), float(self.field_margin_rows_cm)]

    def angular_weight_np(self, directions: np.ndarray, geometry: ConeGeometry, angle: float) -> np.ndarray:
        """b(Omega) at float64 directions from the focal spot (host; for pixels and tests)."""
        d = np.asarray(directions, dtype=np.float64)
        src = np.asarray(geometry.source_position(angle))
        t = geometry.panel_distance_along_np(np.broadcast_to(src, d.shape), d, angle)
        forward = np.isfinite(t) & (t > 0)
        hit = src + np.where(forward, t, 0.0)[..., None] * d
        u, v = geometry.panel_uv_of_points_np(hit, angle)
        half_u, half_v = geometry.panel_half_extent()
        inside = ((np.abs(u + geometry.det_channel_offset) <= half_u + self.field_margin_channels_cm)
                  & (np.abs(v + geometry.det_row_offset) <= half_v + self.field_margin_rows_cm))
        return (forward & inside).astype(np.float64)
