"""Detector and anti-scatter-grid responses and the source model of the scatter step.

Mirrors the parts of ``citrus/scatter_solver/detector.py`` and ``source.py`` that the per-view step evaluates:
``DetectorResponse.at`` (bilinear in energy and angle, ``detector.py:197-241``); ``GridResponse`` (trilinear in the
energy and the grid angles, septa along the channels or the rows, focused or not, crossed septa,
``detector.py:655-766``) with ``grid_angles`` (``:1077-1143``), the focused 1-D grid's septum-shadow table
(``:778-836``) and the classification of how a set of septa varies over the panel (``scatter_image.py:506-539``);
``detector_angle`` (``:1054-1074``); and the source (``source.py:58-533``): the collimated field with its margins, the
off-focal table, the emission profile and the beam filter. These are host-side float64 tables and host evaluations
for pixels and tests; the weights of the image path are built from them once per view, and the device evaluates
the per-point source weights (``citrus_source_field``) and the per-pixel grid transmissions
(``citrus_grid_signal_sum``). Photon data (the reference's XCOM tables) is not part of this package: a grid's septum
material and a filter's attenuation come in as callables.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field, replace
from typing import Callable, Optional

import numpy as np
import torch

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


SEPTA_DIRECTIONS = ("channels", "rows")
LEAD_DENSITY = 11.35  # g/cm^3


def _as_f64(x) -> np.ndarray:
    if isinstance(x, torch.Tensor):
        x = x.detach().cpu().numpy()
    return np.asarray(x, dtype=np.float64)


@dataclass(frozen=True, eq=False)
class GridResponse:
    """Anti-scatter-grid transmission G(E, theta1, theta2) at the grid angles of :func:`grid_angles` (reference
    ``detector.py:655-756``): trilinear in the energy and the absolute grid angles, clamped to the end nodes, for septa
    running along the channels or the rows, focused on a line at ``focal_distance_cm`` from the panel (None: the
    geometry's default, :func:`default_focal_distance`; ``math.inf``: unfocused), with an optional second set of septa
    in the other direction (``crossed``) whose transmission multiplies. Tables are float64 host arrays."""

    energy_kev: np.ndarray
    theta1_rad: np.ndarray
    theta2_rad: np.ndarray
    transmission: np.ndarray
    focal_distance_cm: Optional[float] = None
    name: str = "grid"
    septa_along: str = "channels"
    crossed: Optional["GridResponse"] = None

    def __post_init__(self):
        for k in ("energy_kev", "theta1_rad", "theta2_rad"):
            object.__setattr__(self, k, _as_f64(getattr(self, k)).reshape(-1))
        object.__setattr__(self, "transmission", _as_f64(self.transmission))
        shape = (self.energy_kev.size, self.theta1_rad.size, self.theta2_rad.size)
        if self.transmission.shape != shape:
            raise ValueError(f"transmission must be [E, T1, T2] = {list(shape)}, got {self.transmission.shape}")
        if self.septa_along not in SEPTA_DIRECTIONS:
            raise ValueError(f"septa_along must be one of {SEPTA_DIRECTIONS}, got {self.septa_along!r}")
        if self.crossed is not None and (self.crossed.septa_along == self.septa_along
                                         or self.crossed.crossed is not None):
            raise ValueError("the crossed septa must run in the other direction and have no crossed septa of their own")

    @property
    def depends_on_angles(self) -> bool:
        t = self.transmission
        return self.crossed is not None or not bool(np.all(t == t[:, :1, :1]))

    def table_at_energy(self, group_energy) -> np.ndarray:
        """[G, T1, T2] the table interpolated to the group energies (the first of the three linear steps)."""
        e = _as_f64(group_energy).reshape(-1)
        i0, i1, w = _bracket(self.energy_kev, e)
        t = self.transmission
        return t[i0] + (t[i1] - t[i0]) * w[:, None, None]

    def at(self, group_energy, theta1, theta2) -> np.ndarray:
        """[G, ...] transmission at the grid angles (broadcast), trilinear in (E, |theta1|, |theta2|)."""
        theta1, theta2 = np.broadcast_arrays(_as_f64(theta1), _as_f64(theta2))
        table = self.table_at_energy(group_energy)                                   # [G, T1, T2]
        i10, i11, w1 = _bracket(self.theta1_rad, np.abs(theta1))
        i20, i21, w2 = _bracket(self.theta2_rad, np.abs(theta2))
        a0 = table[:, i10, i20] + (table[:, i10, i21] - table[:, i10, i20]) * w2
        a1 = table[:, i11, i20] + (table[:, i11, i21] - table[:, i11, i20]) * w2
        return a0 + (a1 - a0) * w1

    def transmission_at(self, group_energy, omega, pixel_positions, geometry: ConeGeometry,
                        angle: float) -> np.ndarray:
        """[G, ...] transmission of photons along ``omega`` arriving at ``pixel_positions``; crossed septa multiply
        (reference ``detector.py:704-727``)."""
        theta1, theta2 = grid_angles(omega, pixel_positions, geometry, angle, self.focal_distance_cm,
                                     self.septa_along)
        out = self.at(group_energy, theta1, theta2)
        if self.crossed is not None:
            out = out * self.crossed.transmission_at(group_energy, omega, pixel_positions, geometry, angle)
        return out

    def at_energy(self, group_energy) -> np.ndarray:
        """[G] transmission of a table that does not depend on the angles."""
        if self.depends_on_angles:
            raise ValueError(f"{self.name}: the transmission depends on the grid angles; use transmission_at")
        e = _as_f64(group_energy).reshape(-1)
        i0, i1, w = _bracket(self.energy_kev, e)
        col = self.transmission[:, 0, 0]
        return col[i0] + (col[i1] - col[i0]) * w

    def septa_sets(self) -> tuple:
        """The sets of septa, each without crossed septa: one, or two for a crossed grid."""
        if self.crossed is None:
            return (self,)
        return (replace(self, crossed=None), self.crossed)


def no_grid() -> GridResponse:
    """Transmission 1 everywhere (reference ``detector.py:758-766``)."""
    e = np.array([1.0, 1000.0])
    t = np.array([0.0, math.pi / 2])
    return GridResponse(e, t, t.copy(), np.ones((2, 2, 2)), name="no grid")


def _default_theta1_nodes() -> np.ndarray:
    """Angles dense over 0-10 degrees, where the septum shadow opens, then coarser to 89.5 degrees (rad)."""
    return np.radians(np.unique(np.concatenate([np.linspace(0.0, 10.0, 401), np.linspace(10.0, 89.5, 160)])))


def focused_1d_grid(mass_attenuation: Callable, ratio: float = 10.0, lamella_thickness_cm: float = 0.0036,
                    lamella_height_cm: float = 0.15, pitch_cm: float = 1.0 / 60.0, focal_distance_cm: float = 150.0,
                    lead_density: float = LEAD_DENSITY, energies=None, theta1=None) -> GridResponse:
    """Focused 1-D grid with the geometric septum-shadow model (reference ``detector.py:778-836``): septa of thickness
    t and height h at pitch p; a photon tilted by theta1 in the focusing plane passes the open fraction
    ``max(0, (p - t) - h |tan theta1|) / p`` and the rest crosses the mean septum path ``(t / p) h / cos(theta1) /
    shadow``, so ``G = open + shadow exp(-mu(E) rho L)``, independent of theta2.

    ``mass_attenuation`` maps keV (numpy) to the septum material's total mass attenuation in cm^2/g: the photon data the
    reference reads it from is not part of this package, so the caller supplies it."""
    p, t, h = float(pitch_cm), float(lamella_thickness_cm), float(lamella_height_cm)
    if not (0.0 <= t < p) or h < 0:
        raise ValueError("need 0 <= lamella thickness < pitch and height >= 0")
    energy = np.sort(np.linspace(10.0, 150.0, 281) if energies is None else _as_f64(energies).reshape(-1))
    th1 = np.sort(_default_theta1_nodes() if theta1 is None else _as_f64(theta1).reshape(-1))
    mu = np.asarray(mass_attenuation(energy), dtype=np.float64).reshape(-1)
    tan1 = np.abs(np.tan(np.clip(th1, -math.pi / 2 + 1e-9, math.pi / 2 - 1e-9)))
    open_fraction = np.maximum(0.0, (p - t) - h * tan1) / p
    shadow = 1.0 - open_fraction
    with np.errstate(divide="ignore", invalid="ignore"):
        path = np.where(shadow > 0, (t / p) * h / np.cos(th1) / np.where(shadow > 0, shadow, 1.0), 0.0)
    table = open_fraction[None] + shadow[None] * np.exp(-mu[:, None] * lead_density * path[None])   # [E, T1]
    return GridResponse(energy, th1, np.array([0.0, math.pi / 2]), np.repeat(table[:, :, None], 2, axis=2),
                        focal_distance_cm=float(focal_distance_cm),
                        name=f"focused 1D grid (nominal {ratio:g}:1, h/(p-t) = {h / (p - t):.1f}), {1 / p:.0f} lp/cm")


def default_focal_distance(geometry) -> float:
    """The source-detector distance of a cone beam (a grid focused at the focal spot); infinite for a parallel beam
    (reference ``detector.py:1037-1051``)."""
    return math.inf if getattr(geometry, "is_parallel", False) else float(geometry.source_detector_dist)


def grid_angles(omega, pixel_positions, geometry: ConeGeometry, angle: float, focal_distance=None,
                septa_along: str = "channels") -> tuple:
    """(theta1, theta2) float64 of photons along ``omega`` arriving at pixels (reference ``detector.py:1077-1143``).

    theta1 is the angle of the reversed direction ``a = -omega`` in the plane across the septa, measured from the
    focusing direction (the line from the pixel to the focal line, which lies ``focal_distance`` along the normal;
    the normal itself for an unfocused grid); theta2 is the angle in the plane along the septa from the normal. The
    panel axes are the local ones of the surface at each pixel; septa along the rows swap the roles of u and v. With
    ``omega`` [K, 3] and ``pixel_positions`` [rows, channels, 3] the result is [K, rows, channels]; otherwise the
    two broadcast."""
    if septa_along not in SEPTA_DIRECTIONS:
        raise ValueError(f"septa_along must be one of {SEPTA_DIRECTIONS}, got {septa_along!r}")
    omega = _as_f64(omega)
    pixels = _as_f64(pixel_positions)
    f = default_focal_distance(geometry) if focal_distance is None else float(focal_distance)
    unfocused = math.isinf(f)
    if omega.ndim == 2 and pixels.ndim == 3:
        a = -omega[:, None, None, :]
        pixels = pixels[None]
    else:
        a = -omega
    u_hat, v_hat, n_hat = geometry.local_panel_axes_np(pixels, angle)
    center = np.asarray(geometry.panel_center(angle))
    if unfocused:
        focus = None
    elif geometry.use_curved_detector and septa_along == "channels":  # the focal line over each column's centre row
        focus = pixels - ((pixels - center) * v_hat).sum(-1, keepdims=True) * v_hat + f * n_hat
    elif geometry.use_curved_detector:                                   # along each pixel's own normal
        focus = pixels + f * n_hat
    else:
        focus = center + f * n_hat
    if septa_along == "rows":
        u_hat, v_hat = v_hat, u_hat
    a_n = (a * n_hat).sum(-1)
    theta_a = np.arctan2((a * v_hat).sum(-1), a_n)
    if focus is None:
        theta1 = theta_a + np.zeros(pixels.shape[:-1])
    else:
        to_focus = focus - pixels
        theta1 = theta_a - np.arctan2((to_focus * v_hat).sum(-1), (to_focus * n_hat).sum(-1))
    theta2 = np.arctan2((a * u_hat).sum(-1), a_n)
    return tuple(np.broadcast_arrays(theta1, theta2))


ANGLE_TOLERANCE = 1e-10  # rad: float64 rounding of the grid angles is ~1e-16


def septa_dependence(septa: GridResponse, probe: np.ndarray, pixels: np.ndarray, geometry: ConeGeometry,
                     angle: float) -> str:
    """How one set of septa's transmission varies over the panel (reference ``scatter_image.py:506-539``): "none",
    "direction", "rows", "channels", "sum" (a part per direction and channel plus a part per pixel, the same for
    every direction) or "general", from the grid angles of the probe directions [P, 3] at every pixel."""
    if not septa.depends_on_angles:
        return "none"
    theta = np.stack(grid_angles(probe, pixels, geometry, angle, septa.focal_distance_cm, septa.septa_along))
    first_row = theta[:, :, :1]
    pixel_part = theta - first_row
    if np.abs(pixel_part - pixel_part[:, :1]).max() > ANGLE_TOLERANCE:
        return "general"
    pixel_part = pixel_part[:, :1]
    same_channels = np.abs(first_row - first_row[..., :1]).max() <= ANGLE_TOLERANCE
    if np.abs(pixel_part).max() <= ANGLE_TOLERANCE:
        return "direction" if same_channels else "channels"
    rows_only = np.abs(pixel_part - pixel_part[..., :1]).max() <= ANGLE_TOLERANCE
    return "rows" if rows_only and same_channels else "sum"


def _group_nodes(library) -> list:
    """Per group: (index, two node energies just inside its edges and around its group energy, fine-energy mask)
    (reference ``detector.py:960-983``)."""
    edges = np.asarray(library.group_edges, dtype=np.float64)
    energy = np.asarray(library.group_energy, dtype=np.float64)
    fine_group = np.asarray(library.fine_group)
    out = []
    for g in range(energy.size):
        high, low = float(edges[g]), float(edges[g + 1])
        inset = min(1e-3, 0.25 * (high - low))
        e = float(energy[g])
        out.append((g, min(low + inset, e), max(high - inset, e), fine_group == g))
    return out


def group_averaged_responses(detector: DetectorResponse, grid_response: GridResponse, library) -> tuple:
    """The detector response and the grid transmission averaged over the fine energies of each group (reference
    ``detector.py:986-1034``): the detector weighted by the source photons, the grid by the source photons times the
    detector response at normal incidence; each becomes a table constant over the group (two nodes just inside its
    edges), so an evaluation at the group energy returns the group's mean. A group without source photons keeps the
    value at its group energy."""
    fine_energy = np.asarray(library.fine_energy, dtype=np.float64)
    fine_weight = np.asarray(library.fine_weight, dtype=np.float64)
    group_energy = np.asarray(library.group_energy, dtype=np.float64)
    groups = _group_nodes(library)
    normal = detector.at(fine_energy, np.zeros(1))[:, 0]

    def averaged(values_at, weight):
        nodes, rows = [], []
        for g, low, high, mask in groups:
            w = weight[mask]
            if mask.any() and w.sum() > 0:
                mean = np.tensordot(w, values_at(fine_energy[mask]), axes=1) / w.sum()
            else:
                mean = values_at(group_energy[g:g + 1])[0]
            nodes += [low, high]
            rows += [mean, mean]
        order = sorted(range(len(nodes)), key=lambda i: nodes[i])
        return np.array([nodes[i] for i in order]), np.stack([rows[i] for i in order])

    nodes, table = averaged(lambda e: detector.at(e, detector.theta_rad), fine_weight)
    det = DetectorResponse(nodes, detector.theta_rad, table, f"{detector.name} (group-averaged)")

    def averaged_grid(grid: GridResponse) -> GridResponse:
        t1 = np.broadcast_to(grid.theta1_rad[:, None], (grid.theta1_rad.size, grid.theta2_rad.size))
        t2 = np.broadcast_to(grid.theta2_rad[None, :], t1.shape)
        e_nodes, t = averaged(lambda e: grid.at(e, t1, t2), fine_weight * normal)
        crossed = None if grid.crossed is None else averaged_grid(grid.crossed)
        return replace(grid, energy_kev=e_nodes, transmission=t, crossed=crossed,
                       name=f"{grid.name} (group-averaged)")

    return det, averaged_grid(grid_response)


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
class FilterMaterial:
    """A beam-filter material: its density in g/cm^3 and its total mass attenuation in cm^2/g as a function of keV
    (numpy in and out). The reference resolves a catalogue name through its photon data, which is not part of this
    package; the caller supplies the attenuation here."""

    name: str
    density: float
    mass_attenuation: Callable


def _non_negative(name: str, value) -> float:
    v = float(value)
    if not math.isfinite(v) or v < 0:
        raise ValueError(f"{name} must be finite and >= 0, got {value}")
    return v


def panel_interpolate_np(image: np.ndarray, u, v, geometry: ConeGeometry) -> np.ndarray:
    """Bilinear interpolation of a [rows | 1, channels] pixel-centre table at panel coordinates, held at the outermost
    pixel centres beyond them (reference ``source.py:484-510``); float64."""
    image = np.asarray(image, dtype=np.float64)
    rows, channels = geometry.num_det_rows, geometry.num_det_channels

    def bracket(x, n):
        x = np.clip(x, 0.0, n - 1.0)
        i0 = np.clip(np.floor(x).astype(np.int64), 0, max(n - 2, 0))
        i1 = np.minimum(i0 + 1, n - 1)
        return i0, i1, np.clip(x - i0, 0.0, 1.0)

    c0, c1, wc = bracket((np.asarray(u) + geometry.det_channel_offset) / geometry.delta_det_channel
                         + (channels - 1) / 2.0, channels)
    r0, r1, wr = bracket((np.asarray(v) + geometry.det_row_offset) / geometry.delta_det_row + (rows - 1) / 2.0, rows)
    if image.shape[0] == 1:
        r0 = r1 = np.zeros_like(r0)
    top = image[r0, c0] + (image[r0, c1] - image[r0, c0]) * wc
    bottom = image[r1, c0] + (image[r1, c1] - image[r1, c0]) * wc
    return top + (bottom - top) * wr


@dataclass(frozen=True, eq=False)
class SourceModel:
    """Isotropic point source at the focal spot, collimated to the panel (reference ``source.py:58-450``).

    The angular weight b(Omega) is 1 where the ray from the focal spot meets the field (the active panel area widened
    by the field margins), past the field edge the off-focal fraction of the distance to the field rectangle (0
    without an off-focal table), times the emission profile interpolated at the ray's panel point
    (:func:`panel_interpolate_np`). A beam filter adds ``rho_f t(Omega)`` g/cm^2 to every transmission from the focal
    spot, with the thickness t interpolated like the profile.

    ``emission_profile``: [rows, channels], or [views, rows, channels] with ``emission_profile_angles`` (a view uses
    the profile of the nearest angle). ``off_focal_distance_cm`` / ``off_focal_fraction``: ascending distances past
    the field edge in cm at the panel and the emission there relative to the edge (linear; the first value below the
    first distance, 0 past the last). ``filter_material`` (:class:`FilterMaterial`) with ``filter_thickness_cm``
    [channels] or [rows, channels] at the pixel centres."""

    emission_profile: Optional[object] = None
    emission_profile_angles: Optional[object] = None
    field_margin_channels_cm: float = 0.0
    field_margin_rows_cm: float = 0.0
    off_focal_distance_cm: Optional[object] = None
    off_focal_fraction: Optional[object] = None
    filter_material: Optional[FilterMaterial] = None
    filter_thickness_cm: Optional[object] = None
    _device_cache: dict = field(default_factory=dict, init=False, repr=False)

    def __post_init__(self):
        set_ = lambda k, v: object.__setattr__(self, k, v)  # noqa: E731
        set_("field_margin_channels_cm", _non_negative("field_margin_channels_cm", self.field_margin_channels_cm))
        set_("field_margin_rows_cm", _non_negative("field_margin_rows_cm", self.field_margin_rows_cm))
        if (self.off_focal_distance_cm is None) != (self.off_focal_fraction is None):
            raise ValueError("off_focal_distance_cm and off_focal_fraction must be given together")
        if self.off_focal_distance_cm is not None:
            d = _as_f64(self.off_focal_distance_cm).reshape(-1)
            f = _as_f64(self.off_focal_fraction).reshape(-1)
            if d.size < 1 or d.size != f.size:
                raise ValueError(f"the off-focal table needs as many distances ({d.size}) as fractions ({f.size}), "
                                 "at least one")
            if not np.all(np.isfinite(d)) or np.any(d < 0) or np.any(d[1:] <= d[:-1]):
                raise ValueError("off_focal_distance_cm must be finite, >= 0 and strictly ascending")
            if not np.all(np.isfinite(f)) or np.any(f < 0):
                raise ValueError("off_focal_fraction must be finite and non-negative")
            set_("off_focal_distance_cm", tuple(float(x) for x in d))
            set_("off_focal_fraction", tuple(float(x) for x in f))
        if (self.filter_material is None) != (self.filter_thickness_cm is None):
            raise ValueError("filter_material and filter_thickness_cm must be given together")
        if self.filter_thickness_cm is not None:
            t = _as_f64(self.filter_thickness_cm)
            t = t[None, :] if t.ndim == 1 else t
            if t.ndim != 2 or t.size == 0:
                raise ValueError(f"filter_thickness_cm must be [channels] or [rows, channels], got {t.shape}")
            if not np.all(np.isfinite(t)) or np.any(t < 0):
                raise ValueError("filter_thickness_cm must be finite and non-negative")
            set_("filter_thickness_cm", np.ascontiguousarray(t))
        if self.emission_profile is None:
            if self.emission_profile_angles is not None:
                raise ValueError("emission_profile_angles needs an emission_profile")
            return
        profile = _as_f64(self.emission_profile)
        if profile.ndim not in (2, 3):
            raise ValueError(f"emission_profile must be [rows, channels] or [views, rows, channels], got "
                             f"{profile.shape}")
        if not np.all(np.isfinite(profile)) or np.any(profile < 0):
            raise ValueError("emission_profile must be finite and non-negative")
        angles = None
        if profile.ndim == 3:
            if self.emission_profile_angles is None and profile.shape[0] > 1:
                raise ValueError("a per-view emission_profile needs emission_profile_angles")
            if self.emission_profile_angles is not None:
                angles = tuple(float(a) for a in _as_f64(self.emission_profile_angles).reshape(-1))
                if len(angles) != profile.shape[0]:
                    raise ValueError(f"emission_profile has {profile.shape[0]} views, emission_profile_angles "
                                     f"{len(angles)}")
        elif self.emission_profile_angles is not None:
            raise ValueError("emission_profile_angles applies to a per-view [views, rows, channels] profile only")
        set_("emission_profile", profile)
        set_("emission_profile_angles", angles)

    # ---- tables ---------------------------------------------------------------------------------------------------
    @property
    def has_filter(self) -> bool:
        return self.filter_material is not None

    @property
    def filter_density(self) -> float:
        return 0.0 if self.filter_material is None else float(self.filter_material.density)

    def profile_at(self, angle: float) -> Optional[np.ndarray]:
        """[rows, channels] float64 emission profile of one view (the nearest angle of a per-view profile)."""
        p = self.emission_profile
        if p is None:
            return None
        if p.ndim == 2:
            return p
        if self.emission_profile_angles is None:
            return p[0]
        return p[int(np.argmin(np.abs(np.asarray(self.emission_profile_angles) - float(angle))))]

    def thickness_at(self, geometry: ConeGeometry) -> Optional[np.ndarray]:
        """[rows | 1, channels] float64 filter thickness at the pixel centres, checked against the panel."""
        t = self.filter_thickness_cm
        if t is None:
            return None
        rows, channels = geometry.image_shape
        if t.shape[1] != channels or t.shape[0] not in (1, rows):
            raise ValueError(f"filter_thickness_cm is {t.shape}, the panel {geometry.image_shape} (or [{channels}] for "
                             "every row)")
        return t

    def filter_attenuation(self, library) -> Optional[np.ndarray]:
        """[E] total mass attenuation of the filter at the library's fine energies in cm^2/g (None without one)."""
        if self.filter_material is None:
            return None
        e = np.asarray(library.fine_energy, dtype=np.float64)
        return np.asarray(self.filter_material.mass_attenuation(e), dtype=np.float64).reshape(e.shape)

    def device_tables(self, geometry: ConeGeometry, angle: float, device) -> dict:
        """float64 device copies of the tables one view reads (profile, filter thickness, off-focal nodes and values),
        cached per table and device."""
        out = {}
        profile = self.profile_at(angle)
        if profile is not None and profile.shape != geometry.image_shape:
            raise ValueError(f"emission_profile is {profile.shape} per view, the panel {geometry.image_shape}")
        tables = {"profile": profile, "thickness": self.thickness_at(geometry),
                  "off_nodes": None if self.off_focal_distance_cm is None else np.asarray(self.off_focal_distance_cm),
                  "off_values": None if self.off_focal_fraction is None else np.asarray(self.off_focal_fraction)}
        for k, t in tables.items():
            if t is None:
                out[k] = None
                continue
            key = (k, id(t), str(device))
            hit = self._device_cache.get(key)
            if hit is None or hit[0] is not t:
                hit = (t, torch.as_tensor(np.ascontiguousarray(t), dtype=torch.float64).to(device))
                self._device_cache[key] = hit
            out[k] = hit[1]
        return out

    def field_args(self, geometry: ConeGeometry, angle: float) -> list:
        """The 23 doubles of the field argument of ``citrus_source_field``."""
        u_hat, v_hat, n_hat = geometry.panel_axes(angle)
        half_u, half_v = geometry.panel_half_extent()
        return [1.0 if geometry.use_curved_detector else 0.0, *geometry.source_position(angle),
                *geometry.panel_center(angle), *u_hat, *v_hat, *n_hat, float(geometry.source_detector_dist),
                float(geometry.det_channel_offset), float(geometry.det_row_offset), half_u, half_v,
                float(self.field_margin_channels_cm), float(self.field_margin_rows_cm)]

    def panel_args(self, geometry: ConeGeometry) -> list:
        """The 6 doubles of the panel argument of ``citrus_source_field``: rows, channels, row and channel pitch, row
        and channel offsets."""
        return [float(geometry.num_det_rows), float(geometry.num_det_channels), float(geometry.delta_det_row),
                float(geometry.delta_det_channel), float(geometry.det_row_offset), float(geometry.det_channel_offset)]

    # ---- host evaluation (pixels, tests) ---------------------------------------------------------------------------
    @staticmethod
    def _panel_point(d: np.ndarray, geometry: ConeGeometry, angle: float) -> tuple:
        src = np.asarray(geometry.source_position(angle))
        t = geometry.panel_distance_along_np(np.broadcast_to(src, d.shape), d, angle)
        forward = np.isfinite(t) & (t > 0)
        hit = src + np.where(forward, t, 0.0)[..., None] * d
        u, v = geometry.panel_uv_of_points_np(hit, angle)
        return forward, u, v

    def _field_weight(self, u, v, geometry: ConeGeometry) -> np.ndarray:
        half_u, half_v = geometry.panel_half_extent()
        edge_u = half_u + self.field_margin_channels_cm
        edge_v = half_v + self.field_margin_rows_cm
        off_u = np.abs(u + geometry.det_channel_offset)
        off_v = np.abs(v + geometry.det_row_offset)
        inside = (off_u <= edge_u) & (off_v <= edge_v)
        if self.off_focal_distance_cm is None:
            return inside.astype(np.float64)
        past_u = np.maximum(off_u - edge_u, 0.0)
        past_v = np.maximum(off_v - edge_v, 0.0)
        distance = np.sqrt(past_u * past_u + past_v * past_v)
        nodes = np.asarray(self.off_focal_distance_cm)
        values = np.asarray(self.off_focal_fraction)
        n = nodes.size
        above = np.searchsorted(nodes, distance, side="right")
        i0 = np.clip(above - 1, 0, n - 1)
        i1 = np.minimum(above, n - 1)
        span = nodes[i1] - nodes[i0]
        with np.errstate(divide="ignore", invalid="ignore"):
            w = np.clip(np.where(span > 0, (distance - nodes[i0]) / np.where(span > 0, span, 1.0), 0.0), 0.0, 1.0)
        fraction = values[i0] + (values[i1] - values[i0]) * w
        fraction = np.where(distance > nodes[-1], 0.0, fraction)
        return np.where(inside, 1.0, fraction)

    def angular_weight_np(self, directions: np.ndarray, geometry: ConeGeometry, angle: float) -> np.ndarray:
        """b(Omega) at float64 directions from the focal spot (reference ``source.py:368-382``)."""
        d = np.asarray(directions, dtype=np.float64)
        forward, u, v = self._panel_point(d, geometry, angle)
        w = forward * self._field_weight(u, v, geometry)
        profile = self.profile_at(angle)
        if profile is None:
            return w
        if profile.shape != geometry.image_shape:
            raise ValueError(f"emission_profile is {profile.shape} per view, the panel {geometry.image_shape}")
        return w * panel_interpolate_np(profile, u, v, geometry)

    def filter_path_np(self, directions: np.ndarray, geometry: ConeGeometry, angle: float) -> Optional[np.ndarray]:
        """rho_f t(Omega) in g/cm^2 of the rays from the focal spot (reference ``source.py:402-430``), None without a
        filter; float64."""
        if self.filter_material is None:
            return None
        _, u, v = self._panel_point(np.asarray(directions, dtype=np.float64), geometry, angle)
        return panel_interpolate_np(self.thickness_at(geometry), u, v, geometry) * self.filter_density


def bowtie_emission_profile(geometry: ConeGeometry, edge_weight: float = 0.2) -> np.ndarray:
    """[rows, channels] float64 profile ``edge_weight ** ((u / u_max)^2)`` across the channels, the same on every row
    (reference ``source.py:513-533``)."""
    if not 0.0 < float(edge_weight) <= 1.0:
        raise ValueError("edge_weight must be in (0, 1]")
    u, _ = geometry.pixel_uv()
    u_max = float(np.abs(u).max())
    x = u / u_max if u_max > 0 else np.zeros_like(u)
    return np.repeat(np.exp(math.log(float(edge_weight)) * x * x)[None, :], geometry.num_det_rows, axis=0)
