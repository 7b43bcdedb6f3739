"""Collapsed-cone scatter image and primary image of one view (mirrors ``citrus/scatter_solver/scatter_image.py``).

Per chunk of panel-facing cone directions the image runs: the downstream optical depth of the transport cells
(``Projectors.downstream_cumulative``), the attenuated total emission at the quadrature points with its height sums
(``citrus_attenuated_emission_moments``, which forms the multiple-collision source ``Y_k @ T`` of each point's cell in
registers; with direction-only signal weights the groups are summed there), the projection through every pixel centre
(``Projectors.oblique_project``, written rows-outer), the finite-cone footprint blur (``citrus_box_blur``, widths from
the height sums on the device) and the weighted accumulation (``citrus_weighted_group_sum``,
``citrus_sum_directions``, ``citrus_weighted_direction_sum``).
"""

from __future__ import annotations

import math
import os
from dataclasses import dataclass, field, replace
from typing import Optional

import numpy as np
import torch
from torch import Tensor

from . import _lib, kernels
from .cross_sections import MultigroupLibrary
from .geometry import ConeGeometry, Grid
from .quadrature import Quadrature, hemisphere_quadrature, real_spherical_harmonics, to_device
from .ray_tracing import HostArgs
from .responses import (DetectorResponse, GridResponse, SourceModel, detector_angle, grid_angles,
                        septa_dependence)
from .uncollided import _FCArgs, group_transmission, present_materials

IMAGE_CHUNK_MAX_DIRECTIONS = 32
IMAGE_CHUNK_BUDGET_BYTES = 256 * 2 ** 20


def covering_polar_angle(grid: Grid, geometry: ConeGeometry, angle: float, margin: float = 1e-6) -> float:
    """Smallest cone half-angle about the inward panel normal containing every box-to-panel direction
    (reference ``scatter_image.py:59-95``)."""
    lower, extent = grid.lower_corner(), grid.extent
    corners = np.array([[lower[0] + i * extent[0], lower[1] + j * extent[1], lower[2] + k * extent[2]]
                        for i in (0, 1) for j in (0, 1) for k in (0, 1)])
    u_hat, v_hat, n_hat = (np.asarray(a) for a in geometry.panel_axes(angle))
    pc = np.asarray(geometry.panel_center(angle))
    half_u, half_v = geometry.panel_half_extent()
    cu, cv = -geometry.det_channel_offset, -geometry.det_row_offset
    if geometry.use_curved_detector:
        eu = cu + np.linspace(-half_u, half_u, 4 * geometry.num_det_channels + 1)
        ev = cv + np.array([-half_v, half_v])
        panel = geometry.panel_points_np(eu[:, None], ev[None, :], angle).reshape(-1, 3)
    else:
        panel = np.stack([pc + (cu + su * half_u) * u_hat + (cv + sv * half_v) * v_hat
                          for su in (-1, 1) for sv in (-1, 1)])
    d = panel[:, None, :] - corners[None, :, :]
    normal = (d * (-n_hat)).sum(-1)
    if np.any(normal <= 0):
        return math.pi / 2
    lateral = np.linalg.norm(d - normal[..., None] * (-n_hat), axis=-1)
    return float(min(math.pi / 2, float(np.arctan2(lateral, normal).max()) + margin))


def panel_direction_set(geometry: ConeGeometry, angle: float, counts: tuple, max_polar_angle=math.pi / 2) -> Quadrature:
    """Cone product set about the inward panel normal with gnomonic cell widths (reference ``:98-130``)."""
    if isinstance(max_polar_angle, Grid):
        max_polar_angle = covering_polar_angle(max_polar_angle, geometry, angle)
    u_hat, v_hat, n_hat = geometry.panel_axes(angle)
    return hemisphere_quadrature([-c for c in n_hat], int(counts[0]), int(counts[1]), max_polar_angle,
                                 tangent_axes=(u_hat, v_hat))


@dataclass(eq=False)
class PixelSepta:
    """One set of septa whose grid angles vary along the rows and the channels together (reference ``_PixelGrid``,
    ``scatter_image.py:437-486``, its "sum" form): theta(k, r, c) = theta_channels[:, k, c] + theta_pixels[:, r, c],
    and the table at the group energies. Device float32."""

    theta_channels: Tensor  # [2, K, Cd]
    theta_pixels: Tensor    # [2, Rd, Cd]
    table: Tensor           # [G, T1, T2]
    theta1_nodes: Tensor    # [T1]
    theta2_nodes: Tensor    # [T2]


@dataclass(eq=False)
class DirectionSetContext:
    """The emission-independent part of one view's image (reference ``scatter_image.py:137-405``).

    Device tensors (float32): omega [K, 3], weight [K], cos_theta0 [K], cell_width [K, 2]; ``signal_group_weight``
    [K, G] when the signal weights are the same at every pixel (flat panel, a grid that varies only with the
    direction), else ``signal_channel_weight`` [K, G, Cd] (curved panel: incidence per channel; septa along the
    rows); ``planar_weight`` [K, 1 | Cd]. A curved panel whose detector response separates into a factor of the
    energy and a factor of the incidence (the ideal counting response, for one) also has ``signal_group_weight``
    [K, G] and ``signal_column_weight`` [K, Cd] with
    ``signal_channel_weight[k, g, c] = signal_group_weight[k, g] * signal_column_weight[k, c]``: the signal image is
    then the group sum weighted in the emission, blurred, and weighted per channel in the sum over the directions
    (the channel blur acts before the channel weights in the reference, and the row blur commutes with them).
    An anti-scatter grid that varies along the rows adds ``signal_row_weight`` [K, G, Rd], septa that vary along
    the rows and the channels together add ``pixel_septa``; the signal is then accumulated by
    ``citrus_grid_signal_sum`` from the blurred per-group images (the reference applies these weights after the
    footprint blur too).
    """

    quadrature: Quadrature
    geometry: ConeGeometry
    angle: float
    group_energy: np.ndarray
    omega: Tensor
    weight: Tensor
    cos_theta0: Tensor
    cell_width: Tensor
    signal_group_weight: Optional[Tensor]
    signal_channel_weight: Optional[Tensor]
    planar_weight: Tensor
    chunk_bounds: tuple
    image_shape: tuple
    signal_column_weight: Optional[Tensor] = None
    signal_row_weight: Optional[Tensor] = None
    pixel_septa: tuple = ()
    septa_kinds: tuple = ()
    _cache: dict = field(default_factory=dict, repr=False)

    @property
    def num_directions(self) -> int:
        return int(self.omega.shape[0])

    @property
    def device(self) -> torch.device:
        return self.omega.device

    @property
    def grid_varies_over_panel(self) -> bool:
        """True when the signal needs ``citrus_grid_signal_sum`` (weights per row, or per pixel)."""
        return self.signal_row_weight is not None or bool(self.pixel_septa)

    def harmonics(self, L: int) -> Tensor:
        key = ("Y", int(L))
        if key not in self._cache:
            self._cache[key] = to_device(real_spherical_harmonics(L, self._omega64), self.device)
        return self._cache[key]

    def crossing_tables(self, grid: Grid, projectors) -> Optional[Tensor]:
        """The downstream walk's crossing tables of the set's directions on ``grid``, built once and kept with the
        set (None for projectors that build their own)."""
        if not hasattr(projectors, "crossing_tables"):
            return None
        key = ("crossings", grid)
        if key not in self._cache:
            self._cache[key] = projectors.crossing_tables(grid, self.omega)
        return self._cache[key]

    def footprint(self, grid: Grid) -> tuple:
        """(heights [V] of the point centres above the panel, height of the box centre) (reference ``:1033-1077``)."""
        key = ("footprint", grid)
        if key not in self._cache:
            _, _, n_hat = self.geometry.panel_axes(self.angle)
            pc = np.asarray(self.geometry.panel_center(self.angle))
            x, y, z = (a.double().numpy() for a in grid.axis_coordinates(dtype=torch.float64))
            h = ((x[None, :, None] - pc[0]) * n_hat[0] + (y[:, None, None] - pc[1]) * n_hat[1]
                 + (z[None, None, :] - pc[2]) * n_hat[2])
            lower, extent = grid.lower_corner(), grid.extent
            corner = [sum((lower[a] + c[a] * extent[a] - pc[a]) * n_hat[a] for a in range(3))
                      for c in [(i, j, k) for i in (0, 1) for j in (0, 1) for k in (0, 1)]]
            self._cache[key] = (to_device(np.broadcast_to(h, grid.shape).reshape(-1), self.device),
                                0.5 * (min(corner) + max(corner)))
        return self._cache[key]


def _grid_factors(grid_response: GridResponse, energy: np.ndarray, omega: np.ndarray, geometry: ConeGeometry,
                  angle: float, device) -> tuple:
    """Septa factors of one view (reference ``scatter_image.py:605-657``): ([G, K] per direction, [G, K, Rd] per row
    or None, [G, K, Cd] per channel or None, pixel septa, kinds). How each set of septa varies over the panel is
    decided from probe directions (the inward normal and three of the set's directions)."""
    G, K = energy.size, omega.shape[0]
    pixels = geometry.pixel_centers_np(angle)
    n_hat = np.asarray(geometry.panel_axes(angle)[2])
    probe = -n_hat[None]
    if K:
        probe = np.concatenate([probe, omega[[0, K // 2, K - 1]]])
    direction = np.ones((G, K))
    rows = channels = None
    pixel = []
    kinds = []
    for septa in grid_response.septa_sets():
        kind = septa_dependence(septa, probe, pixels, geometry, angle)
        kinds.append(kind)
        if kind == "none":
            direction = direction * septa.at(energy, 0.0, 0.0)[:, None]
        elif kind == "direction":
            direction = direction * septa.transmission_at(energy, omega, pixels[:1, :1], geometry, angle)[:, :, 0, 0]
        elif kind == "rows":
            t = septa.transmission_at(energy, omega, pixels[:, :1], geometry, angle)[..., 0]        # [G, K, Rd]
            rows = t if rows is None else rows * t
        elif kind == "channels":
            t = septa.transmission_at(energy, omega, pixels[:1], geometry, angle)[:, :, 0]          # [G, K, Cd]
            channels = t if channels is None else channels * t
        elif kind == "sum":
            first_row = np.stack(grid_angles(omega, pixels[:1], geometry, angle, septa.focal_distance_cm,
                                             septa.septa_along))                                     # [2, K, 1, Cd]
            one = np.stack(grid_angles(omega[:1], pixels, geometry, angle, septa.focal_distance_cm,
                                       septa.septa_along))                                           # [2, 1, Rd, Cd]
            pixel.append(PixelSepta(to_device(np.ascontiguousarray(first_row[:, :, 0]), device),
                                    to_device(np.ascontiguousarray((one - one[:, :, :1])[:, 0]), device),
                                    to_device(np.ascontiguousarray(septa.table_at_energy(energy)), device),
                                    to_device(septa.theta1_rad, device), to_device(septa.theta2_rad, device)))
        else:
            raise NotImplementedError(
                f"{septa.name}: grid angles that are not a part per direction and channel plus a part per pixel "
                "(the reference's 'general' septa) are not evaluated on this path")
    return direction, rows, channels, tuple(pixel), tuple(kinds)


def make_direction_context(quadrature: Quadrature, geometry: ConeGeometry, angle: float, detector: DetectorResponse,
                           grid_response: GridResponse, library: MultigroupLibrary, device,
                           chunk: int = 8) -> DirectionSetContext:
    """Keep the panel-facing directions and precompute their weights (reference ``scatter_image.py:542-696``)."""
    energy = np.asarray(library.group_energy, dtype=np.float64)
    G = energy.size
    signal_column = None
    _, _, n_hat = geometry.panel_axes(angle)
    n_hat = np.asarray(n_hat)
    # the selection in the images' float32, as the projectors see a grazing direction
    cos32 = (quadrature.omega.astype(np.float32) * (-n_hat).astype(np.float32)).sum(-1)
    kept = np.nonzero(cos32 > 0)[0]
    omega = quadrature.omega[kept]
    weight = quadrature.weight[kept]
    cos64 = (omega * (-n_hat)).sum(-1)
    K = kept.size
    Rd, Cd = geometry.image_shape
    grid_direction, grid_rows, grid_channels, pixel_septa, kinds = _grid_factors(grid_response, energy, omega,
                                                                                 geometry, angle, device)
    row_weight = None if grid_rows is None else to_device(np.ascontiguousarray(grid_rows.transpose(1, 0, 2)), device)
    if geometry.use_curved_detector:
        pixels = geometry.pixel_centers_np(angle)
        normals = geometry.local_normals_np(pixels[0], angle)                   # [Cd, 3]
        cos_channel = np.clip(omega @ (-normals).T, 0.0, 1.0)                   # [K, Cd]
        planar = weight[:, None] * cos_channel
        response = detector.at(energy, np.arccos(cos_channel))                 # [G, K, Cd]
        channel = planar[None] * response * grid_direction[:, :, None]         # [G, K, Cd]
        if grid_channels is not None:
            channel = channel * grid_channels
        signal_group, signal_channel = None, to_device(channel.transpose(1, 0, 2), device)
        planar_weight = to_device(planar, device)
        # a response D(E, theta) = f(E) h(theta): group factors f_g / f_0 and channel factors D(E_0, theta_kc)
        first = response[:1]
        if K and np.all(first > 0) and grid_channels is None:
            ratio = response / first
            if np.allclose(ratio, ratio[:, :1, :1], rtol=1e-12, atol=0.0):
                group = ratio[:, 0, 0][:, None] * grid_direction                # [G, K]
                signal_group = to_device(np.ascontiguousarray(group.T), device)
                signal_column = to_device(planar * first[0], device)
    else:
        response = detector.at(energy, detector_angle(omega, geometry, angle)) if K else np.zeros((G, 0))
        direction = (weight * cos64)[None] * response * grid_direction          # [G, K]
        if grid_channels is None:
            signal_group, signal_channel = to_device(direction.T, device), None
        else:
            signal_group = None
            signal_channel = to_device((direction[:, :, None] * grid_channels).transpose(1, 0, 2), device)
        planar_weight = to_device((weight * cos64)[:, None], device)
    if row_weight is not None or pixel_septa:
        # weights that vary along the rows: the groups cannot be summed in the emission
        if signal_channel is None:
            signal_channel = signal_group.reshape(K, G, 1).contiguous()
        signal_group = signal_column = None
    chunk = max(1, int(chunk))
    ctx = DirectionSetContext(
        quadrature=quadrature, geometry=geometry, angle=float(angle), group_energy=energy, omega=to_device(omega, device),
        weight=to_device(weight, device), cos_theta0=to_device(cos64, device),
        cell_width=to_device(quadrature.cell_width[kept], device), signal_group_weight=signal_group,
        signal_channel_weight=signal_channel, planar_weight=planar_weight,
        chunk_bounds=tuple((s, min(s + chunk, K)) for s in range(0, K, chunk)), image_shape=(Rd, Cd),
        signal_column_weight=signal_column, signal_row_weight=row_weight, pixel_septa=pixel_septa, septa_kinds=kinds)
    ctx._omega64 = omega
    return ctx


# How the image's emission gets the multiple-collision source: "fused" forms Y_k T per point in registers
# (citrus_attenuated_emission_moments); "product" writes Y_k T with the small-K product first and reads it
# (citrus_attenuated_emission, the reference's interface). CITRUS_EMISSION_FORM picks one (both give the same image
# to float rounding; the product form is the default, measured faster).
EMISSION_FORM = os.environ.get("CITRUS_EMISSION_FORM", "product")
if EMISSION_FORM not in ("product", "fused"):
    raise ValueError(f"CITRUS_EMISSION_FORM must be 'product' or 'fused', got {EMISSION_FORM!r}")


def _blur(src: Tensor, dst: Tensor, lines: int, length: int, strides_in: tuple, strides_out: tuple, k: int,
          height_sums: Tensor, cell_width: Tensor, axis: int, pitch: float, center_height: float) -> None:
    _lib.call("citrus_box_blur", src.data_ptr(), dst.data_ptr(), k, lines, length, *strides_in, *strides_out, None,
              height_sums.data_ptr(), cell_width.data_ptr(), axis, float(pitch), float(center_height),
              _lib.stream_handle(src.device))


def _grid_signal_sum(context: DirectionSetContext, img: Tensor, s: int, e: int, strides: tuple, acc: Tensor,
                     per_group: bool, stream) -> None:
    """Signal of directions [s, e) behind a grid that varies over the panel (``citrus_grid_signal_sum``)."""
    k, Rd, G, Cd = img.shape
    w = context.signal_channel_weight[s:e].contiguous()                       # [k, G, Cd | 1]
    rows = None if context.signal_row_weight is None else context.signal_row_weight[s:e].contiguous()
    host = HostArgs()
    septa = context.pixel_septa
    theta_ch = [ps.theta_channels[:, s:e].contiguous() for ps in septa]       # kept alive for the call
    ptrs = lambda ts: host.pointers([t.data_ptr() for t in ts]) if ts else None  # noqa: E731
    _lib.call("citrus_grid_signal_sum", img.data_ptr(), k, G, Rd, Cd, *strides, w.data_ptr(), int(w.shape[-1]),
              None if rows is None else rows.data_ptr(), len(septa), ptrs(theta_ch),
              ptrs([ps.theta_pixels for ps in septa]), ptrs([ps.table for ps in septa]),
              ptrs([ps.theta1_nodes for ps in septa]),
              host.int64s([ps.theta1_nodes.numel() for ps in septa]) if septa else None,
              ptrs([ps.theta2_nodes for ps in septa]),
              host.int64s([ps.theta2_nodes.numel() for ps in septa]) if septa else None,
              acc.data_ptr(), int(per_group), 1, stream)


def combined_scatter_image(library: MultigroupLibrary, rho_quadrature: Tensor, phi_uncollided: Tensor,
                           grid_quadrature: Grid, q: int, scatter_source_moments: Tensor, L: int,
                           geometry: ConeGeometry, angle: float, mu_t_coarse: Tensor, projectors,
                           context: DirectionSetContext, grid_coarse: Optional[Grid] = None,
                           signal_only: bool = False, footprint: bool = True, rho_coarse: Optional[Tensor] = None,
                           attenuation: Optional[Tensor] = None, precision: str = "fp32") -> dict:
    """Total scatter image of one view, first order plus multiple collision (reference ``scatter_image.py:1141-1323``).

    Returns ``{"signal": [Rd, Cd]}`` with ``signal_only``, else fluence, planar_fluence and signal_per_group
    [G, Rd, Cd] and signal [Rd, Cd]. When ``mu_t_coarse`` is ``sum_m attenuation[m, g] rho_coarse[m]`` (the solver's
    fields) and both are given, the downstream optical depths are traced through the M cell densities instead of the
    G attenuation channels and combined per group in the emission (the same line integrals, by linearity).
    ``precision`` is the arithmetic of the multiple-collision product ``Y_k T`` (``kernels.small_k_gemm``).
    """
    device = phi_uncollided.device
    f = int(q)
    grid_coarse = grid_quadrature.coarsen(f) if grid_coarse is None else grid_coarse
    G = int(mu_t_coarse.shape[0])
    NC = grid_coarse.num_voxels
    V = grid_quadrature.num_voxels
    if scatter_source_moments.dim() == 6:
        scatter_source_moments = scatter_source_moments[:, :, 0]
    N_sh = (L + 1) ** 2
    if tuple(scatter_source_moments.shape) != (G, N_sh, *grid_coarse.shape):
        raise ValueError(f"scatter_source_moments must be [{G}, {N_sh}, {grid_coarse.shape}]")
    # [N_sh, cells, G] (the groups of a cell contiguous, as the emission reads them): a view of cell-major storage,
    # else one copy
    T = scatter_source_moments.permute(1, 2, 3, 4, 0).reshape(N_sh, NC * G).contiguous()
    Y = context.harmonics(L)
    Rd, Cd = context.image_shape
    heights, center_height = context.footprint(grid_quadrature)
    fc = _FCArgs(library, rho_quadrature, phi_uncollided, grid_quadrature, geometry, angle)
    host = HostArgs()
    deltas = host.doubles(grid_quadrature.deltas)
    mu = mu_t_coarse.to(torch.float32).reshape(G, NC).contiguous()
    flat_signal = signal_only and context.signal_group_weight is not None
    C = 1 if flat_signal else G
    acc = torch.zeros(Rd, Cd, device=device) if signal_only else torch.zeros(3, G, Rd, Cd, device=device)
    K_max = max((e - s for s, e in context.chunk_bounds), default=0)
    nblocks = -(-V // 32)
    partial = torch.empty(K_max * nblocks * 2, device=device)
    sums = torch.empty(K_max, 2, device=device)
    stream = _lib.stream_handle(device)
    traced = tau_mu = None
    if rho_coarse is not None and attenuation is not None:
        traced = rho_coarse.to(device=device, dtype=torch.float32).contiguous()
        tau_mu = attenuation.to(device=device, dtype=torch.float32).contiguous()
        if tuple(tau_mu.shape) != (traced.shape[0], G) or tuple(traced.shape[1:]) != tuple(grid_coarse.shape):
            raise ValueError(f"attenuation must be [M, {G}] and rho_coarse [M, {grid_coarse.shape}]")
    tables = context.crossing_tables(grid_coarse, projectors)
    for s, e in context.chunk_bounds:
        k = e - s
        dirs = context.omega[s:e]
        walk = {} if tables is None else {"crossings": tables[s:e]}
        if traced is not None:
            tau = projectors.downstream_cumulative(traced, grid_coarse, geometry, angle, dirs,
                                                   voxel_major=True, **walk)              # [k, cells, M]
        else:
            tau = projectors.downstream_cumulative(mu_t_coarse, grid_coarse, geometry, angle, dirs,
                                                   voxel_major=True, **walk)              # [k, cells, G]
        Yk = Y[s:e].contiguous()
        emission = torch.empty(k, V, C, device=device)
        head = (*fc.common(), f, deltas, fc.focal, fc.table.data_ptr(), fc.num_eta, fc.eta_lo, fc.eta_hi,
                dirs.data_ptr(), k, tau.data_ptr(), None if traced is None else tau_mu.data_ptr(),
                0 if traced is None else int(traced.shape[0]), mu.data_ptr())
        # every tensor whose address a call takes stays bound until the call is queued: a temporary's memory returns
        # to the allocator when the expression ends, before the kernel reads it
        group_weight = context.signal_group_weight[s:e].contiguous() if flat_signal else None
        tail = (heights.data_ptr(), None if group_weight is None else group_weight.data_ptr(),
                emission.data_ptr(), partial.data_ptr(), partial.numel(), sums.data_ptr(), stream)
        if EMISSION_FORM == "fused":
            _lib.call("citrus_attenuated_emission_moments", *head, Yk.data_ptr(), T.data_ptr(), N_sh, *tail)
        else:
            multiple = torch.empty(k, NC * G, device=device)                               # [k, cells, G]
            kernels.small_k_gemm(Yk, T, multiple, precision=precision)
            _lib.call("citrus_attenuated_emission", *head, multiple.data_ptr(), *tail)
            del multiple
        del tau
        rows_outer = torch.empty(k, Rd, C, Cd, device=device)
        projectors.oblique_project(emission, grid_quadrature, geometry, angle, dirs,
                                   out=rows_outer.permute(0, 2, 1, 3), voxel_major=True)
        del emission
        cw = context.cell_width[s:e].contiguous()
        if not footprint:
            blurred = rows_outer
        else:
            blurred = torch.empty_like(rows_outer)  # channels: lines (row, channel-group) of Cd contiguous pixels
            _blur(rows_outer, blurred, Rd * C, Cd, (Rd * C * Cd, Cd, 1), (Rd * C * Cd, Cd, 1), k, sums, cw, 0,
                  geometry.delta_det_channel, center_height)
        grid_sum = context.grid_varies_over_panel
        if signal_only and not flat_signal and not grid_sum:
            single = torch.empty(k, Rd, Cd, device=device)
            channel_weight = context.signal_channel_weight[s:e].contiguous()
            _lib.call("citrus_weighted_group_sum", blurred.data_ptr(), channel_weight.data_ptr(), k, Rd, G, Cd, Cd,
                      single.data_ptr(), stream)
            image, C_img = single, 1
        else:
            image, C_img = blurred, C
        if footprint:  # rows: lines (channel-group, channel) of Rd pixels with stride C_img * Cd
            rows = torch.empty_like(image)
            _blur(image, rows, C_img * Cd, Rd, (Rd * C_img * Cd, 1, C_img * Cd), (Rd * C_img * Cd, 1, C_img * Cd), k,
                  sums, cw, 1, geometry.delta_det_row, center_height)
            image = rows
        if signal_only and flat_signal and context.signal_column_weight is not None:
            columns = context.signal_column_weight[s:e].contiguous()           # [k, Cd]
            _lib.call("citrus_weighted_direction_sum", image.data_ptr(), k, 1, Rd, Cd, Rd * Cd, Rd * Cd, Cd, 1,
                      columns.data_ptr(), 1, Cd, acc.data_ptr(), 1, stream)
            continue
        img = image.view(k, Rd, C_img, Cd)  # rows-outer [k, Rd, G, Cd] seen as [k, G, Rd, Cd] through strides
        strides = (Rd * C_img * Cd, Cd, C_img * Cd, 1)
        if grid_sum:
            _grid_signal_sum(context, img, s, e, strides, acc if signal_only else acc[2], not signal_only, stream)
            if signal_only:
                continue
        elif signal_only:
            _lib.call("citrus_sum_directions", image.data_ptr(), k, Rd * Cd, Rd * Cd, acc.data_ptr(), 1, stream)
            continue
        ones = context.weight[s:e].reshape(k, 1, 1, 1).expand(k, G, 1, 1).contiguous()
        planar = context.planar_weight[s:e]
        planar = planar.reshape(k, 1, 1, -1).expand(k, G, 1, planar.shape[-1]).contiguous()
        weights = [ones, planar]
        if not grid_sum:
            weights.append(context.signal_channel_weight[s:e].reshape(k, G, 1, Cd).contiguous()
                           if context.signal_channel_weight is not None
                           else context.signal_group_weight[s:e].reshape(k, G, 1, 1).contiguous())
        for j, w in enumerate(weights):
            _lib.call("citrus_weighted_direction_sum", img.data_ptr(), k, G, Rd, Cd, *strides, w.data_ptr(), 1,
                      w.shape[-1], acc[j].data_ptr(), 1, stream)
    if signal_only:
        return {"signal": acc}
    return {"fluence": acc[0], "planar_fluence": acc[1], "signal_per_group": acc[2], "signal": acc[2].sum(0)}


# ---- primary ---------------------------------------------------------------------------------------------------------

def primary_subpixel_geometry(geometry: ConeGeometry, samples_per_pixel_axis: int) -> ConeGeometry:
    """The panel with n times finer pixels on which the n^2 sub-rays of every pixel are traced: sub-pixel (i, j) of
    pixel (r, c) is pixel (r n + i, c n + j) (reference ``scatter_image.py:1330-1348``)."""
    n = int(samples_per_pixel_axis)
    if n < 1:
        raise ValueError("samples_per_pixel_axis must be >= 1")
    if n == 1:
        return geometry
    return replace(geometry, num_det_rows=geometry.num_det_rows * n, num_det_channels=geometry.num_det_channels * n,
                   delta_det_row=geometry.delta_det_row / n, delta_det_channel=geometry.delta_det_channel / n)


def primary_samples_per_pixel_axis(projectors, samples_per_pixel_axis: Optional[int]) -> int:
    """The given sub-pixel samples per axis, else the projector's own, else 1 (reference ``:1351-1365``)."""
    n = (int(samples_per_pixel_axis) if samples_per_pixel_axis is not None
         else int(getattr(projectors, "samples_per_pixel_axis", 1) or 1))
    if n < 1:
        raise ValueError("samples_per_pixel_axis must be >= 1")
    return n


def primary_path_lengths(projectors, rho: Tensor, grid: Grid, geometry: ConeGeometry, angle: float,
                         samples_per_pixel_axis: Optional[int] = None) -> Tensor:
    """[M', Rd n, Cd n] density line integrals to the pixel (or sub-pixel) centres, the sub-rays traced as the pixels
    of the refined panel (reference ``scatter_image.py:1368-1392``)."""
    n = primary_samples_per_pixel_axis(projectors, samples_per_pixel_axis)
    fine = primary_subpixel_geometry(geometry, n)
    if getattr(projectors, "samples_per_pixel_axis", None) is not None:  # the projector's own sub-sampling off
        return projectors.primary_project(rho, grid, fine, angle, samples_per_pixel_axis=1)
    return projectors.primary_project(rho, grid, fine, angle)


def primary_from_path_lengths(library: MultigroupLibrary, path: Tensor, materials, geometry: ConeGeometry,
                              angle: float, source: SourceModel, detector: DetectorResponse,
                              grid_response: GridResponse) -> dict:
    """Primary image from per-material line integrals [M', Rd n, Cd n], exact in energy (reference
    ``scatter_image.py:1395-1471``): the fine-energy transmission, with the source's beam filter on every ray, is
    averaged over the n x n sub-pixels of every pixel; the inverse square, the collimation and the responses are
    evaluated at the pixel centres, the grid transmission at every pixel's grid angles."""
    device = path.device
    Rd, Cd = geometry.image_shape
    n = int(path.shape[1]) // Rd if path.dim() == 3 else 0
    if n < 1 or tuple(path.shape[1:]) != (Rd * n, Cd * n):
        raise ValueError(f"path must be [M', {Rd} n, {Cd} n] (n >= 1 sub-pixels per axis), got {tuple(path.shape)}")
    r0 = np.asarray(geometry.source_position(angle))
    filter_path = None
    if source.has_filter:
        sub = primary_subpixel_geometry(geometry, n).pixel_centers_np(angle)
        filter_path = source.filter_path_np(sub - r0, geometry, angle)
    T = group_transmission(library, path, materials,
                           filter_path=None if filter_path is None else to_device(filter_path, device),
                           filter_attenuation=source.filter_attenuation(library))         # [G, Rd n, Cd n]
    if n > 1:
        T = T.reshape(-1, Rd, n, Cd, n).mean(dim=(2, 4))
    pixels = geometry.pixel_centers_np(angle)
    d = pixels - r0
    dist2 = (d * d).sum(-1)
    b = source.angular_weight_np(d, geometry, angle)
    omega_p = d / np.sqrt(dist2)[..., None]
    energy = library.group_energy
    theta0 = detector_angle(omega_p, geometry, angle, pixels)
    grid_t = (grid_response.transmission_at(energy, omega_p, pixels, geometry, angle)
              if grid_response.depends_on_angles else grid_response.at_energy(energy)[:, None, None])
    fluence_factor = to_device(b / dist2, device)
    planar_factor = to_device(b / dist2 * np.cos(theta0), device)
    signal_factor = to_device((b / dist2 * np.cos(theta0))[None] * detector.at(energy, theta0) * grid_t, device)
    fluence = T * fluence_factor
    signal_per_group = T * signal_factor
    return {"fluence": fluence, "planar_fluence": T * planar_factor, "signal_per_group": signal_per_group,
            "signal": signal_per_group.sum(0)}


def primary_image(library: MultigroupLibrary, rho: Tensor, grid: Grid, geometry: ConeGeometry, angle: float,
                  source: SourceModel, projectors, detector: DetectorResponse, grid_response: GridResponse,
                  samples_per_pixel_axis: Optional[int] = None) -> dict:
    """Primary image of one view from the density maps (reference ``scatter_image.py:1474-1506``)."""
    present = present_materials(rho)
    traced = rho if present is None else rho[present]
    path = primary_path_lengths(projectors, traced.contiguous(), grid, geometry, angle, samples_per_pixel_axis)
    return primary_from_path_lengths(library, path, present, geometry, angle, source, detector, grid_response)


def scatter_fraction(scatter_signal: Tensor, primary_signal: Tensor) -> Tensor:
    """S / (P + S), 0 where P + S = 0 (reference ``scatter_image.py:1509-1521``)."""
    den = primary_signal + scatter_signal
    return torch.where(den > 0, scatter_signal / torch.where(den > 0, den, torch.ones_like(den)),
                       torch.zeros_like(den))
