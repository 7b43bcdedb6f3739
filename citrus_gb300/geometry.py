"""Voxel grids and the cone-beam geometry of the scatter step (flat or curved panel, circular views).

Conventions follow the reference (``citrus/scatter_solver/geometry.py``): lengths in cm, angles in radians, volumes
``[rows, cols, slices]`` with columns along x, rows along y and slices along z; the focal spot of view ``angle`` sits at
``(sin a, cos a, 0) * source_iso_dist`` and the panel faces it. Everything here is host arithmetic in float64; device
tensors are produced only for the coordinate tables the kernels read.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, replace

import numpy as np
import torch
from torch import Tensor

_DEVICE_AXES: dict = {}   # (grid, device, dtype) -> axis coordinates on the device


@dataclass(frozen=True)
class Grid:
    """Uniform cuboid voxel grid centred on the rotation axis (reference ``geometry.py:43-239``).

    Attributes:
        shape: (rows, cols, slices), the extents along (y, x, z).
        delta_voxel: voxel pitch along x in cm.
        voxel_row_aspect: pitch along y over ``delta_voxel``.
        voxel_slice_aspect: pitch along z over ``delta_voxel``.
        recon_slice_offset: z of the grid centre in cm.
    """

    shape: tuple
    delta_voxel: float
    voxel_row_aspect: float = 1.0
    voxel_slice_aspect: float = 1.0
    recon_slice_offset: float = 0.0

    def __post_init__(self):
        object.__setattr__(self, "shape", tuple(int(s) for s in self.shape))

    @property
    def num_rows(self) -> int:
        return self.shape[0]

    @property
    def num_cols(self) -> int:
        return self.shape[1]

    @property
    def num_slices(self) -> int:
        return self.shape[2]

    @property
    def num_voxels(self) -> int:
        return self.shape[0] * self.shape[1] * self.shape[2]

    @property
    def deltas(self) -> tuple:
        """(dx, dy, dz) in cm."""
        d = float(self.delta_voxel)
        return (d, self.voxel_row_aspect * d, self.voxel_slice_aspect * d)

    @property
    def extent(self) -> tuple:
        """Box side lengths (x, y, z) in cm."""
        dx, dy, dz = self.deltas
        return (self.num_cols * dx, self.num_rows * dy, self.num_slices * dz)

    def lower_corner(self) -> tuple:
        """Minimum corner (x, y, z) of the box in cm."""
        dx, dy, dz = self.deltas
        nr, nc, ns = self.shape
        return (-nc * dx / 2, -nr * dy / 2, -ns * dz / 2 + self.recon_slice_offset)

    def axis_coordinates(self, device=None, dtype=torch.float32) -> tuple:
        """Voxel-centre coordinates x [cols], y [rows], z [slices] (reference ``geometry.py:104-119``)."""
        dx, dy, dz = self.deltas
        nr, nc, ns = self.shape
        x = dx * (np.arange(nc, dtype=np.float64) - (nc - 1) / 2)
        y = dy * (np.arange(nr, dtype=np.float64) - (nr - 1) / 2)
        z = dz * (np.arange(ns, dtype=np.float64) - (ns - 1) / 2) + self.recon_slice_offset
        return tuple(torch.as_tensor(a, dtype=dtype, device=device) for a in (x, y, z))

    def device_axes(self, device, dtype=torch.float32) -> tuple:
        """``axis_coordinates`` on ``device``, copied there once per (grid, device, dtype) and kept."""
        key = (self, str(torch.device(device)), dtype)
        axes = _DEVICE_AXES.get(key)
        if axes is None:
            axes = tuple(a.to(device) for a in self.axis_coordinates(dtype=dtype))
            _DEVICE_AXES[key] = axes
        return axes

    def center_coordinates(self, device=None, dtype=torch.float32) -> Tensor:
        """[rows, cols, slices, 3] voxel-centre positions (x, y, z)."""
        x, y, z = self.axis_coordinates(device, dtype)
        return torch.stack([x[None, :, None].expand(self.shape), y[:, None, None].expand(self.shape),
                            z[None, None, :].expand(self.shape)], dim=-1)

    @staticmethod
    def covering(grid: "Grid", cell_cm: float) -> "Grid":
        """Grid of cubic cells covering and centred on ``grid`` (reference ``geometry.py:145-170``)."""
        c = float(cell_cm)
        if not c > 0:
            raise ValueError(f"cell size must be > 0, got {cell_cm}")
        ex, ey, ez = grid.extent

        def count(e: float) -> int:
            r = e / c
            k = round(r)
            return max(1, int(k) if abs(r - k) <= 1e-9 * max(1.0, r) else int(math.ceil(r)))

        return Grid((count(ey), count(ex), count(ez)), c, recon_slice_offset=grid.recon_slice_offset)

    def refine(self, factor: int) -> "Grid":
        """The same box with ``factor`` voxels per voxel along each axis."""
        f = int(factor)
        if f < 1:
            raise ValueError(f"refinement factor must be >= 1, got {factor}")
        if f == 1:
            return self
        nr, nc, ns = self.shape
        return replace(self, shape=(nr * f, nc * f, ns * f), delta_voxel=self.delta_voxel / f)

    def coarsen(self, factor: int) -> "Grid":
        """The supervoxel grid with ``factor`` voxels per coarse voxel along each axis."""
        if factor == 1:
            return self
        nr, nc, ns = self.shape
        if nr % factor or nc % factor or ns % factor:
            raise ValueError(f"grid shape {self.shape} not divisible by the coarsening factor {factor}")
        return replace(self, shape=(nr // factor, nc // factor, ns // factor), delta_voxel=self.delta_voxel * factor)

    def axis_edges(self) -> tuple:
        """float64 numpy voxel boundaries along x, y, z."""
        dx, dy, dz = self.deltas
        nr, nc, ns = self.shape
        lx, ly, lz = self.lower_corner()
        return (lx + dx * np.arange(nc + 1), ly + dy * np.arange(nr + 1), lz + dz * np.arange(ns + 1))


def overlap_matrix(edges_from: np.ndarray, edges_to: np.ndarray) -> np.ndarray:
    """1-D overlap fractions ``W[j, i] = |cell_i n cell_j| / |cell_j|``, snapped at 1e-12 (reference ``geometry.py:251-275``)."""
    ef = np.asarray(edges_from, dtype=np.float64)
    et = np.asarray(edges_to, dtype=np.float64)
    lo = np.maximum(et[:-1, None], ef[None, :-1])
    hi = np.minimum(et[1:, None], ef[None, 1:])
    w = np.clip(hi - lo, 0.0, None) / (et[1:] - et[:-1])[:, None]
    w = np.where(w < 1e-12, 0.0, w)
    return np.where(np.abs(w - 1.0) < 1e-12, 1.0, w)


def resample_conservative(field: Tensor, grid_from: Grid, grid_to: Grid) -> Tensor:
    """Exact cell averages of a voxel-wise constant field on another grid (reference ``geometry.py:301-328``).

    Three per-axis matrix products; this is set-up work run once per outer iteration, not per view.
    """
    if tuple(field.shape[-3:]) != tuple(grid_from.shape):
        raise ValueError(f"field spatial shape {tuple(field.shape[-3:])} != grid shape {grid_from.shape}")
    if grid_from == grid_to:
        return field
    xf, yf, zf = grid_from.axis_edges()
    xt, yt, zt = grid_to.axis_edges()
    Wr, Wc, Ws = (torch.as_tensor(overlap_matrix(a, b), device=field.device, dtype=field.dtype)
                  for a, b in ((yf, yt), (xf, xt), (zf, zt)))
    x = torch.matmul(field, Ws.t())
    x = torch.matmul(x.transpose(-1, -2), Wc.t()).transpose(-1, -2)
    x = torch.matmul(x.movedim(-3, -1), Wr.t()).movedim(-1, -3)
    return x.contiguous()


@dataclass(frozen=True)
class ConeGeometry:
    """Circular cone-beam geometry with a flat or cylindrical panel (reference ``geometry.py:330-765``).

    In the view frame the source is at ``(0, source_iso_dist, 0)``, channels run along +x_view and rows along +z; the
    flat panel lies in the plane ``y_view = source_iso_dist - source_detector_dist``, the curved panel on the cylinder
    of radius ``source_detector_dist`` about the vertical axis through the source.
    """

    source_iso_dist: float
    source_detector_dist: float
    num_det_rows: int
    num_det_channels: int
    delta_det_row: float
    delta_det_channel: float
    det_row_offset: float = 0.0
    det_channel_offset: float = 0.0
    use_curved_detector: bool = False

    is_parallel = False

    @property
    def image_shape(self) -> tuple:
        return (int(self.num_det_rows), int(self.num_det_channels))

    @property
    def panel_y_view(self) -> float:
        return self.source_iso_dist - self.source_detector_dist

    def panel_half_extent(self) -> tuple:
        """Half widths (u, v) of the active panel area in cm."""
        return (self.num_det_channels * self.delta_det_channel / 2, self.num_det_rows * self.delta_det_row / 2)

    def source_position(self, angle: float) -> tuple:
        c, s = math.cos(angle), math.sin(angle)
        return (s * self.source_iso_dist, c * self.source_iso_dist, 0.0)

    def panel_center(self, angle: float) -> tuple:
        c, s = math.cos(angle), math.sin(angle)
        yv = self.panel_y_view
        return (s * yv, c * yv, 0.0)

    def panel_axes(self, angle: float) -> tuple:
        """(u_hat, v_hat, n_hat) at the panel centre; n_hat points toward the source."""
        c, s = math.cos(angle), math.sin(angle)
        return (c, -s, 0.0), (0.0, 0.0, 1.0), (s, c, 0.0)

    def pixel_uv(self) -> tuple:
        """float64 numpy u [channels], v [rows] of the pixel centres."""
        nc, nr = self.num_det_channels, self.num_det_rows
        u = (np.arange(nc) - (nc - 1) / 2) * self.delta_det_channel - self.det_channel_offset
        v = (np.arange(nr) - (nr - 1) / 2) * self.delta_det_row - self.det_row_offset
        return u, v

    def panel_points_np(self, u: np.ndarray, v: np.ndarray, angle: float) -> np.ndarray:
        """float64 [..., 3] positions of panel points (u, v) (reference ``geometry.py:560-592``)."""
        u, v = np.broadcast_arrays(np.asarray(u, dtype=np.float64), np.asarray(v, dtype=np.float64))
        u_hat, v_hat, n_hat = (np.asarray(a) for a in self.panel_axes(angle))
        pc = np.asarray(self.panel_center(angle))
        if not self.use_curved_detector:
            return pc + u[..., None] * u_hat + v[..., None] * v_hat
        radius = float(self.source_detector_dist)
        gamma = u / radius
        return (pc + (radius * np.sin(gamma))[..., None] * u_hat
                + (2.0 * radius * np.sin(0.5 * gamma) ** 2)[..., None] * n_hat
                + (v * np.cos(gamma))[..., None] * v_hat)

    def pixel_centers_np(self, angle: float) -> np.ndarray:
        """float64 [rows, channels, 3] pixel-centre positions."""
        u, v = self.pixel_uv()
        return self.panel_points_np(u[None, :], v[:, None], angle)

    def pixel_centers(self, angle: float, device=None, dtype=torch.float32) -> Tensor:
        return torch.as_tensor(self.pixel_centers_np(angle), device=device, dtype=dtype)

    def local_normals_np(self, points: np.ndarray, angle: float) -> np.ndarray:
        """float64 [..., 3] inward-pointing (toward the source axis) unit normals n_hat at panel points."""
        points = np.asarray(points, dtype=np.float64)
        n_hat = np.asarray(self.panel_axes(angle)[2])
        if not self.use_curved_detector:
            return np.broadcast_to(n_hat, points.shape).copy()
        to_axis = np.asarray(self.source_position(angle)) - points
        to_axis[..., 2] = 0.0
        return to_axis / np.linalg.norm(to_axis, axis=-1, keepdims=True)

    def local_panel_axes_np(self, points: np.ndarray, angle: float) -> tuple:
        """float64 (u_hat, v_hat, n_hat) [..., 3] of the panel surface at panel points (reference
        ``geometry.py:624-646``): the panel axes on a flat panel; on a curved one the horizontal normal toward the
        cylinder axis, the vertical v_hat and u_hat = n_hat x v_hat along the arc."""
        points = np.asarray(points, dtype=np.float64)
        u_hat, v_hat, n_hat = (np.broadcast_to(np.asarray(a, dtype=np.float64), points.shape)
                               for a in self.panel_axes(angle))
        if not self.use_curved_detector:
            return u_hat, v_hat, n_hat
        to_axis = np.asarray(self.source_position(angle)) - points
        to_axis = to_axis - (to_axis * v_hat).sum(-1, keepdims=True) * v_hat
        n_local = to_axis / np.linalg.norm(to_axis, axis=-1, keepdims=True)
        return np.cross(n_local, v_hat), v_hat, n_local

    def panel_distance_along_np(self, points: np.ndarray, omega: np.ndarray, angle: float) -> np.ndarray:
        """Distance t with ``points + t omega`` on the panel surface (reference ``geometry.py:673-732``)."""
        points = np.asarray(points, dtype=np.float64)
        omega = np.asarray(omega, dtype=np.float64)
        if not self.use_curved_detector:
            n = np.asarray(self.panel_axes(angle)[2])
            pc = np.asarray(self.panel_center(angle))
            with np.errstate(divide="ignore", invalid="ignore"):
                return ((pc - points) * n).sum(-1) / (omega * n).sum(-1)
        src = np.asarray(self.source_position(angle))
        d = (points - src)[..., :2]
        w = omega[..., :2]
        a = (w * w).sum(-1)
        b = (d * w).sum(-1)
        c = (d * d).sum(-1) - float(self.source_detector_dist) ** 2
        a, b, c = np.broadcast_arrays(a, b, c)
        disc = b * b - a * c
        root = np.sqrt(np.clip(disc, 0.0, None))
        pos = b >= 0
        den = np.where(pos, b + root, np.where(a > 0, a, 1.0))
        num = np.where(pos, -c, root - b)
        with np.errstate(divide="ignore", invalid="ignore"):
            t = num / np.where(den != 0, den, 1.0)
        return np.where((a > 0) & (disc >= 0) & (den != 0), t, np.inf)

    def panel_uv_of_points_np(self, points: np.ndarray, angle: float) -> tuple:
        """Panel coordinates of points on the panel surface (reference ``geometry.py:734-762``)."""
        points = np.asarray(points, dtype=np.float64)
        u_hat, v_hat, n_hat = (np.asarray(a) for a in self.panel_axes(angle))
        if self.use_curved_detector:
            d = points - np.asarray(self.source_position(angle))
            depth = -(d * n_hat).sum(-1)
            radius = float(self.source_detector_dist)
            return radius * np.arctan2((d * u_hat).sum(-1), depth), radius * (d * v_hat).sum(-1) / depth
        d = points - np.asarray(self.panel_center(angle))
        return (d * u_hat).sum(-1), (d * v_hat).sum(-1)
