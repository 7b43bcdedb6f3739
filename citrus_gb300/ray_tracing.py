"""The ``Projectors`` protocol and its sm_103a implementation (mirrors ``citrus/scatter_solver/ray_tracing.py``).

``Projectors`` is the plugin point of the solver (``ScatterSolver(projectors=...)``): five ray operations for one view
angle, batched over a leading channel axis (groups or materials), the field zero outside its grid box.
``GB300Projectors`` runs each operation as one kernel of ``libcitrus_gb300.so`` (``csrc/raytrace.cu``); the volumes
are handed to the kernels voxel-major ([V, C], every channel of a voxel in one load).
"""

from __future__ import annotations

import ctypes
import math
from typing import Optional, Protocol

import numpy as np
import torch
from torch import Tensor

from . import _lib
from .geometry import ConeGeometry, Grid

_PIXELS: dict = {}   # (geometry, angle, device) -> float64 [Rd Cd, 3] pixel centres on the device
_PIXELS_MAX = 512


def _pixel_centers(geometry: ConeGeometry, angle: float, device) -> Tensor:
    """The panel's pixel centres at ``angle`` on ``device``, uploaded once per (geometry, angle) and kept (so that a
    captured CUDA graph reads a buffer that stays put)."""
    key = (geometry, float(angle), str(torch.device(device)))
    t = _PIXELS.get(key)
    if t is None:
        if len(_PIXELS) >= _PIXELS_MAX:
            _PIXELS.pop(next(iter(_PIXELS)))
        t = _lib.upload(geometry.pixel_centers_np(angle).reshape(-1, 3), device, torch.float64)
        _PIXELS[key] = t
    return t


class Projectors(Protocol):
    """The five ray operations of the scatter solver (reference ``ray_tracing.py:27-115``)."""

    def upstream_cumulative(self, mu: Tensor, grid: Grid, geometry: ConeGeometry, angle: float) -> Tensor: ...

    def upstream_to_points(self, mu: Tensor, grid: Grid, geometry: ConeGeometry, angle: float,
                           points: Tensor) -> Tensor: ...

    def primary_project(self, mu: Tensor, grid: Grid, geometry: ConeGeometry, angle: float) -> Tensor: ...

    def downstream_cumulative(self, mu: Tensor, grid: Grid, geometry: ConeGeometry, angle: float,
                              omegas: Tensor) -> Tensor: ...

    def oblique_project(self, field: Tensor, grid: Grid, geometry: ConeGeometry, angle: float, omegas: Tensor,
                        out: Optional[Tensor] = None) -> Tensor: ...


class HostArgs:
    """Keeps ctypes host arrays alive for one call and hands out their addresses."""

    def __init__(self):
        self._keep = []

    def doubles(self, values) -> int:
        arr = (ctypes.c_double * len(values))(*[float(v) for v in values])
        self._keep.append(arr)
        return ctypes.addressof(arr)

    def int64s(self, values) -> int:
        arr = (ctypes.c_int64 * len(values))(*[int(v) for v in values])
        self._keep.append(arr)
        return ctypes.addressof(arr)

    def pointers(self, addresses) -> int:
        """A host array of device addresses."""
        arr = (ctypes.c_void_p * len(addresses))(*[int(a) for a in addresses])
        self._keep.append(arr)
        return ctypes.addressof(arr)


def _grid_args(host: HostArgs, grid: Grid) -> tuple:
    return host.doubles(list(grid.lower_corner()) + list(grid.deltas)), host.int64s(
        (grid.num_cols, grid.num_rows, grid.num_slices))


def _voxel_major(volume: Tensor, grid: Grid) -> Tensor:
    """[C, R, Cc, S] -> contiguous float32 [V, C]."""
    if volume.dim() != 4 or tuple(volume.shape[1:]) != tuple(grid.shape):
        raise ValueError(f"volume must be [C, {grid.shape}], got {tuple(volume.shape)}")
    if volume.device.type != "cuda" or volume.dtype != torch.float32:
        raise ValueError("volume must be a float32 CUDA tensor")
    return volume.reshape(volume.shape[0], -1).t().contiguous()


def panel_args(host: HostArgs, geometry: ConeGeometry, angle: float) -> int:
    _, _, n_hat = geometry.panel_axes(angle)
    return host.doubles([1.0 if geometry.use_curved_detector else 0.0, *geometry.panel_center(angle), *n_hat,
                         *geometry.source_position(angle), float(geometry.source_detector_dist)])


def subpixel_points(geometry: ConeGeometry, angle: float, n: int) -> np.ndarray:
    """float64 [Rd, Cd, n, n, 3] centres of the n x n sub-pixels of every pixel (reference ``geometry.py:617-634``)."""
    u, v = geometry.pixel_uv()
    offsets = (2 * np.arange(n) + 1) / (2 * n) - 0.5
    u_sub = u[None, :, None, None] + (offsets * geometry.delta_det_channel)[None, None, None, :]
    v_sub = v[:, None, None, None] + (offsets * geometry.delta_det_row)[None, None, :, None]
    return geometry.panel_points_np(u_sub, v_sub, angle)


class GB300Projectors:
    """Exact Siddon projectors on sm_103a (reference ``SiddonProjectors``, ``ray_tracing.py:291-620``).

    Args:
        samples_per_pixel_axis: default sub-rays per pixel axis of ``primary_project``.
    """

    def __init__(self, samples_per_pixel_axis: int = 1):
        if samples_per_pixel_axis < 1:
            raise ValueError("samples_per_pixel_axis must be >= 1")
        self.samples_per_pixel_axis = int(samples_per_pixel_axis)

    # ---- core ---------------------------------------------------------------------------------------------------
    def line_integrals(self, volume: Tensor, starts: Tensor, ends: Tensor, grid: Grid) -> Tensor:
        """[C, R] integrals along starts -> ends ([R, 3]) (reference ``ray_tracing.py:205-244``)."""
        vol = _voxel_major(volume, grid)
        starts = starts.to(device=volume.device, dtype=torch.float32).reshape(-1, 3).contiguous()
        ends = ends.to(device=volume.device, dtype=torch.float32).reshape(-1, 3).contiguous()
        if starts.shape != ends.shape:
            raise ValueError("starts and ends must have the same number of rays")
        out = torch.empty(volume.shape[0], starts.shape[0], device=volume.device, dtype=torch.float32)
        host = HostArgs()
        box, dims = _grid_args(host, grid)
        _lib.call("citrus_line_integrals", vol.data_ptr(), volume.shape[0], box, dims, starts.data_ptr(),
                  ends.data_ptr(), starts.shape[0], out.data_ptr(), _lib.stream_handle(volume.device))
        return out

    def _from_source(self, volume: Tensor, grid: Grid, source, points: Optional[Tensor] = None,
                     point_grid: Optional[Grid] = None) -> Tensor:
        vol = _voxel_major(volume, grid)
        host = HostArgs()
        box, dims = _grid_args(host, grid)
        device = volume.device
        C = volume.shape[0]
        if points is not None:
            pts = points.to(device=device, dtype=torch.float64).reshape(-1, 3).contiguous()
            P = pts.shape[0]
            out = torch.empty(C, P, device=device, dtype=torch.float32)
            _lib.call("citrus_trace_from_source", vol.data_ptr(), C, box, dims, host.doubles(source), pts.data_ptr(),
                      None, None, None, None, P, out.data_ptr(), _lib.stream_handle(device))
            return out
        ax = point_grid.device_axes(device, torch.float64)
        P = point_grid.num_voxels
        out = torch.empty(C, P, device=device, dtype=torch.float32)
        _lib.call("citrus_trace_from_source", vol.data_ptr(), C, box, dims, host.doubles(source), None,
                  ax[0].data_ptr(), ax[1].data_ptr(), ax[2].data_ptr(), host.int64s(point_grid.shape), P,
                  out.data_ptr(), _lib.stream_handle(device))
        return out

    # ---- (a) upstream -------------------------------------------------------------------------------------------
    def upstream_cumulative(self, mu: Tensor, grid: Grid, geometry: ConeGeometry, angle: float) -> Tensor:
        """[C, R, Cc, S] optical depth from the focal spot to every voxel centre."""
        return self._from_source(mu, grid, geometry.source_position(angle), point_grid=grid).reshape(mu.shape)

    def upstream_to_points(self, mu: Tensor, grid: Grid, geometry: ConeGeometry, angle: float,
                           points) -> Tensor:
        """[C, N] from the focal spot to each point; ``points`` is a float [N, 3] tensor or a point ``Grid``."""
        if isinstance(points, Grid):
            return self._from_source(mu, grid, geometry.source_position(angle), point_grid=points)
        return self._from_source(mu, grid, geometry.source_position(angle), points=points)

    # ---- (b) primary --------------------------------------------------------------------------------------------
    def primary_project(self, mu: Tensor, grid: Grid, geometry: ConeGeometry, angle: float,
                        samples_per_pixel_axis: Optional[int] = None) -> Tensor:
        """[C, Rd, Cd] from the focal spot to every pixel centre, or ``-log(mean(exp(-tau)))`` over n x n sub-rays."""
        n = self.samples_per_pixel_axis if samples_per_pixel_axis is None else int(samples_per_pixel_axis)
        Rd, Cd = geometry.image_shape
        if n == 1:
            pts = torch.as_tensor(geometry.pixel_centers_np(angle).reshape(-1, 3))
            return self._from_source(mu, grid, geometry.source_position(angle), points=pts).reshape(-1, Rd, Cd)
        pts = torch.as_tensor(subpixel_points(geometry, angle, n).reshape(-1, 3))
        tau = self._from_source(mu, grid, geometry.source_position(angle), points=pts).reshape(-1, Rd, Cd, n * n)
        return -(torch.logsumexp(-tau, dim=-1) - math.log(n * n))

    # ---- (c) downstream -----------------------------------------------------------------------------------------
    def crossing_tables(self, grid: Grid, omegas: Tensor) -> Tensor:
        """[K, 3 (nx + ny + nz)] int32 crossing tables of the lattice walk for directions [K, 3] on ``grid`` (one
        launch for the whole set; ``downstream_cumulative(crossings=...)`` takes rows of it)."""
        device = omegas.device
        om = omegas.to(dtype=torch.float32).reshape(-1, 3).contiguous()
        K = om.shape[0]
        E = grid.num_rows + grid.num_cols + grid.num_slices
        tables = torch.empty(K, 3 * E, dtype=torch.int32, device=device)
        host = HostArgs()
        box, dims = _grid_args(host, grid)
        _lib.call("citrus_crossing_tables", box, dims, om.data_ptr(), K, tables.data_ptr(), tables.numel(),
                  _lib.stream_handle(device))
        return tables

    def downstream_cumulative(self, mu: Tensor, grid: Grid, geometry: ConeGeometry, angle: float,
                              omegas: Tensor, out: Optional[Tensor] = None, lattice: bool = True,
                              voxel_major: bool = False, crossings: Optional[Tensor] = None) -> Tensor:
        """[K, C, R, Cc, S] from every voxel centre along each direction to the panel; +inf where the direction does
        not face the panel (``omega . (-n_hat) <= 0``), 0 beyond the panel. ``lattice`` walks every ray down its
        direction's shared crossing table (the default), else each ray runs its own walk; ``crossings`` gives those
        tables prebuilt (``crossing_tables`` of these directions on ``grid``). ``voxel_major`` returns the same
        values as a contiguous [K, V, C] tensor (``out`` ignored)."""
        vol = _voxel_major(mu, grid)
        device = mu.device
        omegas = omegas.to(device=device, dtype=torch.float32).reshape(-1, 3).contiguous()
        K = omegas.shape[0]
        n = [float(v) for v in geometry.panel_axes(angle)[2]]
        toward = ((omegas[:, 0] * -n[0] + omegas[:, 1] * -n[1] + omegas[:, 2] * -n[2]) > 0).to(torch.uint8)
        C, V = int(mu.shape[0]), grid.num_voxels
        if voxel_major:
            out = torch.empty(K, V, C, device=device, dtype=torch.float32)
            strides = (V * C, 1, C)
        else:
            if out is None:
                out = torch.empty(K, *mu.shape, device=device, dtype=torch.float32)
            if tuple(out.shape) != (K, *mu.shape) or out.dtype != torch.float32 or not out.is_contiguous():
                raise ValueError(f"out must be a contiguous float32 tensor of shape {(K, *mu.shape)}")
            strides = (C * V, V, 1)
        host = HostArgs()
        box, dims = _grid_args(host, grid)
        diagonal = math.sqrt(sum(e * e for e in grid.extent)) * (1 + 1e-9) + 1e-9
        E = grid.num_rows + grid.num_cols + grid.num_slices
        if crossings is not None:
            if (crossings.dtype != torch.int32 or not crossings.is_contiguous()
                    or tuple(crossings.shape) != (K, 3 * E) or crossings.device != device):
                raise ValueError(f"crossings must be the contiguous int32 [{K}, {3 * E}] tables of these directions")
            _lib.call("citrus_downstream_cumulative_tables", vol.data_ptr(), mu.shape[0], box, dims,
                      omegas.data_ptr(), toward.data_ptr(), K, panel_args(host, geometry, angle), diagonal,
                      out.data_ptr(), *strides, crossings.data_ptr(), crossings.numel(), _lib.stream_handle(device))
            return out
        crossings = torch.empty(3 * E * K, dtype=torch.int32, device=device) if lattice else None
        _lib.call("citrus_downstream_cumulative", vol.data_ptr(), mu.shape[0], box, dims, omegas.data_ptr(),
                  toward.data_ptr(), K, panel_args(host, geometry, angle), diagonal, out.data_ptr(), *strides,
                  None if crossings is None else crossings.data_ptr(), 0 if crossings is None else crossings.numel(),
                  _lib.stream_handle(device))
        return out

    # ---- (d) oblique --------------------------------------------------------------------------------------------
    def oblique_project(self, field: Tensor, grid: Grid, geometry: ConeGeometry, angle: float, omegas: Tensor,
                        out: Optional[Tensor] = None, voxel_major: bool = False) -> Tensor:
        """[K, C, Rd, Cd] line integrals through every pixel centre along each direction (``out`` any strides).

        ``field`` is [K, C, R, Cc, S] or [C, R, Cc, S] (shared), or with ``voxel_major`` already [K, V, C]."""
        device = field.device
        omegas = omegas.to(device=device, dtype=torch.float32).reshape(-1, 3).contiguous()
        K = omegas.shape[0]
        if voxel_major:
            if field.dim() != 3 or field.shape[1] != grid.num_voxels or not field.is_contiguous():
                raise ValueError("a voxel-major field must be contiguous [K, V, C]")
            vol, C, stride = field, int(field.shape[2]), int(field.shape[1] * field.shape[2])
        elif field.dim() == 4:
            vol, C, stride = _voxel_major(field, grid), int(field.shape[0]), 0
        elif field.dim() == 5 and field.shape[0] == K:
            if tuple(field.shape[2:]) != tuple(grid.shape):
                raise ValueError(f"field spatial shape {tuple(field.shape[2:])} != grid shape {grid.shape}")
            C = int(field.shape[1])
            vol = field.reshape(K, C, -1).permute(0, 2, 1).contiguous()
            stride = grid.num_voxels * C
        else:
            raise ValueError(f"field must be [C, ...] or [K={K}, C, ...], got {tuple(field.shape)}")
        Rd, Cd = geometry.image_shape
        pixels = _pixel_centers(geometry, angle, device)
        if out is None:
            out = torch.empty(K, C, Rd, Cd, device=device, dtype=torch.float32)
        if tuple(out.shape) != (K, C, Rd, Cd):
            raise ValueError(f"out must be [K, C, Rd, Cd] = {(K, C, Rd, Cd)}, got {tuple(out.shape)}")
        host = HostArgs()
        box, dims = _grid_args(host, grid)
        scratch_bytes = int(_lib.library().citrus_oblique_scratch_bytes(K))
        scratch = torch.empty(max(1, scratch_bytes), device=device, dtype=torch.uint8)  # per-direction constants
        _lib.call("citrus_oblique_project_scratch", vol.data_ptr(), C, stride, box, dims, omegas.data_ptr(), K,
                  pixels.data_ptr(), Rd, Cd, out.data_ptr(), out.stride(0), out.stride(1), out.stride(2),
                  out.stride(3), scratch.data_ptr(), scratch_bytes, _lib.stream_handle(device))
        return out
