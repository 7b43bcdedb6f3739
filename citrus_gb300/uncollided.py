"""Uncollided fluence and first-collision source of one view (mirrors ``citrus/scatter_solver/uncollided.py``).

The uncollided fluence is exact in energy within each group: the upstream density line integrals of the present
materials (``Projectors.upstream_to_points``) feed the fine-energy transmission, times the focal-spot weight
``b(Omega) / |r - r0|^2`` (one fused launch, ``citrus_group_transmission`` with the factor of
``citrus_source_weight``). The first-collision source is evaluated from the per-steradian transfer table at the angle
between the primary direction and each direction (``citrus_first_collision_source``), corrected so that the sweep
quadrature reproduces its exact l = 0, 1 moments (``citrus_first_collision_correction``: sums and float64 factors in
one kernel) and restricted to linear-discontinuous moments per transport cell, cell-major, straight into the sweep's
store (``citrus_first_collision_moments``).
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Optional, Sequence

import numpy as np
import torch
from torch import Tensor

from . import _lib
from .cross_sections import MultigroupLibrary
from .geometry import ConeGeometry, Grid
from .ray_tracing import HostArgs
from .responses import SourceModel


def present_materials(rho: Tensor) -> Optional[list]:
    """Indices of the materials with a nonzero density, or None for all (reference ``uncollided.py:27-45``)."""
    M = int(rho.shape[0])
    if M <= 2:
        return None
    present = [int(i) for i in torch.nonzero(rho.reshape(M, -1).ne(0).any(1)).flatten().tolist()]
    return None if len(present) == M else (present if present else [0])


# ---- device tables of the library ---------------------------------------------------------------------------------

def transfer_table(library: MultigroupLibrary, device) -> Tensor:
    """[M, N, G_out, G_in] float32 per-steradian transfer, zero for upscatter (the kernels' layout)."""
    key = ("transfer_table", str(device))
    t = library._device_cache.get(key)
    if t is None:
        G = library.num_groups
        tab = library.mu_s_eta * np.triu(np.ones((G, G)))[None, :, :, None]          # [M, Gi, Go, N]
        t = torch.as_tensor(np.ascontiguousarray(tab.transpose(0, 3, 2, 1)), dtype=torch.float32).to(device)
        library._device_cache[key] = t
    return t


def moment_table(library: MultigroupLibrary, device) -> Tensor:
    """[M, 2, G_out, G_in] float32 Legendre transfer moments l = 0, 1, zero for upscatter."""
    key = ("moment_table", str(device))
    t = library._device_cache.get(key)
    if t is None:
        if library.legendre_order < 1:
            raise ValueError("the sampling correction needs Legendre moments of order >= 1")
        G = library.num_groups
        mom = library.mu_s_l[..., :2] * np.triu(np.ones((G, G)))[None, :, :, None]   # [M, Gi, Go, 2]
        t = torch.as_tensor(np.ascontiguousarray(mom.transpose(0, 3, 2, 1)), dtype=torch.float32).to(device)
        library._device_cache[key] = t
    return t


def point_axes(grid: Grid, device) -> Tensor:
    """float32 x [cols], y [rows], z [slices] of a point grid, back to back (as the kernels read them)."""
    return torch.cat(grid.device_axes(device, torch.float32))


def _eta_range(library: MultigroupLibrary) -> tuple:
    eta = library.eta_grid
    uniform = np.allclose(np.diff(eta), eta[1] - eta[0], rtol=1e-9, atol=1e-12)
    if not uniform:
        raise NotImplementedError("only uniform cosine tables are supported")
    return float(eta[0]), float(eta[-1]), int(eta.size)


# ---- uncollided fluence -------------------------------------------------------------------------------------------

def source_field(source: SourceModel, geometry: ConeGeometry, angle: float, points: Grid, device,
                 divide_by_distance_squared: bool = True) -> tuple:
    """([V] b(Omega) / |r - r0|^2, [V] filter path in g/cm^2 or None) at the centres of a point grid (reference
    ``source.py:368-430`` at ``uncollided.py:183-197``)."""
    host = HostArgs()
    ax = points.device_axes(device, torch.float64)
    out = torch.empty(points.num_voxels, device=device, dtype=torch.float32)
    tables = source.device_tables(geometry, angle, device)
    thickness = tables["thickness"]
    path = None if thickness is None else torch.empty(points.num_voxels, device=device, dtype=torch.float32)
    ptr = lambda t: None if t is None else t.data_ptr()  # noqa: E731
    extras = tables["profile"] is not None or thickness is not None
    _lib.call("citrus_source_field", host.doubles(source.field_args(geometry, angle)),
              host.doubles(source.panel_args(geometry)) if extras else None, ptr(tables["profile"]), ptr(thickness),
              0 if thickness is None else int(thickness.shape[0]), source.filter_density, ptr(tables["off_nodes"]),
              ptr(tables["off_values"]), 0 if tables["off_nodes"] is None else int(tables["off_nodes"].numel()), None,
              ax[0].data_ptr(), ax[1].data_ptr(), ax[2].data_ptr(), host.int64s(points.shape), points.num_voxels,
              int(divide_by_distance_squared), out.data_ptr(), ptr(path), _lib.stream_handle(device))
    return out, path


def source_weight(source: SourceModel, geometry: ConeGeometry, angle: float, points: Grid, device,
                  divide_by_distance_squared: bool = True) -> Tensor:
    """[V] b(Omega) / |r - r0|^2 at the centres of a point grid."""
    return source_field(source, geometry, angle, points, device, divide_by_distance_squared)[0]


def group_transmission(library: MultigroupLibrary, path: Tensor, materials: Optional[Sequence[int]] = None,
                       factor: Optional[Tensor] = None, filter_path: Optional[Tensor] = None,
                       filter_attenuation=None) -> Tensor:
    """[G, ...] fine-energy group transmission of line integrals path [M', ...] in g/cm^2, times ``factor`` [...]
    (reference ``cross_sections.py:797-883``); a beam filter adds ``filter_attenuation[e] * filter_path`` to each
    exponent (``transmission_kernels.py:187-275``)."""
    device = path.device
    Mp = int(path.shape[0])
    spatial = tuple(path.shape[1:])
    P = int(np.prod(spatial)) if spatial else 1
    fine_mu = library.fine_mu_t if materials is None else library.fine_mu_t[list(materials)]
    if fine_mu.shape[0] != Mp:
        raise ValueError(f"path has {Mp} materials, the library {fine_mu.shape[0]}")
    if (filter_path is None) != (filter_attenuation is None):
        raise ValueError("filter_path and filter_attenuation go together")
    key = ("fine", None if materials is None else tuple(int(m) for m in materials), str(device))
    cached = library._device_cache.get(key)
    if cached is None:
        cached = (torch.as_tensor(np.ascontiguousarray(fine_mu), dtype=torch.float32).to(device),
                  library.tensor("fine_weight", device),
                  torch.as_tensor(library.fine_group.astype(np.int32)).to(device))
        library._device_cache[key] = cached
    mu, w, g = cached
    p = path.to(torch.float32).reshape(Mp, P).contiguous()
    G = library.num_groups
    out = torch.empty(G, P, device=device, dtype=torch.float32)
    fac = None if factor is None else factor.to(torch.float32).reshape(P).contiguous()
    fp = fmu = None
    if filter_path is not None:
        fp = filter_path.to(device=device, dtype=torch.float32).reshape(P).contiguous()
        fmu = torch.as_tensor(np.asarray(filter_attenuation, dtype=np.float64), dtype=torch.float32).to(device)
        if fmu.numel() != w.numel():
            raise ValueError(f"filter_attenuation has {fmu.numel()} energies, the library {w.numel()}")
    _lib.call("citrus_group_transmission", p.data_ptr(), Mp, P, mu.data_ptr(), w.data_ptr(), g.data_ptr(),
              int(w.numel()), G, None if fp is None else fp.data_ptr(), None if fmu is None else fmu.data_ptr(),
              None if fac is None else fac.data_ptr(), out.data_ptr(), _lib.stream_handle(device))
    return out.reshape(G, *spatial)


def uncollided_path_lengths(projectors, rho: Tensor, grid: Grid, geometry: ConeGeometry, angle: float,
                            points: Optional[Grid] = None) -> Tensor:
    """[M', *points.shape] upstream density line integrals (reference ``uncollided.py:134-157``)."""
    point_grid = grid if points is None else points
    if point_grid == grid:
        return projectors.upstream_cumulative(rho, grid, geometry, angle)
    return projectors.upstream_to_points(rho, grid, geometry, angle, point_grid).reshape(-1, *point_grid.shape)


def uncollided_from_path_lengths(library: MultigroupLibrary, path_lengths: Tensor, materials, points: Grid,
                                 geometry: ConeGeometry, angle: float, source: SourceModel) -> Tensor:
    """[G, *points.shape] phi_UC = b / |r - r0|^2 sum_e w_e exp(-sum_m P_m mu_m(e)) (reference ``uncollided.py:160-197``)."""
    factor, filter_path = source_field(source, geometry, angle, points, path_lengths.device)
    return group_transmission(library, path_lengths, materials, factor, filter_path,
                              source.filter_attenuation(library) if filter_path is not None else None)


def uncollided_fluence(library: MultigroupLibrary, rho: Tensor, grid: Grid, geometry: ConeGeometry, angle: float,
                       source: SourceModel, projectors, points: Optional[Grid] = None, materials="auto") -> Tensor:
    """[G, *points.shape] uncollided fluence at the point centres (reference ``uncollided.py:99-131``)."""
    point_grid = grid if points is None else points
    present = present_materials(rho) if isinstance(materials, str) else (None if materials is None
                                                                        else [int(m) for m in materials])
    traced = rho if present is None else rho[present]
    path = uncollided_path_lengths(projectors, traced.contiguous(), grid, geometry, angle, point_grid)
    return uncollided_from_path_lengths(library, path, present, point_grid, geometry, angle, source)


# ---- first-collision source ---------------------------------------------------------------------------------------

@dataclass(frozen=True, eq=False)
class FirstCollisionSamplingCorrection:
    """Per-point, per-group ``scale`` and ``beta`` [G, R, C, S] of ``S <- scale S (1 + beta Omega . Omega_UC)``
    (reference ``uncollided.py:382-411``); ``sums`` [5, G, R, C, S] holds I0, I1, I2, E0, E1 when kept, and ``cache``
    the first-collision source at the correction's directions, which the LD moments of the sweep's source read back."""

    scale: Tensor
    beta: Tensor
    sums: Optional[Tensor] = None
    cache: Optional[Tensor] = None  # [K, G, V] source values at the correction's directions, when kept


class _FCArgs:
    """The shared pointer/size arguments of the first-collision entry points for one view."""

    def __init__(self, library: MultigroupLibrary, rho: Tensor, phi_uncollided: Tensor, grid: Grid,
                 geometry: ConeGeometry, angle: float):
        device = phi_uncollided.device
        if tuple(rho.shape[1:]) != tuple(grid.shape) or tuple(phi_uncollided.shape[1:]) != tuple(grid.shape):
            raise ValueError("rho and phi_uncollided must live on the point grid")
        if rho.shape[0] != library.num_materials or phi_uncollided.shape[0] != library.num_groups:
            raise ValueError("rho / phi_uncollided do not match the library's materials / groups")
        self.host = HostArgs()
        self.device = device
        self.rho = rho.to(torch.float32).reshape(rho.shape[0], -1).contiguous()
        self.phi = phi_uncollided.to(torch.float32).reshape(phi_uncollided.shape[0], -1).contiguous()
        self.axes = point_axes(grid, device)
        self.dims = self.host.int64s(grid.shape)
        self.focal = self.host.doubles(geometry.source_position(angle))
        self.table = transfer_table(library, device)
        self.eta_lo, self.eta_hi, self.num_eta = _eta_range(library)
        self.M, self.G = library.num_materials, library.num_groups
        self.V = grid.num_voxels
        self.stream = _lib.stream_handle(device)

    def common(self) -> tuple:
        return (self.rho.data_ptr(), self.M, self.phi.data_ptr(), self.G, self.axes.data_ptr(), self.dims)


def first_collision_sampling_correction(library: MultigroupLibrary, rho: Tensor, phi_uncollided: Tensor, grid: Grid,
                                        geometry: ConeGeometry, angle: float, omegas: Tensor, weights: Tensor,
                                        keep_sums: bool = False,
                                        keep_cache: bool = False) -> FirstCollisionSamplingCorrection:
    """Factors that make the sweep quadrature integrate the sampled first-collision source exactly for l = 0, 1
    (reference ``uncollided.py:414-461``); ``keep_cache`` keeps the source values [K, G, V] as well."""
    a = _FCArgs(library, rho, phi_uncollided, grid, geometry, angle)
    om = omegas.to(device=a.device, dtype=torch.float32).reshape(-1, 3).contiguous()
    w = weights.to(device=a.device, dtype=torch.float32).reshape(-1).contiguous()
    scale = torch.empty(a.G, *grid.shape, device=a.device)
    beta = torch.empty_like(scale)
    sums = torch.empty(5, a.G, *grid.shape, device=a.device) if keep_sums else None
    cache = torch.empty(om.shape[0], a.G, a.V, device=a.device) if keep_cache else None
    _lib.call("citrus_first_collision_correction", *a.common(), a.focal, a.table.data_ptr(), a.num_eta, a.eta_lo,
              a.eta_hi, om.data_ptr(), w.data_ptr(), om.shape[0], moment_table(library, a.device).data_ptr(),
              None if sums is None else sums.data_ptr(), scale.data_ptr(), beta.data_ptr(),
              None if cache is None else cache.data_ptr(), a.stream)
    return FirstCollisionSamplingCorrection(scale, beta, sums, cache)


def first_collision_source_at_directions(library: MultigroupLibrary, rho: Tensor, phi_uncollided: Tensor, grid: Grid,
                                         geometry: ConeGeometry, angle: float, omegas: Tensor) -> Tensor:
    """[K, G, R, C, S] first-collision source at the point centres (reference ``uncollided.py:200-233``)."""
    a = _FCArgs(library, rho, phi_uncollided, grid, geometry, angle)
    om = omegas.to(device=a.device, dtype=torch.float32).reshape(-1, 3).contiguous()
    out = torch.empty(om.shape[0], a.G, *grid.shape, device=a.device)
    _lib.call("citrus_first_collision_source", *a.common(), a.focal, a.table.data_ptr(), a.num_eta, a.eta_lo, a.eta_hi,
              om.data_ptr(), om.shape[0], out.data_ptr(), a.stream)
    return out


def first_collision_means_at_directions(library: MultigroupLibrary, rho: Tensor, phi_uncollided: Tensor, grid: Grid,
                                        geometry: ConeGeometry, angle: float, omegas: Tensor,
                                        correction: FirstCollisionSamplingCorrection, direction_index: Tensor,
                                        out: Optional[Tensor] = None) -> Tensor:
    """[K, NC, G] means of the LD moments of the corrected source with one point per cell (whose slopes vanish), read
    from the correction's cached source values: the first components of ``first_collision_moments_at_directions``
    (reference ``uncollided.py:464-511``), for the fused source expansion of an accumulator sweep."""
    if correction.cache is None:
        raise ValueError("the correction did not keep its source values")
    a = _FCArgs(library, rho, phi_uncollided, grid, geometry, angle)
    om = omegas.to(device=a.device, dtype=torch.float32).reshape(-1, 3).contiguous()
    K = om.shape[0]
    index = direction_index.to(device=a.device, dtype=torch.int32).reshape(-1).contiguous()
    if index.numel() != K:
        raise ValueError("direction_index must give one cache row per direction")
    expected = (K, a.V, a.G)
    if out is None:
        out = torch.empty(expected, device=a.device)
    elif out.numel() != K * a.V * a.G or not out.is_contiguous() or out.dtype != torch.float32:
        raise ValueError(f"out must be a contiguous float32 tensor of {K * a.V * a.G} elements")
    scale, beta = correction.scale.contiguous(), correction.beta.contiguous()  # bound until the call is queued
    _lib.call("citrus_first_collision_means", a.G, a.axes.data_ptr(), a.dims, a.focal, om.data_ptr(), K,
              scale.data_ptr(), beta.data_ptr(), correction.cache.data_ptr(), index.data_ptr(), out.data_ptr(),
              a.V * a.G, a.stream)
    return out.view(expected)


def first_collision_moments_at_directions(library: MultigroupLibrary, rho: Tensor, phi_uncollided: Tensor, grid: Grid,
                                          geometry: ConeGeometry, angle: float, omegas: Tensor,
                                          correction: FirstCollisionSamplingCorrection, factor: int,
                                          out: Optional[Tensor] = None, cell_major: bool = True,
                                          direction_index: Optional[Tensor] = None) -> Tensor:
    """LD moments of the corrected source per cell (reference ``uncollided.py:464-511``): cell-major
    [K, Rc, Cc, Sc, G, 4] (the sweep's layout, written into ``out`` when given) or [K, G, 4, Rc, Cc, Sc]. When the
    correction kept its source values and ``direction_index`` gives the rows of ``omegas`` among the correction's
    directions, the values are read back instead of evaluated again."""
    a = _FCArgs(library, rho, phi_uncollided, grid, geometry, angle)
    f = int(factor)
    coarse = grid.coarsen(f)
    om = omegas.to(device=a.device, dtype=torch.float32).reshape(-1, 3).contiguous()
    K = om.shape[0]
    expected = (K, *coarse.shape, a.G, 4)
    if out is None:
        out = torch.empty(expected, device=a.device)
    elif tuple(out.shape) != expected or not out.is_contiguous() or out.dtype != torch.float32:
        raise ValueError(f"out must be a contiguous float32 tensor of shape {expected}")
    scale = correction.scale.contiguous()
    beta = correction.beta.contiguous()
    cache = index = None
    if correction.cache is not None and direction_index is not None:
        cache = correction.cache
        index = direction_index.to(device=a.device, dtype=torch.int32).reshape(-1).contiguous()
        if index.numel() != K:
            raise ValueError("direction_index must give one cache row per direction")
    _lib.call("citrus_first_collision_moments", *a.common(), f, a.focal, a.table.data_ptr(), a.num_eta, a.eta_lo,
              a.eta_hi, om.data_ptr(), K, scale.data_ptr(), beta.data_ptr(), None if cache is None else cache.data_ptr(),
              None if index is None else index.data_ptr(), out.data_ptr(), coarse.num_voxels * a.G * 4, a.stream)
    return out if cell_major else out.permute(0, 4, 5, 1, 2, 3)
