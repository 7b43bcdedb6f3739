"""The assembled scatter solver of one view (mirrors ``citrus/scatter_solver/scatter_solver.py``).

``ScatterSolver`` keeps the reference's stage methods — material fields, uncollided fluence, first-collision sampling
correction and moment source, scattering-moment source, transport sweep, source iteration, multiple-collision moments,
scatter image, primary, ``solve_view`` — so that the per-view CITRUS step (``citrus_step``) calls the same surface.
Every stage runs on the device through ``libcitrus_gb300.so``; the caches of the reference (transport grids, sweep
contexts, cone direction sets, direction contexts) are kept, sized for a GB300 (an 8 GiB sweep store per chunk and
up to 64 image directions per chunk instead of the reference's 512 MiB and 32).
"""

from __future__ import annotations

import time
from collections import OrderedDict
from contextlib import contextmanager
from dataclasses import dataclass, field
from typing import Optional

import numpy as np
import torch
from torch import Tensor

from . import kernels
from .cross_sections import MultigroupLibrary, mu_t_volume, transfer_moments_volume
from .geometry import ConeGeometry, Grid, resample_conservative
from .quadrature import Quadrature, product_quadrature
from .ray_tracing import GB300Projectors
from .responses import DetectorResponse, GridResponse, SourceModel, group_averaged_responses
from .scatter_image import (combined_scatter_image, make_direction_context, panel_direction_set, primary_image,
                            scatter_fraction)
from .source_iteration import (SourceIterationResult, multiple_collision_source_moments, scatter_moments,
                               scatter_source_function, source_iteration)
from .transport_sweep import SweepContext, make_sweep_context, sweep
from .uncollided import (FirstCollisionSamplingCorrection, first_collision_means_at_directions,
                         first_collision_moments_at_directions, first_collision_sampling_correction,
                         present_materials, uncollided_fluence)

SWEEP_CHUNK_BUDGET_BYTES = 8 * 2 ** 30
IMAGE_CHUNK_BUDGET_BYTES = 4 * 2 ** 30
IMAGE_CHUNK_MAX_DIRECTIONS = 64


@dataclass(frozen=True)
class SolverConfig:
    """The discretization parameters of the path (reference ``config.py:20-222``, the fields the per-view step reads)."""

    num_groups: int = 6
    legendre_order: int = 7
    num_polar: int = 8
    num_azimuthal: int = 16
    transport_cell_cm: float = 1.0
    quadrature_point_spacing_cm: float = 0.5
    uncollided_trace_grid: str = "quadrature"
    source_iteration_tolerance: float = 1.0e-3
    max_source_iterations: int = 30
    cone_num_polar: int = 16
    cone_num_azimuthal: int = 32
    direction_chunk: int = 8
    dtype: str = "float32"
    moment_precision: str = "fp32"  # the spherical-harmonic products: "fp32" or "bf16x3" (tensor-core hi/lo split)
    group_averaged_responses: bool = False  # the responses as their means over each group's fine energies

    def quadrature_points(self, fine_voxel_cm: float) -> int:
        """q = min(max(1, round(cell / spacing)), max(1, round(cell / voxel))) (reference ``config.py:130-144``)."""
        cell = float(self.transport_cell_cm)
        target = max(1, round(cell / float(self.quadrature_point_spacing_cm)))
        return min(target, max(1, round(cell / float(fine_voxel_cm))))

    def validate(self) -> None:
        L = self.legendre_order
        if L < 0:
            raise ValueError("legendre_order must be >= 0")
        if self.num_polar < L + 1:
            raise ValueError(f"num_polar={self.num_polar} must be >= legendre_order+1={L + 1}")
        if self.num_azimuthal < 2 * L + 1:
            raise ValueError(f"num_azimuthal={self.num_azimuthal} must be >= 2*legendre_order+1={2 * L + 1}")
        if self.num_polar % 2 or self.num_azimuthal % 4:
            raise ValueError("the sweep set needs an even num_polar and num_azimuthal divisible by 4")
        if self.moment_precision not in kernels.PRECISIONS:
            raise ValueError(f"moment_precision must be one of {kernels.PRECISIONS}")
        if self.uncollided_trace_grid not in ("coarse", "quadrature", "fine"):
            raise ValueError(f"uncollided_trace_grid must be 'coarse', 'quadrature' or 'fine'")
        if self.max_source_iterations < 1 or self.source_iteration_tolerance <= 0:
            raise ValueError("need max_source_iterations >= 1 and source_iteration_tolerance > 0")
        if self.cone_num_polar < 1 or self.cone_num_azimuthal < 1 or self.direction_chunk < 1:
            raise ValueError("cone counts and direction_chunk must be >= 1")
        if self.dtype != "float32":
            raise ValueError("the GB300 path computes in float32 (the oracle is the float64 reference)")
        if not isinstance(self.group_averaged_responses, bool):
            raise ValueError(f"group_averaged_responses must be True or False, got {self.group_averaged_responses!r}")


@dataclass(frozen=True, eq=False)
class MaterialFields:
    """Density-only fields of a volume on the fine, transport and quadrature grids (reference ``:154-227``)."""

    grid_fine: Grid
    grid_coarse: Grid
    grid_quadrature: Grid
    q: int
    rho_fine: Tensor
    rho_coarse: Tensor
    rho_quadrature: Tensor
    mu_t_coarse: Tensor
    mu_s_l_coarse: Tensor
    traced_materials: Optional[tuple] = None


@dataclass
class ViewResult:
    """Images of one view (reference ``scatter_solver.py:234-307``)."""

    angle: float
    primary: dict
    scatter: dict
    scatter_signal: Tensor
    scatter_fraction: Tensor
    source_iteration_result: SourceIterationResult
    phi_total: Optional[Tensor] = None
    timings: dict = field(default_factory=dict)


class ScatterSolver:
    """Deterministic CT scatter solver of a cone beam, one view at a time, on sm_103a (reference ``:314-1394``)."""

    def __init__(self, library: MultigroupLibrary, config: SolverConfig, geometry: ConeGeometry, projectors=None,
                 detector: Optional[DetectorResponse] = None, grid_response: Optional[GridResponse] = None,
                 source: Optional[SourceModel] = None, device="cuda", direction_context_cache_size: int = 128,
                 primary_samples_per_pixel_axis: Optional[int] = None):
        if detector is None or grid_response is None:
            raise TypeError("ScatterSolver needs a detector and a grid_response")
        config.validate()
        if library.legendre_order < config.legendre_order:
            raise ValueError(f"library Legendre order {library.legendre_order} < {config.legendre_order}")
        if library.num_groups != config.num_groups:
            raise ValueError(f"library has {library.num_groups} groups, the configuration {config.num_groups}")
        self.config = config
        self.L = int(config.legendre_order)
        self.device = torch.device(device)
        ok, why = kernels.kernels_usable(self.device)
        if not ok:
            raise RuntimeError(f"the GB300 kernels are unusable on {self.device}: {why}")
        self.library = library
        self.transport_library = library.truncated(self.L)
        self.geometry = geometry
        self.projectors = projectors if projectors is not None else GB300Projectors()
        self.detector = detector
        self.grid_response = grid_response
        self.source = source if source is not None else SourceModel()
        self._averaged_responses = None
        # sub-pixel samples per axis of the primary (n^2 sub-rays per pixel); None: the projector's own, else 1
        self.primary_samples_per_pixel_axis = primary_samples_per_pixel_axis
        self._sweep_contexts: dict = {}
        self._transport_grids: dict = {}
        self._cone_quadratures: dict = {}
        self.direction_context_cache_size = int(direction_context_cache_size)
        self._direction_contexts: OrderedDict = OrderedDict()

    # ---- grids and caches --------------------------------------------------------------------------------------
    @property
    def num_groups(self) -> int:
        return self.library.num_groups

    def quadrature_points(self, grid_fine: Grid) -> int:
        return self.config.quadrature_points(max(grid_fine.deltas))

    def transport_grid(self, grid_fine: Grid) -> Grid:
        g = self._transport_grids.get(grid_fine)
        if g is None:
            g = self._transport_grids[grid_fine] = Grid.covering(grid_fine, self.config.transport_cell_cm)
        return g

    def quadrature_grid(self, grid_fine: Grid) -> Grid:
        return self.transport_grid(grid_fine).refine(self.quadrature_points(grid_fine))

    def sweep_quadrature(self) -> Quadrature:
        return product_quadrature(self.config.num_polar, self.config.num_azimuthal)

    def sweep_context(self, grid_coarse: Grid) -> SweepContext:
        ctx = self._sweep_contexts.get(grid_coarse)
        if ctx is None:
            ctx = make_sweep_context(grid_coarse, self.sweep_quadrature(), self.L, self.device)
            self._sweep_contexts[grid_coarse] = ctx
        return ctx

    def cone_quadrature(self, grid: Grid, angle: float) -> Quadrature:
        key = (grid, float(angle))
        q = self._cone_quadratures.get(key)
        if q is None:
            q = panel_direction_set(self.geometry, angle, (self.config.cone_num_polar, self.config.cone_num_azimuthal),
                                    max_polar_angle=self.transport_grid(grid))
            self._cone_quadratures[key] = q
        return q

    def image_direction_chunk(self, fields: MaterialFields) -> int:
        """Directions per image chunk: as many as fit the budget, between ``direction_chunk`` and 64."""
        G = self.num_groups
        Rd, Cd = self.geometry.image_shape
        per_direction = 4 * G * (2 * fields.grid_quadrature.num_voxels + 2 * fields.grid_coarse.num_voxels
                                 + 3 * Rd * Cd)
        return int(max(self.config.direction_chunk,
                       min(IMAGE_CHUNK_MAX_DIRECTIONS, IMAGE_CHUNK_BUDGET_BYTES // max(1, per_direction))))

    def sweep_direction_chunk(self, fields: MaterialFields) -> int:
        """Directions per octant of a sweep chunk: as many as fit the store budget, in equal chunks."""
        ctx = self.sweep_context(fields.grid_coarse)
        D8 = ctx.directions_per_octant
        per_direction = 8 * ctx.num_cells * 4 * self.num_groups * 4
        largest = max(self.config.direction_chunk, min(D8, SWEEP_CHUNK_BUDGET_BYTES // max(1, per_direction)))
        chunks = -(-D8 // largest)
        return -(-D8 // chunks)

    def direction_context(self, fields: MaterialFields, angle: float, quadrature: Optional[Quadrature] = None):
        quadrature = self.cone_quadrature(fields.grid_fine, angle) if quadrature is None else quadrature
        chunk = self.image_direction_chunk(fields)
        key = (float(angle), id(quadrature), chunk)
        ctx = self._direction_contexts.get(key)
        if ctx is not None and ctx.quadrature is quadrature:
            self._direction_contexts.move_to_end(key)
            return ctx
        ctx = make_direction_context(quadrature, self.geometry, angle, *self.responses(), self.library, self.device,
                                     chunk=chunk)
        if self.direction_context_cache_size > 0:
            self._direction_contexts[key] = ctx
            while len(self._direction_contexts) > self.direction_context_cache_size:
                self._direction_contexts.popitem(last=False)
        return ctx

    # ---- stages -----------------------------------------------------------------------------------------------------
    def material_fields(self, rho_fine: Tensor, grid_fine: Grid) -> MaterialFields:
        """Fields of fine densities on the transport and quadrature grids (reference ``:658-690``)."""
        if tuple(rho_fine.shape[1:]) != tuple(grid_fine.shape):
            raise ValueError(f"rho spatial shape {tuple(rho_fine.shape[1:])} != grid shape {grid_fine.shape}")
        if int(rho_fine.shape[0]) != self.library.num_materials:
            raise ValueError(f"rho has {int(rho_fine.shape[0])} materials, the library {self.library.num_materials}")
        rho = rho_fine.to(device=self.device, dtype=torch.float32).contiguous()
        gc = self.transport_grid(grid_fine)
        q = self.quadrature_points(grid_fine)
        gq = gc.refine(q)
        rho_c = resample_conservative(rho, grid_fine, gc)
        rho_q = rho_c if gq == gc else resample_conservative(rho, grid_fine, gq)
        traced = present_materials(rho_q)
        return MaterialFields(grid_fine, gc, gq, q, rho, rho_c.contiguous(), rho_q.contiguous(),
                              mu_t_volume(self.transport_library, rho_c), transfer_moments_volume(
                                  self.transport_library, rho_c), None if traced is None else tuple(traced))

    def material_fields_from_attenuation(self, X: Tensor, grid_fine: Grid, density_model) -> MaterialFields:
        """The fields of the densities ``density_model(X)``, one material map at a time (reference ``:692-743``).

        Every material map is resampled onto the transport and quadrature grids as it is made; the maps of the
        materials present are kept as the fine densities (the primary traces them). Equals :meth:`material_fields`
        of the stacked maps.
        """
        if tuple(X.shape) != tuple(grid_fine.shape):
            raise ValueError(f"X shape {tuple(X.shape)} != grid shape {grid_fine.shape}")
        X = X.to(device=self.device, dtype=torch.float32).contiguous()
        M = self.library.num_materials
        maps = [density_model.material(X, m) for m in range(M)]
        return self.material_fields(torch.stack(maps), grid_fine)

    def uncollided_fluence(self, fields: MaterialFields, angle: float) -> Tensor:
        """[G, Rq, Cq, Sq] uncollided fluence at the quadrature points (reference ``:745-772``)."""
        trace = self.config.uncollided_trace_grid
        rho, grid = {"fine": (fields.rho_fine, fields.grid_fine),
                     "quadrature": (fields.rho_quadrature, fields.grid_quadrature),
                     "coarse": (fields.rho_coarse, fields.grid_coarse)}[trace]
        return uncollided_fluence(self.library, rho, grid, self.geometry, angle, self.source, self.projectors,
                                  points=fields.grid_quadrature, materials=fields.traced_materials)

    def first_collision_sampling_correction(self, fields: MaterialFields, angle: float, phi_uncollided: Tensor,
                                            sweep_context: Optional[SweepContext] = None
                                            ) -> FirstCollisionSamplingCorrection:
        ctx = self.sweep_context(fields.grid_coarse) if sweep_context is None else sweep_context
        om, w = ctx.omega, ctx.weight
        # keep the source values for the LD moments of the sweep's source when they fit the chunk budget
        keep = om.shape[0] * self.num_groups * fields.grid_quadrature.num_voxels * 4 <= SWEEP_CHUNK_BUDGET_BYTES
        return first_collision_sampling_correction(self.library, fields.rho_quadrature, phi_uncollided,
                                                   fields.grid_quadrature, self.geometry, angle, om, w,
                                                   keep_cache=keep)

    def first_collision_moment_source(self, fields: MaterialFields, angle: float, phi_uncollided: Tensor,
                                      sweep_context: Optional[SweepContext] = None):
        """Cell-major sweep source function of the corrected first-collision source (reference ``:774-826``)."""
        ctx = self.sweep_context(fields.grid_coarse) if sweep_context is None else sweep_context
        omega = ctx.omega
        correction = self.first_collision_sampling_correction(fields, angle, phi_uncollided, ctx)
        library, geometry = self.library, self.geometry

        def source_function(direction_index: Tensor, out: Optional[Tensor] = None) -> Tensor:
            index = direction_index.to(self.device)
            directions = omega.index_select(0, index)
            return first_collision_moments_at_directions(library, fields.rho_quadrature, phi_uncollided,
                                                         fields.grid_quadrature, geometry, angle, directions,
                                                         correction, fields.q, out=out, cell_major=True,
                                                         direction_index=index)

        def means(direction_index: Tensor, out: Optional[Tensor] = None) -> Tensor:
            """[K, NC, G] means of the same moments (one point per cell, cached source values only)."""
            index = direction_index.to(self.device)
            return first_collision_means_at_directions(library, fields.rho_quadrature, phi_uncollided,
                                                       fields.grid_quadrature, geometry, angle,
                                                       omega.index_select(0, index), correction, index, out=out)

        source_function.cell_major = True  # type: ignore[attr-defined]
        # the moments are (mean, 0, 0, 0) quadruples when a cell holds one point and the correction kept its source
        # values: then the means alone describe them
        source_function.means = means if (fields.q == 1 and correction.cache is not None) else None  # type: ignore
        return source_function

    def scatter_moment_source(self, fields: MaterialFields, phi: Tensor,
                              sweep_context: Optional[SweepContext] = None):
        ctx = self.sweep_context(fields.grid_coarse) if sweep_context is None else sweep_context
        return scatter_source_function(ctx, scatter_moments(fields.mu_s_l_coarse, phi),
                                       precision=self.config.moment_precision)

    def transport_sweep(self, fields: MaterialFields, source_function) -> Tensor:
        return sweep(self.sweep_context(fields.grid_coarse), fields.mu_t_coarse, source_function,
                     direction_chunk=self.sweep_direction_chunk(fields), precision=self.config.moment_precision)

    def run_source_iteration(self, fields: MaterialFields, first_collision_source_function) -> SourceIterationResult:
        return source_iteration(self.sweep_context(fields.grid_coarse), fields.mu_t_coarse, fields.mu_s_l_coarse,
                                first_collision_source_function, self.config.source_iteration_tolerance,
                                self.config.max_source_iterations, self.sweep_direction_chunk(fields),
                                precision=self.config.moment_precision)

    def multiple_collision_source_moments(self, fields: MaterialFields, phi_collided: Tensor) -> Tensor:
        return multiple_collision_source_moments(fields.mu_s_l_coarse, phi_collided)

    def scatter_image(self, fields: MaterialFields, angle: float, phi_uncollided: Tensor,
                      scatter_source_moments: Tensor, quadrature: Optional[Quadrature] = None, context=None,
                      signal_only: bool = False) -> dict:
        context = self.direction_context(fields, angle, quadrature) if context is None else context
        return combined_scatter_image(self.library, fields.rho_quadrature, phi_uncollided, fields.grid_quadrature,
                                      fields.q, scatter_source_moments, self.L, self.geometry, angle,
                                      fields.mu_t_coarse, self.projectors, context, fields.grid_coarse,
                                      signal_only=signal_only, rho_coarse=fields.rho_coarse,
                                      attenuation=self.transport_library.tensor("mu_t", self.device),
                                      precision=self.config.moment_precision)

    def primary(self, fields: MaterialFields, angle: float) -> dict:
        return primary_image(self.library, fields.rho_fine, fields.grid_fine, self.geometry, angle, self.source,
                             self.projectors, *self.responses(),
                             samples_per_pixel_axis=self.primary_samples_per_pixel_axis)

    def responses(self) -> tuple:
        """(detector, grid response) the solver evaluates: as given, or with ``config.group_averaged_responses`` their
        means over each group's fine energies, computed once per library and responses (reference
        ``scatter_solver.py:401-415``)."""
        if not self.config.group_averaged_responses:
            return self.detector, self.grid_response
        inputs = (self.detector, self.grid_response, self.library)
        cached = self._averaged_responses
        if cached is None or any(a is not b for a, b in zip(cached[0], inputs)):
            self._averaged_responses = cached = (inputs, group_averaged_responses(*inputs))
        return cached[1]

    # ---- one view ------------------------------------------------------------------------------------------------
    @contextmanager
    def _stage(self, name: str, timings: dict):
        torch.cuda.synchronize(self.device)
        t0 = time.perf_counter()
        yield
        torch.cuda.synchronize(self.device)
        timings[name] = time.perf_counter() - t0

    def solve_view(self, rho_fine: Tensor, grid_fine: Grid, angle: float, keep_phi_total: bool = False,
                   signal_only: bool = False) -> ViewResult:
        """Fields, uncollided fluence, source iteration, image, primary and scatter fraction (reference ``:1038-1123``)."""
        timings: dict = {}
        start = time.perf_counter()
        with self._stage("materials", timings):
            fields = self.material_fields(rho_fine, grid_fine)
        with self._stage("uncollided", timings):
            phi_uc = self.uncollided_fluence(fields, angle)
        with self._stage("source_iteration", timings):
            result = self.run_source_iteration(fields, self.first_collision_moment_source(fields, angle, phi_uc))
        with self._stage("scatter_image", timings):
            T = self.multiple_collision_source_moments(fields, result.phi_total)
            scatter = self.scatter_image(fields, angle, phi_uc, T, signal_only=signal_only)
        with self._stage("primary", timings):
            primary = self.primary(fields, angle)
        timings["total"] = time.perf_counter() - start
        phi_total = result.phi_total if keep_phi_total else None
        if not keep_phi_total:
            result.phi_total = torch.empty(0)
        return ViewResult(float(angle), primary, scatter, scatter["signal"],
                          scatter_fraction(scatter["signal"], primary["signal"]), result, phi_total, timings)
