"""Seeded synthetic workloads of the scatter step: phantoms, spectra, libraries, geometries and solver settings.

Two configurations are defined by their sizes (there is no public dataset behind them; everything is generated here
from seeds):

* ``single_view``: a 32^3 grid of 0.5 cm cells, an axial water cylinder (radius 7 cm, 1.0 g/cc) in air
  (0.0012 g/cc) with two bone cylinders (radius 1 cm, 1.85 g/cc) at seeded offsets, a monoenergetic 60 keV point
  source at 100 cm, a flat 64 x 64 panel of 0.4 cm pixels at 150 cm, P3 and a 4 x 12 = 48 direction sweep set.
  Water 0.206 and bone 0.315 cm^2/g total; scattering albedo 0.923 (water) and 0.611 (bone), split 85 % Compton
  (Klein-Nishina shape) and 15 % Rayleigh (Thomson shape).
* ``mixed_precision_views``: 128 x 128 x 96 cells of 0.25 cm, 16 groups over 20-140 keV, P7, 240 directions, 90
  views, a curved 512 x 384 panel (the configuration the mixed-precision products are measured on).
* ``batched_views``: 64^3 cells of 0.4 cm, an axial water cylinder of radius 11 cm with two bone cylinders of radius
  1.5 cm at seeded offsets, 8 groups from 30 to 120 keV of a seeded bremsstrahlung-like spectrum (Kramers shape with
  2 mm of aluminium), power-law photoelectric plus Klein-Nishina Compton and Rayleigh cross sections, P5, a 6 x 20 =
  120 direction sweep set, 60 views over 360 degrees and a curved 256-channel x 192-row panel.
"""

from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np
import torch

from .cross_sections import BONE, WATER, MultigroupLibrary, klein_nishina, spectral_library, table_moments
from .geometry import ConeGeometry, Grid


def cylinder_phantom(grid: Grid, water_radius: float, bone_radius: float, seed: int = 1) -> np.ndarray:
    """[2, R, C, S] float64 densities (water, bone): an axial water cylinder in air with two bone cylinders whose
    centres are drawn from ``seed`` inside the water."""
    x, y, _ = (a.double().numpy() for a in grid.axis_coordinates(dtype=torch.float64))
    rng = np.random.default_rng(seed)
    r = np.hypot(x[None, :], y[:, None])                                   # [rows, cols]
    bone = np.zeros_like(r, dtype=bool)
    for _ in range(2):
        rad = rng.uniform(0.25, 0.6) * water_radius
        ang = rng.uniform(0, 2 * math.pi)
        bone |= np.hypot(x[None, :] - rad * math.cos(ang), y[:, None] - rad * math.sin(ang)) < bone_radius
    water = np.where(r < water_radius, 1.0, 0.0012)
    water = np.where(bone, 0.0, water)
    S = grid.num_slices
    return np.stack([np.repeat(water[:, :, None], S, 2), np.repeat(np.where(bone, 1.85, 0.0)[:, :, None], S, 2)])


def monoenergetic_library(energy_kev: float, totals, albedos, compton_fraction: float, L: int,
                          num_eta: int = 401) -> MultigroupLibrary:
    """One group at a line: mu/rho totals and scattering albedos per material, the scattering split between a
    Klein-Nishina and a Thomson-shaped kernel; table and Legendre moments consistent."""
    eta = np.linspace(-1.0, 1.0, num_eta)
    kn, _ = klein_nishina(energy_kev, eta)
    kn = kn / table_moments(kn, eta, 0)[0]
    th = 1.0 + eta * eta
    th = th / table_moments(th, eta, 0)[0]
    shape = compton_fraction * kn + (1.0 - compton_fraction) * th               # unit l = 0 moment
    totals, albedos = np.asarray(totals, float), np.asarray(albedos, float)
    M = totals.size
    mu_s = totals * albedos
    mu_s_eta = (mu_s[:, None] * shape[None, :]).reshape(M, 1, 1, num_eta)
    mu_s_l = table_moments(mu_s_eta, eta, L)
    mu_t = totals.reshape(M, 1)
    return MultigroupLibrary(np.array([energy_kev + 0.5, energy_kev - 0.5]), np.array([energy_kev]), np.ones(1),
                             mu_t, mu_t - mu_s_l[..., 0].sum(2), mu_s_l, eta, mu_s_eta, np.array([energy_kev]),
                             mu_t.copy(), np.ones(1), np.zeros(1, dtype=np.int64))


def bremsstrahlung_spectrum(kvp: float = 120.0, filter_mm_al: float = 2.0, seed: int = 0) -> tuple:
    """(energies, photons per keV) every 0.5 keV: Kramers ``(kVp - E) / E`` through an aluminium filter, with a seeded
    +-3 % ripple."""
    e = np.arange(10.0, kvp + 0.25, 0.5)
    mu_al = 0.98 * (e / 30.0) ** -3 + 0.15                                     # cm^2/g, power law
    shape = np.clip(kvp - e, 0.0, None) / e * np.exp(-mu_al * 2.70 * filter_mm_al / 10.0)
    rng = np.random.default_rng(seed)
    return e, shape * (1.0 + 0.03 * rng.standard_normal(e.size))


@dataclass(frozen=True)
class Workload:
    """Everything that defines one synthetic configuration."""

    name: str
    grid: Grid
    geometry: ConeGeometry
    rho: np.ndarray            # [M, R, C, S] float64 densities on the fine grid
    library: MultigroupLibrary
    num_polar: int
    num_azimuthal: int
    legendre_order: int
    transport_cell_cm: float
    num_views: int
    cone_num_polar: int = 16
    cone_num_azimuthal: int = 32

    def angles(self) -> np.ndarray:
        return np.arange(self.num_views) * (2 * math.pi / self.num_views)


def single_view(seed: int = 1) -> Workload:
    grid = Grid((32, 32, 32), 0.5)
    lib = monoenergetic_library(60.0, [0.206, 0.315], [0.923, 0.611], 0.85, 3)
    lib.materials, lib.nominal_density = ("water", "bone_cortical_icrp"), np.array([1.0, 1.85])
    return Workload("single_view", grid, ConeGeometry(100.0, 150.0, 64, 64, 0.4, 0.4),
                    cylinder_phantom(grid, 7.0, 1.0, seed), lib, 4, 12, 3, 0.5, 1)


def batched_views(seed: int = 1, cells: int = 64) -> Workload:
    """The circular cone-beam workload: a 25.6 cm cube of ``cells``^3 cells (64: 0.4 cm), 8 groups from 120 to 30 keV,
    P5, 6 x 20 sweep directions, cone 16 x 32, curved 256 x 192 panel of 0.16 cm pixels, 60 views. Smaller ``cells``
    give the same scene on a coarser grid (the small case of the profiles)."""
    grid = Grid((cells, cells, cells), 25.6 / cells)
    edges = np.linspace(120.0, 30.0, 9)
    lib = spectral_library(edges, bremsstrahlung_spectrum(seed=0), [WATER, BONE], legendre_order=5)
    geo = ConeGeometry(100.0, 150.0, 192, 256, 0.16, 0.16, use_curved_detector=True)
    return Workload("batched_views", grid, geo, cylinder_phantom(grid, 11.0, 1.5, seed), lib, 6, 20, 5, 25.6 / cells,
                    60)


def mixed_precision_views(seed: int = 1, cells: tuple = (128, 128, 96)) -> Workload:
    """The mixed-precision workload: 128 x 128 x 96 cells of 0.25 cm (32 x 32 x 24 cm), the water cylinder of radius
    11 cm with two bone cylinders, 16 groups from 140 to 20 keV of a 140 kVp spectrum, P7 (64 moments), a 10 x 24 =
    240 direction sweep set (8 x 30 would leave the octants unbalanced), cone 16 x 32, 90 views over 360 degrees and a
    curved 512-channel x 384-row panel of 0.08 cm pixels. Smaller ``cells`` give the same scene on coarser cells."""
    rows, cols, slices = (int(c) for c in cells)
    cell = 32.0 / rows
    grid = Grid((rows, cols, slices), cell)
    edges = np.linspace(140.0, 20.0, 17)
    lib = spectral_library(edges, bremsstrahlung_spectrum(kvp=140.0, seed=0), [WATER, BONE], legendre_order=7)
    geo = ConeGeometry(100.0, 150.0, 384, 512, 0.08, 0.08, use_curved_detector=True)
    return Workload("mixed_precision_views", grid, geo, cylinder_phantom(grid, 11.0, 1.5, seed), lib, 10, 24, 7,
                    cell, 90)


INSERT_DENSITIES = (0.0012, 1.04, 1.85)   # air, soft tissue (water material), bone


def ellipsoid_phantom(grid: Grid, seed: int) -> np.ndarray:
    """[2, R, C, S] float64 densities (water, bone) of one random phantom: a water ellipsoid (1.0 g/cc) in air with
    semi-axes drawn uniformly from 8-18 cm (truncated by the volume) and 0-4 ellipsoid inserts of air, soft tissue
    or bone, each with semi-axes of 1-4 cm and a centre inside the water ellipsoid."""
    rng = np.random.default_rng(seed)
    x, y, z = (a.double().numpy() for a in grid.axis_coordinates(dtype=torch.float64))
    Y, X, Z = np.meshgrid(y, x, z, indexing="ij")
    axes = rng.uniform(8.0, 18.0, 3)
    inside = (X / axes[0]) ** 2 + (Y / axes[1]) ** 2 + (Z / axes[2]) ** 2 < 1.0
    water = np.where(inside, 1.0, 0.0012)
    bone = np.zeros_like(water)
    for _ in range(int(rng.integers(0, 5))):
        u = rng.standard_normal(3)
        centre = u / np.linalg.norm(u) * rng.uniform(0.0, 0.7) * axes
        semi = rng.uniform(1.0, 4.0, 3)
        rho = INSERT_DENSITIES[int(rng.integers(0, 3))]
        region = (((X - centre[0]) / semi[0]) ** 2 + ((Y - centre[1]) / semi[1]) ** 2
                  + ((Z - centre[2]) / semi[2]) ** 2 < 1.0) & inside
        if rho > 1.5:
            water[region], bone[region] = 0.0, rho
        else:
            water[region], bone[region] = rho, 0.0
    return np.stack([water, bone])


def learned_proposal(seed: int = 1, cells: tuple = (96, 96, 64)) -> Workload:
    """The learned-proposal workload: a 38.4 x 38.4 x 25.6 cm volume of ``cells`` cubic cells (96 x 96 x 64: 0.4 cm),
    a random ellipsoid phantom of ``seed``, 12 groups from 120 to 30 keV, P5, 6 x 28 = 168 sweep directions, cone
    16 x 32, the curved 256 x 192 panel and 120 views. Smaller ``cells`` give the same scene on coarser cells."""
    rows, cols, slices = (int(c) for c in cells)
    cell = 38.4 / rows
    grid = Grid((rows, cols, slices), cell)
    edges = np.linspace(120.0, 30.0, 13)
    lib = spectral_library(edges, bremsstrahlung_spectrum(seed=0), [WATER, BONE], legendre_order=5)
    geo = ConeGeometry(100.0, 150.0, 192, 256, 0.16, 0.16, use_curved_detector=True)
    return Workload("learned_proposal", grid, geo, ellipsoid_phantom(grid, seed), lib, 6, 28, 5, cell, 120)


# ---- sweep-only problem of the benchmark ----------------------------------------------------------------------------

def config2_sweep_problem_host() -> dict:
    """Host tables of one view's accumulator sweep of ``batched_views`` (for the CPU baseline)."""
    from .quadrature import product_quadrature
    w = batched_views()
    q = product_quadrature(w.num_polar, w.num_azimuthal)
    omega = q.reordered(q.by_octant()).omega
    mu_t = np.einsum("mg,mijk->gijk", w.library.mu_t, w.rho)
    c = (np.abs(omega) / np.asarray(w.grid.deltas)).reshape(8, -1, 3)
    return {"shape": w.grid.shape, "G": w.library.num_groups, "mu_t": mu_t, "c": c}


def config2_sweep_problem(device) -> dict:
    """Device tensors of one view's accumulator sweep of ``batched_views``: the sweep context, mu_t, the transfer
    moments and a seeded collided-fluence accumulator."""
    from .cross_sections import mu_t_volume, transfer_moments_volume
    from .quadrature import product_quadrature
    from .transport_sweep import make_sweep_context
    w = batched_views()
    lib = w.library.truncated(w.legendre_order)
    rho = torch.as_tensor(w.rho, dtype=torch.float32, device=device)
    ctx = make_sweep_context(w.grid, product_quadrature(w.num_polar, w.num_azimuthal), w.legendre_order, device)
    G = lib.num_groups
    N_sh = ctx.num_moments
    gen = torch.Generator(device="cpu").manual_seed(0)
    storage = torch.rand(N_sh, *w.grid.shape, G, 4, generator=gen).to(device) * 0.01
    storage[0, ..., 0] += 1.0
    phi = storage.permute(4, 0, 5, 1, 2, 3)
    return {"ctx": ctx, "mu_t": mu_t_volume(lib, rho), "transfer": transfer_moments_volume(lib, rho), "phi": phi}
