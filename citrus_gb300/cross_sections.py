"""Multigroup cross-section library of the scatter step and its per-voxel fields.

``MultigroupLibrary`` has the fields and units of the reference's library (``citrus/scatter_solver/cross_sections.py:
493-650``): per-unit-density total and photoelectric attenuation per group, Legendre transfer moments
``mu_s_l [M, G, G, L+1]``, the per-steradian transfer tabulated in the scattering cosine ``mu_s_eta [M, G, G, N]``,
and the fine-energy attenuation and weights of the exact-in-energy transmission. ``synthetic_library`` reproduces the
reference's test library (``:1043-1131``) exactly; ``spectral_library`` synthesizes a library from a spectrum, a
power-law photoelectric term, Klein-Nishina Compton scattering with its kinematic energy loss and Rayleigh scattering,
with table and moments consistent to float64 rounding.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field, replace
from typing import Optional, Sequence

import numpy as np
import torch
from torch import Tensor


@dataclass
class MultigroupLibrary:
    """Per-unit-density multigroup coefficients (float64 numpy on the host; ``tensors`` gives device copies)."""

    group_edges: np.ndarray      # [G+1] keV, descending
    group_energy: np.ndarray     # [G] keV
    spectrum_fraction: np.ndarray  # [G]
    mu_t: np.ndarray             # [M, G] cm^2/g
    mu_pe: np.ndarray            # [M, G]
    mu_s_l: np.ndarray           # [M, G, G, L+1]
    eta_grid: np.ndarray         # [N] ascending -1 .. 1 (uniform)
    mu_s_eta: np.ndarray         # [M, G, G, N] cm^2/g/sr
    fine_energy: np.ndarray      # [E]
    fine_mu_t: np.ndarray        # [M, E]
    fine_weight: np.ndarray      # [E]
    fine_group: np.ndarray       # [E] int64
    materials: tuple = ()
    nominal_density: Optional[np.ndarray] = None
    _device_cache: dict = field(default_factory=dict, repr=False, compare=False)

    def __post_init__(self):
        M = self.mu_t.shape[0]
        if not self.materials:
            self.materials = ("water", "bone_cortical_icrp") if M == 2 else tuple(f"m{m}" for m in range(M))
        if self.nominal_density is None:
            self.nominal_density = np.array([1.0, 1.85]) if M == 2 else np.arange(1.0, M + 1.0)

    @property
    def num_materials(self) -> int:
        return int(self.mu_t.shape[0])

    @property
    def num_groups(self) -> int:
        return int(self.mu_t.shape[1])

    @property
    def legendre_order(self) -> int:
        return int(self.mu_s_l.shape[-1]) - 1

    def truncated(self, L: int) -> "MultigroupLibrary":
        """The library with ``mu_s_l`` truncated to order L (reference ``scatter_solver.py:83-101``)."""
        if self.legendre_order < L:
            raise ValueError(f"library Legendre order {self.legendre_order} < {L}")
        return self if self.legendre_order == L else replace(self, mu_s_l=self.mu_s_l[..., :L + 1].copy(),
                                                              _device_cache={})

    def tensor(self, name: str, device, dtype=torch.float32) -> Tensor:
        """A device copy of one field, cached per device and dtype."""
        key = (name, str(device), dtype)
        t = self._device_cache.get(key)
        if t is None:
            t = torch.as_tensor(np.ascontiguousarray(getattr(self, name)), dtype=dtype).to(device)
            self._device_cache[key] = t
        return t

    _FIELDS = ("group_edges", "group_energy", "spectrum_fraction", "mu_t", "mu_pe", "mu_s_l", "eta_grid", "mu_s_eta",
               "fine_energy", "fine_mu_t", "fine_weight", "fine_group")

    def save(self, path: str) -> None:
        """Write the library in the reference's on-disk format (``cross_sections.py:624-630``): ``torch.save`` of a
        dict of every field of its dataclass, float64 tensors (``fine_group`` int64), ``materials`` a tuple of names
        and ``eta_map`` None (a uniform table), so the reference's ``MultigroupLibrary.load`` reads the file."""
        fields = {k: torch.as_tensor(np.asarray(getattr(self, k)),
                                     dtype=torch.int64 if k == "fine_group" else torch.float64) for k in self._FIELDS}
        fields["materials"] = tuple(str(m) for m in self.materials)
        fields["nominal_density"] = torch.as_tensor(np.asarray(self.nominal_density), dtype=torch.float64)
        fields["eta_map"] = None
        torch.save(fields, path)

    @staticmethod
    def load(path: str) -> "MultigroupLibrary":
        """Read a library written by ``save`` or by the reference's ``MultigroupLibrary.save`` (``:632-650``); a
        file without ``eta_map`` is a uniform table. Raises KeyError for a missing field (as the reference does) and
        ValueError for an adaptive table (``eta_map`` set), whose node placement this package does not evaluate."""
        fields = torch.load(path, map_location="cpu", weights_only=True)
        missing = [k for k in (*MultigroupLibrary._FIELDS, "materials", "nominal_density") if k not in fields]
        if missing:
            raise KeyError(f"library file {path!r} lacks fields {missing}")
        if fields.get("eta_map") is not None:
            raise ValueError(f"library file {path!r} holds an adaptive eta table (eta_map); only uniform tables "
                             "are evaluated here")
        arrays = {k: fields[k].detach().cpu().numpy() for k in MultigroupLibrary._FIELDS}
        return MultigroupLibrary(materials=tuple(fields["materials"]),
                                 nominal_density=fields["nominal_density"].detach().cpu().numpy(), **arrays)


# the reference's seven default materials and their nominal densities (``cross_sections.py:211-214``), and the
# (scale, bone fraction) of each row of its seven-material synthetic library (``cross_sections.py:1112-1117``)
REFERENCE_MATERIALS = ("air", "lung_icrp", "adipose_icrp", "water", "muscle_icru44", "soft_tissue_icru44",
                       "bone_cortical_icrp")
REFERENCE_NOMINAL_DENSITIES = (0.0012, 0.26, 0.95, 1.0, 1.05, 1.06, 1.85)
_SYNTHETIC_BLENDS = {"air": (0.90, 0.0), "lung_icrp": (0.95, 0.02), "adipose_icrp": (0.97, 0.0), "water": (1.0, 0.0),
                     "muscle_icru44": (1.0, 0.02), "soft_tissue_icru44": (1.0, 0.04), "bone_cortical_icrp": (1.0, 1.0)}


def synthetic_library(num_groups: int = 4, legendre_order: int = 5, num_eta: int = 401,
                      num_fine_per_group: int = 4, fine_spread: float = 0.0,
                      num_materials: int = 2) -> MultigroupLibrary:
    """The reference's test library: kernel ``a (1 + b eta) / 4 pi``, linear in eta, so table and moments agree
    exactly (reference ``cross_sections.py:1043-1131``). Two materials are (water, bone); seven are the reference's
    default materials, each row a scaled blend of the two; any other M > 2 blends named "m0", "m1", ..."""
    G, L = num_groups, legendre_order
    edges = np.linspace(125.0, 10.0, G + 1)
    energy = 0.5 * (edges[:-1] + edges[1:])
    fraction = np.ones(G) / G
    eta = np.linspace(-1.0, 1.0, num_eta)
    mu_s_eta = np.zeros((2, G, G, num_eta))
    mu_s_l = np.zeros((2, G, G, L + 1))
    for m in range(2):
        for gi in range(G):
            for go in range(gi, G):
                a = (0.15 if m == 0 else 0.12) * (0.6 ** (go - gi))
                b = 0.5 if go == gi else 0.2
                mu_s_eta[m, gi, go] = a * (1.0 + b * eta) / (4.0 * math.pi)
                mu_s_l[m, gi, go, 0] = a
                if L >= 1:
                    mu_s_l[m, gi, go, 1] = a * b / 3.0
    mu_pe = np.array([[0.05 * (1.5 ** g) for g in range(G)], [0.2 * (1.5 ** g) for g in range(G)]])
    mu_t = mu_pe + mu_s_l[..., 0].sum(axis=2)
    n = int(num_fine_per_group)
    t = (np.arange(n) + 0.5) / n
    x = 1.0 - 2.0 * np.arange(n) / (n - 1) if n > 1 else np.zeros(1)
    fine_energy = np.concatenate([edges[g + 1] + t * (edges[g] - edges[g + 1]) for g in range(G)])
    fine_group = np.repeat(np.arange(G), n)
    fine_weight = fraction[fine_group] / n
    fine_mu_t = mu_t[:, fine_group] * (1.0 + float(fine_spread) * np.tile(x, G))[None, :]
    M = int(num_materials)
    if M == 2:
        return MultigroupLibrary(edges, energy, fraction, mu_t, mu_pe, mu_s_l, eta, mu_s_eta, fine_energy, fine_mu_t,
                                 fine_weight, fine_group)
    if M < 2:
        raise ValueError("num_materials must be >= 2")
    if M == len(REFERENCE_MATERIALS):
        rows = [_SYNTHETIC_BLENDS[n] for n in REFERENCE_MATERIALS]
        names, nominal = REFERENCE_MATERIALS, np.array(REFERENCE_NOMINAL_DENSITIES)
    else:
        rows = [(1.0, 0.0), (1.0, 1.0)] + [(1.0 + 0.1 * m, (m - 1) / (M - 1)) for m in range(2, M)]
        names, nominal = tuple(f"m{m}" for m in range(M)), np.arange(1.0, M + 1.0)

    def blend(a):
        # a pure row (scale 1, fraction 0 or 1) is that material's row itself, bit for bit
        return np.stack([a[int(t)].copy() if s == 1.0 and t in (0.0, 1.0) else s * ((1.0 - t) * a[0] + t * a[1])
                         for s, t in rows])

    return MultigroupLibrary(edges, energy, fraction, blend(mu_t), blend(mu_pe), blend(mu_s_l), eta, blend(mu_s_eta),
                             fine_energy, blend(fine_mu_t), fine_weight, fine_group, materials=names,
                             nominal_density=nominal)


# ---- spectral library ---------------------------------------------------------------------------------------------

ELECTRON_REST_KEV = 510.99895
CLASSICAL_RADIUS_CM = 2.8179403262e-13
AVOGADRO = 6.02214076e23


def klein_nishina(energy_kev, eta):
    """Klein-Nishina cross section per electron per steradian in cm^2/sr, and the scattered energy."""
    k = np.asarray(energy_kev, dtype=np.float64) / ELECTRON_REST_KEV
    eta = np.asarray(eta, dtype=np.float64)
    P = 1.0 / (1.0 + k * (1.0 - eta))
    return 0.5 * CLASSICAL_RADIUS_CM ** 2 * P * P * (P + 1.0 / P - (1.0 - eta * eta)), np.asarray(energy_kev) * P


def _legendre(L: int, x: np.ndarray) -> np.ndarray:
    out = [np.ones_like(x), x.copy()]
    for l in range(1, L):
        out.append(((2 * l + 1) * x * out[l] - l * out[l - 1]) / (l + 1))
    return np.stack(out[:L + 1], axis=-1)


def table_moments(table: np.ndarray, eta: np.ndarray, L: int) -> np.ndarray:
    """Legendre moments ``2 pi int P_l(eta) f(eta) d eta`` of the piecewise-linear interpolant of a table [.., N]
    (8-point Gauss-Legendre per interval: exact for the polynomial pieces up to degree L + 1 <= 15)."""
    xg, wg = np.polynomial.legendre.leggauss(8)
    a, b = eta[:-1], eta[1:]
    h = 0.5 * (b - a)
    x = 0.5 * (a + b)[:, None] + h[:, None] * xg[None, :]            # [N-1, 8]
    w = h[:, None] * wg[None, :]
    s = (x - a[:, None]) / (2 * h[:, None])                          # interpolation weight of node i+1
    P = _legendre(L, x)                                              # [N-1, 8, L+1]
    lo = np.einsum("pq,pql->pl", w * (1 - s), P)                     # [N-1, L+1]
    hi = np.einsum("pq,pql->pl", w * s, P)
    return 2.0 * math.pi * (np.einsum("...p,pl->...l", table[..., :-1], lo)
                            + np.einsum("...p,pl->...l", table[..., 1:], hi))


@dataclass(frozen=True)
class MaterialModel:
    """Synthetic material: electrons per gram, photoelectric mass attenuation at 60 keV (E^-3 power law), Rayleigh
    mass attenuation at 60 keV (E^-2), and a scale of the Compton term."""

    name: str
    electrons_per_gram: float
    photoelectric_60kev: float
    rayleigh_60kev: float
    nominal_density: float


WATER = MaterialModel("water", AVOGADRO * 10.0 / 18.015, 0.0159, 0.0107, 1.0)
BONE = MaterialModel("bone_cortical_icrp", AVOGADRO * 0.5148, 0.1225, 0.0257, 1.85)


def spectral_library(edges_kev: Sequence[float], spectrum: tuple, materials: Sequence[MaterialModel],
                     legendre_order: int, num_eta: int = 401, fine_per_group: int = 16,
                     compton_scale: Optional[Sequence[float]] = None) -> MultigroupLibrary:
    """A library from a spectrum (energies [K] keV, photons per keV [K]) and synthetic materials.

    Compton scattering follows Klein-Nishina with the kinematic energy loss ``E' = E / (1 + k (1 - eta))`` (a fine
    energy of group g scattered at cosine eta lands in the group of E'; below the last edge it is absorbed);
    Rayleigh scattering keeps the energy with the Thomson shape ``3/(16 pi) (1 + eta^2)``. The per-steradian table is
    averaged over the fine energies of the incoming group with the spectrum weights; the Legendre moments are those of
    its piecewise-linear interpolant, so table and moments are consistent.
    """
    edges = np.asarray(edges_kev, dtype=np.float64)
    G = edges.size - 1
    L = int(legendre_order)
    e_spec, p_spec = (np.asarray(a, dtype=np.float64) for a in spectrum)
    fine_e, fine_w, fine_g = [], [], []
    if e_spec.size == 1:  # a monoenergetic line: one fine energy in the group that holds it
        g_line = int(np.searchsorted(-edges, -e_spec[0], side="right") - 1)
        if not 0 <= g_line < G:
            raise ValueError(f"the line at {e_spec[0]} keV lies outside the group edges")
        fine_e, fine_w, fine_g = [e_spec[:1]], [np.ones(1)], [np.full(1, g_line)]
    for g in range(G if e_spec.size > 1 else 0):
        hi, lo = edges[g], edges[g + 1]
        mids = lo + (np.arange(fine_per_group) + 0.5) / fine_per_group * (hi - lo)
        density = np.interp(mids, e_spec, p_spec, left=0.0, right=0.0)
        fine_e.append(mids)
        fine_w.append(density * (hi - lo) / fine_per_group)
        fine_g.append(np.full(fine_per_group, g))
    fine_e, fine_w, fine_g = np.concatenate(fine_e), np.concatenate(fine_w), np.concatenate(fine_g)
    fine_w = fine_w / fine_w.sum()
    fraction = np.bincount(fine_g, weights=fine_w, minlength=G)
    with np.errstate(invalid="ignore", divide="ignore"):
        energy = np.bincount(fine_g, weights=fine_w * fine_e, minlength=G) / fraction
    energy = np.where(fraction > 0, energy, 0.5 * (edges[:-1] + edges[1:]))
    eta = np.linspace(-1.0, 1.0, num_eta)
    M = len(materials)
    scale = np.ones(M) if compton_scale is None else np.asarray(compton_scale, dtype=np.float64)
    thomson = 3.0 / (16.0 * math.pi) * (1.0 + eta * eta)
    eta_fine = np.linspace(-1.0, 1.0, 20001)
    mu_s_eta = np.zeros((M, G, G, num_eta))
    fine_mu_t = np.zeros((M, fine_e.size))
    for m, mat in enumerate(materials):
        for e_idx, (E, w, g) in enumerate(zip(fine_e, fine_w, fine_g)):
            dsig, E_out = klein_nishina(E, eta)
            compton = scale[m] * mat.electrons_per_gram * dsig                      # cm^2/g/sr at the nodes
            go = np.searchsorted(-edges, -E_out, side="right") - 1                  # group of the scattered energy
            rayleigh = mat.rayleigh_60kev * (E / 60.0) ** -2 * thomson
            wg = w / fraction[g] if fraction[g] > 0 else 0.0
            for out_group in range(g, G):
                mu_s_eta[m, g, out_group] += wg * np.where(go == out_group, compton, 0.0)
            mu_s_eta[m, g, g] += wg * rayleigh
            ds_f, _ = klein_nishina(E, eta_fine)
            sigma_c = scale[m] * mat.electrons_per_gram * 2 * math.pi * np.trapezoid(ds_f, eta_fine)
            fine_mu_t[m, e_idx] = (mat.photoelectric_60kev * (E / 60.0) ** -3 + sigma_c
                                   + mat.rayleigh_60kev * (E / 60.0) ** -2)
    mu_s_l = table_moments(mu_s_eta, eta, L)
    mu_t = np.stack([np.bincount(fine_g, weights=fine_w * fine_mu_t[m], minlength=G) / np.where(fraction > 0,
                                                                                               fraction, 1.0)
                     for m in range(M)])
    mu_pe = mu_t - mu_s_l[..., 0].sum(axis=2)
    return MultigroupLibrary(edges, energy, fraction, mu_t, mu_pe, mu_s_l, eta, mu_s_eta, fine_e, fine_mu_t, fine_w,
                             fine_g, materials=tuple(m.name for m in materials),
                             nominal_density=np.array([m.nominal_density for m in materials]))


# ---- per-voxel fields --------------------------------------------------------------------------------------------

def mu_t_volume(library: MultigroupLibrary, rho: Tensor) -> Tensor:
    """[G, R, C, S] total attenuation of densities rho [M, R, C, S] (reference ``cross_sections.py:762-773``)."""
    mu = library.tensor("mu_t", rho.device, rho.dtype)
    return torch.einsum("mg,mijk->gijk", mu, rho).contiguous()


def transfer_moments_volume(library: MultigroupLibrary, rho: Tensor) -> Tensor:
    """[G, G, L+1, R, C, S] Legendre transfer moments (reference ``cross_sections.py:886-897``)."""
    t = library.tensor("mu_s_l", rho.device, rho.dtype)
    return torch.einsum("mabl,mijk->ablijk", t, rho).contiguous()
