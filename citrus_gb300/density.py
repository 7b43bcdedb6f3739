"""The density model of the CITRUS loop: reconstructed attenuation to reference-material densities (mirrors
``citrus/citrus.py:466-563``, ``DensityModel``, and ``citrus/utilities.py:577-799``).

The materials of the library, ordered by their nominal attenuation at the model energy (the spectrum-mean energy by
default), bracket each voxel's attenuation X; the two bracketing materials share the voxel in proportion to where X
falls between their nominal attenuations, and below the first (from the last) nominal attenuation that material
alone carries it. Each material's map is one kernel of ``libcitrus_gb300.so`` (``citrus_attenuation_to_density``);
the float64 tables (effective energy, log-log interpolated mass attenuation, order) are built here on the host.
"""

from __future__ import annotations

from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch
from torch import Tensor

from . import _lib
from .cross_sections import MultigroupLibrary

MINIMUM_ATTENUATION_GAP = 1e-3  # smallest relative gap between neighbouring nominal attenuations


def effective_energy(library: MultigroupLibrary) -> float:
    """Spectrum-mean fine energy ``sum w E / sum w`` in keV (reference ``utilities.py:577-587``)."""
    w = np.asarray(library.fine_weight, dtype=np.float64)
    return float((w * np.asarray(library.fine_energy, dtype=np.float64)).sum() / w.sum())


def mass_attenuation_at(library: MultigroupLibrary, energy_kev: float) -> np.ndarray:
    """[M] total mass attenuation at one energy, linear in (log E, log mu) between the sorted fine energies; a fine
    energy gives its tabulated values (reference ``utilities.py:590-619``)."""
    E = np.asarray(library.fine_energy, dtype=np.float64)
    mu = np.asarray(library.fine_mu_t, dtype=np.float64)
    order = np.argsort(E, kind="stable")
    E, mu = E[order], mu[:, order]
    e = float(energy_kev)
    if not E[0] <= e <= E[-1]:
        raise ValueError(f"energy {e} keV outside the library's fine-energy range [{E[0]}, {E[-1]}]")
    i = int(np.searchsorted(E, e, side="right")) - 1
    if E[max(i, 0)] == e:
        return mu[:, max(i, 0)].copy()
    i = min(max(i, 0), E.size - 2)
    t = (np.log(e) - np.log(E[i])) / (np.log(E[i + 1]) - np.log(E[i]))
    return np.exp(np.log(mu[:, i]) + t * (np.log(mu[:, i + 1]) - np.log(mu[:, i])))


def nominal_attenuation(library: MultigroupLibrary, energy_kev: Optional[float] = None) -> np.ndarray:
    e = effective_energy(library) if energy_kev is None else float(energy_kev)
    return np.asarray(library.nominal_density, dtype=np.float64) * mass_attenuation_at(library, e)


def material_order(library: MultigroupLibrary, energy_kev: Optional[float] = None) -> list:
    """Material indices by increasing nominal attenuation; neighbours closer than 0.1 % cannot be bracketed
    (reference ``utilities.py:647-670``, ``cross_section_library.py:227-256``)."""
    attenuation = nominal_attenuation(library, energy_kev)
    order = np.argsort(attenuation, kind="stable")
    s = attenuation[order]
    if s.size > 1:
        gaps = np.diff(s) / np.maximum(s[1:], np.finfo(np.float64).tiny)
        bad = np.nonzero(~(gaps >= MINIMUM_ATTENUATION_GAP))[0]
        if bad.size:
            i = int(bad[0])
            names = list(library.materials) if library.materials is not None else [str(k) for k in range(s.size)]
            raise ValueError(f"materials {names[order[i]]!r} and {names[order[i + 1]]!r} have nearly the same nominal "
                             f"attenuation ({s[i]:.6g} and {s[i + 1]:.6g} 1/cm): the density model cannot tell them "
                             f"apart")
    return [int(k) for k in order]


@dataclass
class DensityModel:
    """Attenuation X in 1/cm to the densities of the library's materials at ``energy_kev`` (reference
    ``citrus.py:466-563``)."""

    library: MultigroupLibrary
    energy_kev: float
    last_negative_fraction: float = 0.0

    @classmethod
    def from_library(cls, library: MultigroupLibrary, energy_kev: Optional[float] = None) -> "DensityModel":
        return cls(library, effective_energy(library) if energy_kev is None else float(energy_kev))

    def _tables(self, device) -> tuple:
        key = (str(device), self.energy_kev)
        cache = self.__dict__.setdefault("_cache", {})
        if key not in cache:
            order = material_order(self.library, self.energy_kev)
            mass = mass_attenuation_at(self.library, self.energy_kev)[order].astype(np.float32)
            nominal = np.asarray(self.library.nominal_density, dtype=np.float64)[order].astype(np.float32)
            mu = nominal * mass                                   # float32 products, as on the device
            cache[key] = (order, *(torch.as_tensor(np.ascontiguousarray(a)).to(device) for a in (mu, mass, nominal)))
        return cache[key]

    def material(self, X: Tensor, m: int) -> Tensor:
        """Density map in g/cm^3 of library material ``m`` (reference ``citrus.py:536-555``)."""
        M = self.library.num_materials
        if not 0 <= int(m) < M:
            raise ValueError(f"material {m} outside the library's {M} materials")
        if X.device.type != "cuda" or X.dtype != torch.float32:
            raise ValueError("X must be a float32 CUDA tensor")
        order, mu, mass, nominal = self._tables(X.device)
        x = X.contiguous()
        out = torch.empty_like(x)
        _lib.call("citrus_attenuation_to_density", x.data_ptr(), x.numel(), mu.data_ptr(), mass.data_ptr(),
                  nominal.data_ptr(), M, order.index(int(m)), out.data_ptr(), _lib.stream_handle(X.device))
        return out

    def __call__(self, X: Tensor) -> Tensor:
        """[M, ...] densities of all materials; also sets ``last_negative_fraction``."""
        self.last_negative_fraction = float((X < 0).float().mean())
        return torch.stack([self.material(X, m) for m in range(self.library.num_materials)])

    def negative_fraction(self, X: Tensor) -> float:
        self.last_negative_fraction = int(torch.count_nonzero(X < 0)) / max(1, X.numel())
        return self.last_negative_fraction


def densities_to_attenuation(library: MultigroupLibrary, rho: Tensor, energy_kev: Optional[float] = None) -> Tensor:
    """X = sum_m rho_m m_m(E) (reference ``utilities.py:688-707``)."""
    e = effective_energy(library) if energy_kev is None else float(energy_kev)
    m = torch.as_tensor(mass_attenuation_at(library, e), dtype=rho.dtype).to(rho.device)
    X = rho[0] * m[0]
    for k in range(1, rho.shape[0]):
        X = X + rho[k] * m[k]
    return X
