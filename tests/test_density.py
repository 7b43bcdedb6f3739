"""The density model of the CITRUS loop (reference ``citrus/citrus.py:466-563``, ``citrus/utilities.py:577-799``)
against the reference's own maps (``tests/golden/density_model.npz``)."""

from __future__ import annotations

from types import SimpleNamespace

import numpy as np
import pytest
import torch

from conftest import golden
from citrus_gb300.density import (DensityModel, effective_energy, mass_attenuation_at, material_order,
                                  nominal_attenuation)


def _library(g):
    return SimpleNamespace(fine_energy=g["lib_fine_energy"], fine_mu_t=g["lib_fine_mu_t"],
                           fine_weight=g["lib_fine_weight"], nominal_density=g["lib_nominal"], num_materials=3,
                           materials=("water", "bone_cortical_icrp", "soft_tissue"))


def test_host_tables_match_reference():
    g = golden("density_model")
    lib = _library(g)
    assert effective_energy(lib) == pytest.approx(float(g["energy"]), rel=1e-15)
    np.testing.assert_allclose(mass_attenuation_at(lib, float(g["energy"])), g["mass"], rtol=1e-14)
    assert material_order(lib) == list(g["order"])
    # a fine energy gives its tabulated coefficients, energies outside the table are refused
    e0 = float(lib.fine_energy[3])
    np.testing.assert_array_equal(mass_attenuation_at(lib, e0), lib.fine_mu_t[:, 3])
    with pytest.raises(ValueError):
        mass_attenuation_at(lib, 1.0)
    # two materials closer than 0.1 % in nominal attenuation cannot be bracketed
    close = SimpleNamespace(**dict(vars(lib), nominal_density=np.array([1.0, 1.0005, 2.0]),
                                   fine_mu_t=np.repeat(lib.fine_mu_t[:1], 3, 0)))
    assert nominal_attenuation(close)[1] > nominal_attenuation(close)[0]
    with pytest.raises(ValueError):
        material_order(close)


@pytest.mark.gpu
def test_density_maps_are_the_reference_maps(cuda_device):
    g = golden("density_model")
    model = DensityModel.from_library(_library(g))
    X = torch.as_tensor(g["X"], device=cuda_device)
    for m in range(3):
        assert torch.equal(model.material(X, m).cpu(), torch.as_tensor(g["rho"][m]))
        assert torch.equal(model.material(X, m).cpu(), torch.as_tensor(g["single"][m]))
    all_maps = model(X)
    assert torch.equal(all_maps.cpu(), torch.as_tensor(g["rho"]))
    assert model.last_negative_fraction == pytest.approx(float((g["X"] < 0).mean()))
    at50 = DensityModel(_library(g), 50.0)
    assert torch.equal(at50(torch.as_tensor(g["X50"], device=cuda_device)).cpu(), torch.as_tensor(g["rho50"]))
    with pytest.raises(ValueError):
        model.material(X, 3)


@pytest.mark.gpu
def test_fields_from_attenuation_equal_fields_of_the_maps(cuda_device):
    from citrus_gb300.geometry import ConeGeometry, Grid
    from citrus_gb300.responses import ideal_counting_response, no_grid
    from citrus_gb300.scatter_solver import ScatterSolver, SolverConfig
    from citrus_gb300.workloads import batched_views
    w = batched_views(cells=16)
    lib = w.library
    solver = ScatterSolver(lib, SolverConfig(num_groups=8, legendre_order=5, num_polar=6, num_azimuthal=20,
                                             transport_cell_cm=3.2), w.geometry, detector=ideal_counting_response(),
                           grid_response=no_grid(), device=cuda_device)
    model = DensityModel.from_library(lib)
    rng = np.random.default_rng(3)
    X = torch.as_tensor(rng.random(w.grid.shape) * 0.5 - 0.02, dtype=torch.float32, device=cuda_device)
    a = solver.material_fields_from_attenuation(X, w.grid, model)
    b = solver.material_fields(model(X), w.grid)
    for name in ("rho_fine", "rho_coarse", "rho_quadrature", "mu_t_coarse", "mu_s_l_coarse"):
        assert torch.equal(getattr(a, name), getattr(b, name)), name
