"""The scatter step on sm_103a against the reference's own end-to-end results.

* The reference's regression anchor of ``solve_view`` (its ``tests/data/pre_quadrature_reference.json``, cases
  ``synthetic_cuda`` at 1e-5 and ``synthetic_cpu``, checked as its ``tests/test_quadrature_grid.py:333-342`` does):
  seven-material synthetic library, WLAB phantom on the 2 cm grid, 4 cm cells, the fine uncollided trace, CsI panel.
* The single-view workload (32^3 cells of 0.5 cm, one 60 keV group, P3, 48 sweep directions, cone 16 x 32, flat
  64 x 64 panel): two ``citrus_view_step`` calls against the reference's float64 run, element by element.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import check_regression_case, elementwise_rel_err, golden, rel_err
from citrus_gb300.cross_sections import MultigroupLibrary
from citrus_gb300.geometry import ConeGeometry, Grid
from citrus_gb300.responses import DetectorResponse, ideal_counting_response, no_grid
from citrus_gb300.scatter_solver import ScatterSolver, SolverConfig

pytestmark = pytest.mark.gpu


def _pre_quadrature_solver(device):
    g = golden("pre_quadrature_synthetic")
    fields = {k[4:]: g[k] for k in g if k.startswith("lib_") and k != "lib_materials"}
    library = MultigroupLibrary(materials=tuple(str(m) for m in g["lib_materials"]), **fields)
    src_iso, src_det, rows, cols, d_row, d_col = g["geometry"]
    geo = ConeGeometry(float(src_iso), float(src_det), int(rows), int(cols), float(d_row), float(d_col))
    config = SolverConfig(num_groups=4, legendre_order=3, num_polar=4, num_azimuthal=8, cone_num_polar=8,
                          cone_num_azimuthal=16, transport_cell_cm=4.0, quadrature_point_spacing_cm=2.0,
                          source_iteration_tolerance=1e-4, max_source_iterations=40, direction_chunk=8,
                          uncollided_trace_grid="fine")
    det = DetectorResponse(g["det_e"], g["det_theta"], g["det_table"])
    return g, ScatterSolver(library, config, geo, detector=det, grid_response=no_grid(), device=device)


def test_solve_view_reproduces_the_reference_regression_cases(cuda_device):
    """float32 on the GPU against the reference's committed cases: ``synthetic_cuda`` at its own 1e-5 and the float64
    ``synthetic_cpu`` at 1e-5; the full images against the reference's float64 solve element by element (pixels
    above 1e-3 of the maximum) at 1e-4 (scatter) and 1e-5 (primary)."""
    g, solver = _pre_quadrature_solver(cuda_device)
    rho = torch.as_tensor(g["rho"], dtype=torch.float32, device=cuda_device)
    r = solver.solve_view(rho, Grid((10, 16, 20), 2.0), 0.4)
    si = r.source_iteration_result
    for name in ("synthetic_cuda", "synthetic_cpu"):
        check_regression_case(r.scatter_signal, r.primary["signal"], si.num_iterations, float(si.history[-1]), g,
                              name, 1e-5)
    assert elementwise_rel_err(r.scatter_signal, g["scatter_signal"]) < 1e-4
    assert elementwise_rel_err(r.primary["signal"], g["primary_signal"]) < 1e-5
    np.testing.assert_allclose(si.history, g["si_history"], rtol=1e-3, atol=1e-7)


def _config1_solver(device, **overrides):
    from citrus_gb300.workloads import single_view
    w = single_view()
    config = SolverConfig(num_groups=1, legendre_order=w.legendre_order, num_polar=w.num_polar,
                          num_azimuthal=w.num_azimuthal, transport_cell_cm=w.transport_cell_cm,
                          quadrature_point_spacing_cm=0.5, cone_num_polar=w.cone_num_polar,
                          cone_num_azimuthal=w.cone_num_azimuthal, direction_chunk=6, **overrides)
    solver = ScatterSolver(w.library, config, w.geometry, detector=ideal_counting_response(), grid_response=no_grid(),
                           device=device)
    return w, solver


def _block_means(a: np.ndarray, b: int) -> np.ndarray:
    *lead, R, C, S = a.shape
    return a.reshape(*lead, R // b, b, C // b, b, S // b, b).mean(axis=(-5, -3, -1))


@pytest.mark.parametrize("precision", ["fp32", "bf16x3"])
def test_single_view_workload_steps_match_reference_elementwise(cuda_device, precision):
    """Two scatter steps of the single-view workload (citrus_view_step with the primary, cold start) against the
    reference's float64 CPU run: scatter images and the collided scalar flux's LD moments element by element (values
    above 1e-3 of the maximum) within 1e-4, the cell means of all 16 moments over 2^3-cell blocks within 1e-4 of their
    maximum, primary within 1e-5 element by element, SPR within 1e-4 (0.5 % is the bound of the mixed forms)."""
    from citrus_gb300.citrus_step import CitrusState, citrus_view_step
    g = golden("config1_view")
    w, solver = _config1_solver(cuda_device, moment_precision=precision)
    rho = torch.as_tensor(w.rho, dtype=torch.float32, device=cuda_device)
    fields = solver.material_fields(rho, w.grid)
    state = CitrusState()
    tol = 1e-4 if precision == "fp32" else 2e-4
    for step in (1, 2):
        scatter, primary, state = citrus_view_step(solver, state, fields, 0.0, primary=True)
        phi = state.collided_moments.detach().cpu().double().numpy()
        assert elementwise_rel_err(scatter, g[f"step{step}_scatter"]) < tol
        assert elementwise_rel_err(phi[:, 0], g[f"step{step}_scalar"]) < tol
        means = _block_means(phi[:, :, 0], 2)
        ref = g[f"step{step}_means_b2"]
        for n in range(ref.shape[1]):
            assert rel_err(means[:, n], ref[:, n]) < tol, n
        assert abs(state.history[-1] - float(g[f"step{step}_change"])) < 1e-4
    assert elementwise_rel_err(primary, g["primary"]) < 1e-5
    p = g["primary"]
    mask = p > 1e-3 * p.max()
    spr = scatter.detach().cpu().double().numpy()[mask] / primary.detach().cpu().double().numpy()[mask]
    assert np.abs(spr / (g["step2_scatter"][mask] / p[mask]) - 1).max() < (1e-4 if precision == "fp32" else 5e-3)
