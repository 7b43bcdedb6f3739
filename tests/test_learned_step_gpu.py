"""What the trained proposal gains: the learned higher-order proposal against the method without it.

The solver generates its own training triples on a reduced learned-proposal workload (random ellipsoid phantoms,
24 x 24 x 16 cells of 1.6 cm, 12 groups, P5, 168 directions), the network trains on the GPU with the library's kernels,
and on phantoms it never saw:

* the proposal's Phi_{>1} is within 10 % (relative L2) of the converged solve's, where the cold start (Phi_{>1} = 0)
  is 100 % off;
* the first CITRUS step started from the proposal projects an SPR within 0.5 % of the converged one, where the cold
  start's first step is off by more than 10 %;
* converging the SPR to within 0.5 % takes at most two thirds of the sweeps of the plain source iteration from the
  cold start (about half on most views), and for both starts the true SPR error against the converged solve is
  within 0.5 % on every unseen view.
"""

from __future__ import annotations

import numpy as np
import pytest
import torch

from citrus_gb300 import learned
from citrus_gb300.citrus_step import CitrusState, citrus_view_step, project_scatter
from citrus_gb300.responses import ideal_counting_response, no_grid
from citrus_gb300.scatter_solver import ScatterSolver, SolverConfig
from citrus_gb300.workloads import ellipsoid_phantom, learned_proposal

pytestmark = pytest.mark.gpu
CELLS = (24, 24, 16)


@pytest.fixture(scope="module")
def trained(cuda_device):
    w = learned_proposal(1, CELLS)
    config = SolverConfig(num_groups=w.library.num_groups, legendre_order=w.legendre_order,
                          num_polar=w.num_polar, num_azimuthal=w.num_azimuthal,
                          transport_cell_cm=w.transport_cell_cm, quadrature_point_spacing_cm=w.transport_cell_cm,
                          cone_num_polar=w.cone_num_polar, cone_num_azimuthal=w.cone_num_azimuthal)
    solver = ScatterSolver(w.library, config, w.geometry, detector=ideal_counting_response(), grid_response=no_grid(),
                           device=cuda_device)
    rng = np.random.default_rng(0)
    samples = []
    for seed in range(64):
        samples += learned.generate_training_data(solver, [ellipsoid_phantom(w.grid, 1000 + seed)], w.grid,
                                                  [float(a) for a in rng.uniform(0, 2 * np.pi, 2)])
    proposal = learned.HigherOrderProposal(w.library.num_materials, w.library.num_groups, seed=0,
                                           device=cuda_device)
    losses = proposal.fit(samples, epochs=60, batch=4, lr=1e-3, seed=0)
    return w, solver, proposal, losses


def test_training_lowers_the_loss(trained):
    _, _, _, losses = trained
    assert losses[-1] < 0.2 * losses[0]


@pytest.mark.parametrize("seed", [5000, 5001, 5002, 5003, 5004, 5005])
def test_proposal_gain_on_unseen_phantoms(trained, seed):
    w, solver, proposal, _ = trained
    angle = float(np.random.default_rng(seed).uniform(0, 2 * np.pi))
    rho = torch.as_tensor(ellipsoid_phantom(w.grid, seed), dtype=torch.float32, device=solver.device)
    fields = solver.material_fields(rho, w.grid)
    first, total = learned.collided_orders(solver, fields, angle, tolerance=1e-6)
    higher = learned.scalar_flux(total) - learned.scalar_flux(first)
    predicted = proposal.predict(fields.rho_coarse, learned.scalar_flux(first))
    proposal_error = float(torch.linalg.vector_norm(predicted - higher) / torch.linalg.vector_norm(higher))
    assert proposal_error < 0.10

    phi_uc = solver.uncollided_fluence(fields, angle)
    cone = solver.cone_quadrature(w.grid, angle)
    converged = project_scatter(solver, None, w.grid, angle, phi_uc, total, fields, cone, signal_only=True)["signal"]
    primary = solver.primary(fields, angle)["signal"]
    mask = primary > 1e-3 * primary.max()

    def spr_error(scatter):
        return float(((scatter - converged)[mask].abs() / converged[mask].abs()).max())

    cold, _, _ = citrus_view_step(solver, CitrusState(cone_quadrature=cone), fields, angle, primary=False)
    step, _, state, judged = learned.learned_view_step(solver, CitrusState(cone_quadrature=cone), fields, angle,
                                                       proposal, primary=primary)
    assert spr_error(cold) > 0.10
    assert spr_error(step) < 0.005
    assert state.collided_moments is judged.accumulator and judged.spr_error_estimate[-1] <= 0.005

    plain, _ = learned.converged_view_step(solver, fields, angle, None, primary=primary, cone=cone)
    assert plain.spr_error_estimate[-1] <= 0.005 and spr_error(plain.scatter) < 0.005
    assert 3 * judged.sweeps <= 2 * plain.sweeps
