"""Generate the golden fixtures of the test suite by running the reference itself (cabouman/citrus v0.28.0).

Run in a checkout where the reference is available (it is read from /root/reference by default, or from the path in
CITRUS_REFERENCE). The reference imports xraylib at module level for element tables only; ``_shims/xraylib.py``
stands in for it (the synthetic library used here never reads those tables). Every fixture is small, float64, and
produced by the reference's own float64 CPU path; the script is deterministic (seeded).

    python tests/golden/make_golden.py [case ...]
"""

from __future__ import annotations

import math
import os
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REFERENCE = os.environ.get("CITRUS_REFERENCE", "/root/reference")
sys.path[:0] = [str(HERE / "_shims"), REFERENCE]

import torch  # noqa: E402

F64 = torch.float64
CASES = {}


def case(fn):
    CASES[fn.__name__] = fn
    return fn


def save(name, **arrays):
    out = {}
    for k, v in arrays.items():
        out[k] = v.detach().cpu().numpy() if isinstance(v, torch.Tensor) else np.asarray(v)
    np.savez_compressed(HERE / f"{name}.npz", **out)
    size = (HERE / f"{name}.npz").stat().st_size
    print(f"{name}.npz: {len(out)} arrays, {size / 1024:.1f} KiB")


@case
def sweep_small():
    """Reference sweep (PyTorch path, float64) of a random direction-dependent source on an anisotropic grid."""
    from citrus.scatter_solver.angular_quadrature import product_quadrature
    from citrus.scatter_solver.geometry import Grid
    from citrus.scatter_solver.transport_sweep import make_sweep_context, sweep

    g = torch.Generator().manual_seed(1234)
    grid = Grid((3, 4, 5), 0.7, 1.3 / 0.7, 0.9 / 0.7)
    quadrature = product_quadrature(4, 8, dtype=F64)
    L, G = 2, 3
    ctx = make_sweep_context(grid, quadrature, L, device="cpu", dtype=F64, backend="torch")
    mu = torch.rand(G, *grid.shape, generator=g, dtype=F64) * 1.5 + 0.1
    src = torch.randn(ctx.num_directions, G, 4, *grid.shape, generator=g, dtype=F64)
    phi, psi = sweep(ctx, mu, lambda idx: src.index_select(0, idx), direction_chunk=3, return_psi=True)
    save("sweep_small", shape=np.array(grid.shape), deltas=np.array(grid.deltas), L=L, mu=mu, source=src,
         omega=ctx.quadrature.omega, weight=ctx.quadrature.weight, permutation=ctx.permutation, phi=phi, psi=psi,
         c=ctx.c, plane_offsets=ctx.plan.plane_offsets, octant=ctx.plan.octant, cell=ctx.plan.cell,
         upstream=ctx.plan.upstream)


@case
def quadrature_tables():
    """Sweep product sets, harmonics and a cone set with cell widths."""
    from citrus.scatter_solver.angular_quadrature import (hemisphere_quadrature, product_quadrature,
                                                          real_spherical_harmonics)

    arrays = {}
    for p, a, L in ((4, 12, 3), (6, 20, 5), (10, 24, 7)):
        q = product_quadrature(p, a, dtype=F64)
        arrays[f"omega_{p}x{a}"] = q.omega
        arrays[f"weight_{p}x{a}"] = q.weight
        arrays[f"Y_{p}x{a}_L{L}"] = real_spherical_harmonics(L, q.omega)
    cone = hemisphere_quadrature([0.3, -0.9, 0.1], 8, 16, 0.4, dtype=F64, tangent_axes=((0.9, 0.3, 0.0),
                                                                                         (0.0, 0.0, 1.0)))
    arrays.update(cone_omega=cone.omega, cone_weight=cone.weight, cone_width=cone.cell_width)
    save("quadrature_tables", **arrays)


@case
def scatter_moments_small():
    """Scattering-source moments with and without the LD axis (angular_quadrature.scatter_source_moments)."""
    from citrus.scatter_solver.angular_quadrature import scatter_source_moments

    g = torch.Generator().manual_seed(77)
    G, L, spatial = 3, 2, (3, 4, 5)
    transfer = torch.rand(G, G, L + 2, *spatial, generator=g, dtype=F64)
    transfer[1, 0] = 0.0
    phi4 = torch.randn(G, (L + 1) ** 2, 4, *spatial, generator=g, dtype=F64)
    phi1 = torch.randn(G, (L + 1) ** 2, *spatial, generator=g, dtype=F64)
    save("scatter_moments_small", transfer=transfer, phi4=phi4, phi1=phi1,
         T4=scatter_source_moments(transfer, phi4), T1=scatter_source_moments(transfer, phi1))


@case
def siddon_small():
    """The five Siddon ray operations of the reference (PyTorch path, float64) on a small anisotropic grid, with a flat
    and a curved panel."""
    from citrus.scatter_solver.geometry import ConeGeometry, Grid
    from citrus.scatter_solver.ray_tracing import SiddonProjectors

    g = torch.Generator().manual_seed(99)
    grid = Grid((6, 7, 5), 1.1, 0.9, 1.3, recon_slice_offset=0.4)
    vol = torch.rand(2, *grid.shape, generator=g, dtype=F64)
    proj = SiddonProjectors(backend="torch")
    arrays = dict(volume=vol)
    omegas = torch.nn.functional.normalize(torch.randn(5, 3, generator=g, dtype=F64), dim=-1)
    points = (torch.rand(20, 3, generator=g, dtype=F64) - 0.5) * 14.0
    arrays.update(omegas=omegas, points=points)
    for name, curved in (("flat", False), ("curved", True)):
        geo = ConeGeometry(30.0, 45.0, 5, 7, 1.7, 1.9, det_row_offset=0.3, det_channel_offset=-0.2,
                           use_curved_detector=curved)
        angle = 0.7
        arrays[f"{name}_upstream"] = proj.upstream_cumulative(vol, grid, geo, angle)
        arrays[f"{name}_to_points"] = proj.upstream_to_points(vol, grid, geo, angle, points)
        arrays[f"{name}_primary"] = proj.primary_project(vol, grid, geo, angle)
        arrays[f"{name}_primary_n2"] = proj.primary_project(vol, grid, geo, angle, samples_per_pixel_axis=2)
        down = proj.downstream_cumulative(vol, grid, geo, angle, omegas)
        arrays[f"{name}_downstream"] = down
        arrays[f"{name}_oblique"] = proj.oblique_project(vol, grid, geo, angle, omegas)
        arrays[f"{name}_pixels"] = geo.pixel_centers(angle, dtype=F64)
    save("siddon_small", **arrays)


if __name__ == "__main__":
    names = sys.argv[1:] or list(CASES)
    for n in names:
        CASES[n]()
