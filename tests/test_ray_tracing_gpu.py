"""Parity of the sm_103a Siddon kernels with the reference fixtures and the float64 oracle."""

from __future__ import annotations

import math

import numpy as np
import pytest
import torch

from conftest import golden, rel_err
from citrus_gb300.geometry import ConeGeometry, Grid
from citrus_gb300.ray_tracing import GB300Projectors
from oracle import siddon
from test_oracle_golden import _siddon_setup, finite_rel_err

pytestmark = pytest.mark.gpu
PATH_REL = 1e-6  # path lengths of the upstream and primary traces, relative to the largest


@pytest.mark.parametrize("name", ["flat", "curved"])
def test_projectors_match_reference_fixture(cuda_device, name):
    g = golden("siddon_small")
    grid, geos = _siddon_setup()
    geo, angle = geos[name], 0.7
    vol = torch.as_tensor(g["volume"], dtype=torch.float32, device=cuda_device)
    p = GB300Projectors()
    assert rel_err(p.upstream_cumulative(vol, grid, geo, angle), g[f"{name}_upstream"]) < 2e-6
    pts = torch.as_tensor(g["points"], device=cuda_device)
    assert rel_err(p.upstream_to_points(vol, grid, geo, angle, pts), g[f"{name}_to_points"]) < 2e-6
    assert rel_err(p.primary_project(vol, grid, geo, angle), g[f"{name}_primary"]) < 2e-6
    assert rel_err(p.primary_project(vol, grid, geo, angle, samples_per_pixel_axis=2), g[f"{name}_primary_n2"]) < 2e-6
    om = torch.as_tensor(g["omegas"], dtype=torch.float32, device=cuda_device)
    down = p.downstream_cumulative(vol, grid, geo, angle, om).cpu().numpy()
    assert finite_rel_err(down, g[f"{name}_downstream"]) < 1e-5
    assert rel_err(p.oblique_project(vol, grid, geo, angle, om), g[f"{name}_oblique"]) < 1e-5
    # a rows-outer output buffer, as the scatter image writes it
    K, C = om.shape[0], vol.shape[0]
    Rd, Cd = geo.image_shape
    rows_outer = torch.empty(K, Rd, C, Cd, device=cuda_device)
    p.oblique_project(vol, grid, geo, angle, om, out=rows_outer.permute(0, 2, 1, 3))
    assert rel_err(rows_outer.permute(0, 2, 1, 3), g[f"{name}_oblique"]) < 1e-5


def _cylinder_phantom(grid):
    c = siddon.centers(grid)
    r = np.hypot(c[..., 0], c[..., 1])
    water = (r < 7.0).astype(np.float64)
    bone = (np.hypot(c[..., 0] - 3.0, c[..., 1] + 1.5) < 1.0).astype(np.float64)
    return np.stack([water * (1 - bone) + 0.0012 * (1 - water), 1.85 * bone])


@pytest.mark.parametrize("curved", [False, True])
def test_path_lengths_within_one_part_per_million(cuda_device, curved):
    """The 32^3 water-cylinder phantom: upstream traces to every voxel centre and primary traces to every pixel of a
    64 x 64 panel against the float64 oracle, within 1e-6 of the largest path."""
    grid = Grid((32, 32, 32), 0.5)
    geo = ConeGeometry(100.0, 150.0, 64, 64, 0.4, 0.4, use_curved_detector=curved)
    rho = _cylinder_phantom(grid)
    vol = torch.as_tensor(rho, dtype=torch.float32, device=cuda_device)
    p = GB300Projectors()
    for angle in (0.0, 0.37, 2.2):
        up = p.upstream_cumulative(vol, grid, geo, angle)
        ref = siddon.upstream_to_points(rho, grid, geo.source_position(angle), siddon.centers(grid).reshape(-1, 3))
        assert rel_err(up.reshape(2, -1), ref) < PATH_REL
        prim = p.primary_project(vol, grid, geo, angle)
        assert rel_err(prim, siddon.primary_project(rho, grid, geo, angle)) < PATH_REL


def test_random_segments_and_edge_cases(cuda_device):
    rng = np.random.default_rng(3)
    grid = Grid((5, 9, 4), 0.8, 1.2, 0.7)
    vol = rng.random((3, *grid.shape))
    ext = np.asarray(grid.extent)
    starts = (rng.random((500, 3)) - 0.5) * ext * 3
    ends = (rng.random((500, 3)) - 0.5) * ext * 3
    # axis-aligned rays along grid planes, zero-length rays, rays missing the box and rays inside one voxel
    starts[:4] = [[-10, 0.0, 0.1], [0.4, -10, 0.35], [0.2, 0.3, 0.0], [50, 50, 50]]
    ends[:4] = [[10, 0.0, 0.1], [0.4, 10, 0.35], [0.2, 0.3, 0.0], [60, 50, 50]]
    starts[4], ends[4] = [0.1, 0.1, 0.1], [0.2, 0.15, 0.12]
    got = GB300Projectors().line_integrals(torch.as_tensor(vol, dtype=torch.float32, device=cuda_device),
                                           torch.as_tensor(starts), torch.as_tensor(ends), grid)
    assert rel_err(got, siddon.line_integrals(vol, starts, ends, grid)) < 1e-5


def test_oblique_line_grazing_a_box_face(cuda_device):
    """Pixel centres whose float64 z lies just outside a face of the box, with cone directions whose z component is
    ~1e-17: the lines miss the box in float64 (the reference) and must not integrate the face slice after a float32
    rounding of the pixel centre."""
    from citrus_gb300.scatter_image import panel_direction_set
    grid = Grid((8, 8, 6), 1.0)
    rng = np.random.default_rng(0)
    field = rng.random((3, *grid.shape))
    geo = ConeGeometry(40.0, 60.0, 12, 16, 1.2, 1.2)
    cone = panel_direction_set(geo, 0.6, (3, 6), max_polar_angle=Grid.covering(grid, 2.0))
    om = cone.omega[:6]
    assert np.abs(om[:, 2]).min() < 1e-15
    ref = siddon.oblique_project(field, grid, geo, 0.6, om)
    got = GB300Projectors().oblique_project(torch.as_tensor(field, dtype=torch.float32, device=cuda_device), grid,
                                            geo, 0.6, torch.as_tensor(om, dtype=torch.float32, device=cuda_device))
    assert rel_err(got, ref) < 1e-5


@pytest.mark.parametrize("channels", [1, 2, 3, 8])
@pytest.mark.parametrize("curved", [False, True])
@pytest.mark.parametrize("sdd", [45.0, 32.0])
def test_downstream_lattice_walk_matches_per_ray_walk_and_oracle(cuda_device, channels, curved, sdd):
    """The shared per-direction crossing table against the independent per-ray walk and the float64 oracle, with
    directions along the axes, in the planes of two axes and oblique, on a grid with unequal voxel sizes; with the
    panel beyond the grid (sdd 45) and through it (sdd 32: rays end at the panel, inside the box)."""
    grid = Grid((9, 7, 6), 1.1, 0.8 / 1.1, 1.3 / 1.1)
    rng = np.random.default_rng(channels)
    vol_np = rng.random((channels, *grid.shape))
    geo = ConeGeometry(30.0, sdd, 10, 12, 1.5, 1.5, use_curved_detector=curved)
    angle = 0.4
    n_hat = np.asarray(geo.panel_axes(angle)[2])
    om = rng.standard_normal((40, 3))
    om[0] = -n_hat
    om[1] = [0.0, 0.0, 1.0]
    om[2] = [1.0, 0.0, 0.0]
    om[3] = [0.0, -1.0, 0.0]
    om[4] = [0.6, -0.8, 0.0]
    om[5] = [0.0, 0.6, 0.8]
    om /= np.linalg.norm(om, axis=1, keepdims=True)
    om32 = om.astype(np.float32)
    vol = torch.as_tensor(vol_np, dtype=torch.float32, device=cuda_device)
    omt = torch.as_tensor(om32, device=cuda_device)
    p = GB300Projectors()
    lattice = p.downstream_cumulative(vol, grid, geo, angle, omt).cpu().numpy()
    walk = p.downstream_cumulative(vol, grid, geo, angle, omt, lattice=False).cpu().numpy()
    ref = siddon.downstream_cumulative(vol_np, grid, geo, angle, om32.astype(np.float64))
    assert np.array_equal(np.isinf(lattice), np.isinf(ref))
    assert finite_rel_err(lattice, walk) < 1e-5
    assert finite_rel_err(lattice, ref) < 1e-5


@pytest.mark.parametrize("channels, curved", [(1, False), (2, True), (8, True), (3, False)])
def test_oblique_direction_table_equals_per_block_set_up(cuda_device, channels, curved):
    """The oblique projection with its per-direction constants formed once by the set-up kernel (the scratch entry
    point) gives the same bits as with the constants formed in every block."""
    from citrus_gb300 import _lib
    from citrus_gb300.ray_tracing import HostArgs, _grid_args, _pixel_centers
    grid = Grid((9, 11, 7), 0.7)
    geo = ConeGeometry(40.0, 70.0, 24, 30, 0.6, 0.5, det_channel_offset=0.3, use_curved_detector=curved)
    rng = np.random.default_rng(channels)
    K = 37
    om = rng.normal(size=(K, 3))
    om /= np.linalg.norm(om, axis=1, keepdims=True)
    omegas = torch.as_tensor(om, dtype=torch.float32, device=cuda_device)
    field = torch.as_tensor(rng.random((K, grid.num_voxels, channels)), dtype=torch.float32, device=cuda_device)
    pixels = _pixel_centers(geo, 1.3, cuda_device)
    Rd, Cd = geo.image_shape
    host = HostArgs()
    box, dims = _grid_args(host, grid)
    outs = []
    for scratch in (False, True):
        out = torch.full((K, channels, Rd, Cd), float("nan"), device=cuda_device)
        head = (field.data_ptr(), channels, grid.num_voxels * channels, box, dims, omegas.data_ptr(), K,
                pixels.data_ptr(), Rd, Cd, out.data_ptr(), *out.stride())
        if scratch:
            n = int(_lib.library().citrus_oblique_scratch_bytes(K))
            buf = torch.empty(n, device=cuda_device, dtype=torch.uint8)
            _lib.call("citrus_oblique_project_scratch", *head, buf.data_ptr(), n, _lib.stream_handle(cuda_device))
            with pytest.raises(_lib.CitrusKernelError, match="direction scratch"):
                _lib.call("citrus_oblique_project_scratch", *head, buf.data_ptr(), n - 17,
                          _lib.stream_handle(cuda_device))
        else:
            _lib.call("citrus_oblique_project", *head, _lib.stream_handle(cuda_device))
        outs.append(out)
    assert torch.isfinite(outs[0]).all() and float(outs[0].abs().max()) > 0
    assert torch.equal(outs[0], outs[1])


@pytest.mark.parametrize("curved", [False, True])
def test_prebuilt_crossing_tables_give_the_same_walk(cuda_device, curved):
    """The downstream walk over crossing tables built once for a whole direction set (``crossing_tables``, taken
    in row slices per chunk) equals the walk that builds the tables of its own chunk."""
    grid = Grid((10, 12, 9), 0.8)
    geo = ConeGeometry(40.0, 70.0, 16, 20, 0.8, 0.8, use_curved_detector=curved)
    rng = np.random.default_rng(3)
    mu = torch.as_tensor(rng.random((2, *grid.shape)) * 0.3, dtype=torch.float32, device=cuda_device)
    om = rng.normal(size=(29, 3))
    om /= np.linalg.norm(om, axis=1, keepdims=True)
    omegas = torch.as_tensor(om, dtype=torch.float32, device=cuda_device)
    p = GB300Projectors()
    tables = p.crossing_tables(grid, omegas)
    for s, e in ((0, 13), (13, 29)):
        own = p.downstream_cumulative(mu, grid, geo, 0.7, omegas[s:e], voxel_major=True)
        kept = p.downstream_cumulative(mu, grid, geo, 0.7, omegas[s:e], voxel_major=True, crossings=tables[s:e])
        assert torch.equal(own, kept)
    with pytest.raises(ValueError, match="crossings"):
        p.downstream_cumulative(mu, grid, geo, 0.7, omegas[:13], voxel_major=True, crossings=tables[:12])
