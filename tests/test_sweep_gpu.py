"""Parity of the sm_103a sweep, small-K products and scattering moments with the float64 oracle."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import golden, rel_err
from citrus_gb300 import _lib, kernels
from citrus_gb300.geometry import Grid
from citrus_gb300.quadrature import product_quadrature
from citrus_gb300.source_iteration import scatter_moments, scatter_source_function, source_iteration
from citrus_gb300.transport_sweep import make_sweep_context, sweep
from oracle import sweep as osweep

pytestmark = pytest.mark.gpu
F32_REL = 1e-5  # float32 sweep vs float64 oracle, relative to the field maximum


def _direction_source(src):
    return lambda idx: src.index_select(0, idx)


@pytest.mark.parametrize("method", ["persistent", "planes"])
@pytest.mark.parametrize("chunk", [None, 3])
def test_sweep_matches_reference_fixture(cuda_device, method, chunk):
    g = golden("sweep_small")
    grid = Grid(tuple(g["shape"]), 0.7, 1.3 / 0.7, 0.9 / 0.7)
    ctx = make_sweep_context(grid, product_quadrature(4, 8), int(g["L"]), cuda_device)
    mu = torch.as_tensor(g["mu"], dtype=torch.float32, device=cuda_device)
    src = torch.as_tensor(g["source"], dtype=torch.float32, device=cuda_device)
    phi, psi = sweep(ctx, mu, _direction_source(src), direction_chunk=chunk, return_psi=True, method=method)
    assert rel_err(psi, g["psi"]) < F32_REL
    assert rel_err(phi, g["phi"]) < F32_REL


@pytest.mark.parametrize("shape, G, L, polar, azimuthal", [((9, 7, 8), 1, 3, 4, 12), ((6, 10, 5), 8, 5, 6, 20),
                                                           ((2, 2, 2), 12, 1, 2, 4), ((1, 5, 3), 16, 2, 4, 8)])
def test_sweep_matches_oracle(cuda_device, shape, G, L, polar, azimuthal):
    rng = np.random.default_rng(sum(shape) + G)
    grid = Grid(shape, 0.5, 1.2, 0.8)
    q = product_quadrature(polar, azimuthal)
    ctx = make_sweep_context(grid, q, L, cuda_device)
    mu = rng.random((G, *shape)) * 2.0 + 0.05
    src = rng.standard_normal((q.num_directions, G, 4, *shape))
    phi_ref, psi_ref = osweep.sweep(shape, grid.deltas, ctx.quadrature.omega, ctx.quadrature.weight, L, mu, src)
    for method in ("persistent", "planes"):
        phi, psi = sweep(ctx, torch.as_tensor(mu, dtype=torch.float32, device=cuda_device),
                         _direction_source(torch.as_tensor(src, dtype=torch.float32, device=cuda_device)),
                         return_psi=True, method=method)
        assert rel_err(psi, psi_ref) < F32_REL, method
        assert rel_err(phi, phi_ref) < F32_REL, method


def test_persistent_and_per_plane_sweeps_agree_bitwise(cuda_device):
    rng = np.random.default_rng(5)
    shape, G = (12, 9, 10), 8
    ctx = make_sweep_context(Grid(shape, 0.4), product_quadrature(6, 20), 5, cuda_device)
    mu = torch.as_tensor(rng.random((G, *shape)) + 0.1, dtype=torch.float32, device=cuda_device)
    src = torch.as_tensor(rng.standard_normal((120, G, 4, *shape)), dtype=torch.float32, device=cuda_device)
    a = sweep(ctx, mu, _direction_source(src), method="persistent")
    b = sweep(ctx, mu, _direction_source(src), method="planes")
    assert torch.equal(a, b)


def test_batched_views_sweep_matches_single_views(cuda_device):
    rng = np.random.default_rng(6)
    shape, G, V = (6, 5, 7), 4, 3
    ctx = make_sweep_context(Grid(shape, 0.5), product_quadrature(4, 8), 2, cuda_device)
    N = ctx.num_cells
    mu = torch.as_tensor(rng.random((N, G)) + 0.1, dtype=torch.float32, device=cuda_device)
    c = ctx.c.contiguous()
    stores = torch.as_tensor(rng.standard_normal((V, 8, 4, N, 4 * G)), dtype=torch.float32, device=cuda_device)
    single = stores.clone()
    for v in range(V):
        kernels.sweep_planes(ctx.flat_index, single[v], mu, c, method="planes")
    for form in (1, 2, 3, 4, 5):   # every thread form the autotuner chooses between
        batched = stores.clone()
        sync = kernels.sweep_planes(ctx.flat_index, batched, mu, c, method="persistent", thread_form=form)
        assert torch.equal(single, batched), form
        assert int(sync[2]) == 0


def test_persistent_barrier_timeout_is_reported(cuda_device):
    """A block that never arrives makes every barrier wait run out after the bounded timeout; the kernel returns and
    the sync word records it (no hang, the context stays usable)."""
    ctx = make_sweep_context(Grid((4, 4, 4), 1.0), product_quadrature(2, 4), 1, cuda_device)
    N, G = ctx.num_cells, 2
    store = torch.zeros(8, 1, N, 4 * G, device=cuda_device)
    mu = torch.ones(N, G, device=cuda_device)
    sync = kernels.sweep_planes(ctx.flat_index, store, mu, ctx.c.contiguous(), max_blocks=4,
                                timeout_ns=20_000_000, skip_block=1)
    torch.cuda.synchronize()
    assert int(sync[2]) != 0
    ok = kernels.sweep_planes(ctx.flat_index, store, mu, ctx.c.contiguous(), max_blocks=4)
    torch.cuda.synchronize()
    assert int(ok[2]) == 0


@pytest.mark.parametrize("shape, G, V, tile", [((5, 7, 6), 3, 2, 2), ((12, 9, 10), 8, 3, 4), ((9, 8, 17), 1, 1, 8),
                                              ((16, 16, 16), 4, 2, 8), ((6, 5, 7), 2, 2, 3)])
def test_tiled_sweep_equals_per_plane_sweep_bitwise(cuda_device, shape, G, V, tile):
    """The tiled schedule (grid barrier per tile diagonal, block barrier per sub-plane) gives the per-plane kernel's
    store bit for bit, for tiles that divide the grid or not, every thread form and directions per task."""
    rng = np.random.default_rng(sum(shape) + G)
    ctx = make_sweep_context(Grid(shape, 0.5), product_quadrature(4, 12), 2, cuda_device)
    N, D8 = ctx.num_cells, ctx.directions_per_octant
    mu = torch.as_tensor(rng.random((N, G)) + 0.1, dtype=torch.float32, device=cuda_device)
    c = ctx.c.contiguous()
    stores = torch.as_tensor(rng.standard_normal((V, 8, D8, N, 4 * G)), dtype=torch.float32, device=cuda_device)
    expected = stores.clone()
    for v in range(V):
        kernels.sweep_planes(ctx.flat_index, expected[v], mu, c, method="planes")
    for form in (1, 2):
        for dpb in sorted({1, 2, D8}):
            got = stores.clone()
            sync = kernels.sweep_tiled(ctx.tiled_index(tile), got, mu, c, dirs_per_block=dpb, thread_form=form)
            assert torch.equal(got, expected), (form, dpb)
            assert int(sync[2]) == 0


def test_tiled_sweep_inside_the_accumulator_step_form(cuda_device):
    """kernels.sweep_chunk with a tiled form on one view equals the plane wavefront's persistent form."""
    rng = np.random.default_rng(9)
    shape, G = (10, 8, 9), 4
    ctx = make_sweep_context(Grid(shape, 0.5), product_quadrature(4, 8), 2, cuda_device)
    N, D8 = ctx.num_cells, ctx.directions_per_octant
    mu = torch.as_tensor(rng.random((N, G)) + 0.1, dtype=torch.float32, device=cuda_device)
    store = torch.as_tensor(rng.standard_normal((2, 8, D8, N, 4 * G)), dtype=torch.float32, device=cuda_device)
    a, b = store.clone(), store.clone()
    kernels.sweep_chunk(ctx, a, mu, ctx.c, kernels.SweepForm(1, 0, 1))
    kernels.sweep_chunk(ctx, b, mu, ctx.c, kernels.SweepForm(2, 4, 2))
    assert torch.equal(a, b)


def test_tiled_barrier_timeout_is_reported(cuda_device):
    """A block of the tiled launch that never arrives makes every diagonal's barrier wait run out after the bounded
    timeout; the kernel returns, the sync word records it, and the next launch runs normally."""
    ctx = make_sweep_context(Grid((8, 8, 8), 1.0), product_quadrature(2, 4), 1, cuda_device)
    N, G = ctx.num_cells, 2
    store = torch.zeros(8, 1, N, 4 * G, device=cuda_device)
    mu = torch.ones(N, G, device=cuda_device)
    index = ctx.tiled_index(4)
    sync = kernels.sweep_tiled(index, store, mu, ctx.c.contiguous(), max_blocks=4, timeout_ns=20_000_000,
                               skip_block=1)
    torch.cuda.synchronize()
    assert int(sync[2]) != 0
    ok = kernels.sweep_tiled(index, store, mu, ctx.c.contiguous(), max_blocks=4)
    torch.cuda.synchronize()
    assert int(ok[2]) == 0


@pytest.mark.parametrize("M, K, J, batch, accumulate", [(120, 36, 4096, 1, False), (36, 120, 1028, 1, True),
                                                        (5, 7, 64, 3, True), (240, 64, 512, 2, False),
                                                        (1, 1, 4, 1, False), (133, 36, 515, 1, True),
                                                        (129, 17, 1000, 2, False), (64, 65, 777, 1, True),
                                                        (3, 300, 258, 2, False), (100, 80, 96, 1, True),
                                                        (512, 36, 2050, 1, False)])
def test_small_k_gemm_matches_numpy(cuda_device, M, K, J, batch, accumulate):
    rng = np.random.default_rng(M * 7 + K)
    A = rng.standard_normal((M, K))
    B = rng.standard_normal((batch, K, J))
    C0 = rng.standard_normal((batch, M, J))
    expected = np.einsum("mk,bkj->bmj", A, B) + (C0 if accumulate else 0)
    dev = lambda x: torch.as_tensor(x, dtype=torch.float32, device=cuda_device)  # noqa: E731
    C = dev(C0)
    kernels.small_k_gemm(dev(A), dev(B), C, accumulate=accumulate)
    assert rel_err(C, expected) < 1e-5


@pytest.mark.parametrize("M, K, J, batch", [(120, 36, 4096, 2), (133, 36, 2060, 1), (5, 7, 64, 3), (1, 1, 4, 1),
                                            (64, 64, 1032, 2), (17, 20, 516, 1)])
def test_source_expansion_with_first_collision_means_equals_two_passes(cuda_device, M, K, J, batch):
    """C = A B + (F, 0, 0, 0) in one pass equals the quadruples written into C and an accumulating product over them
    (the same products in the same order), bit for bit."""
    rng = np.random.default_rng(M + K + J)
    dev = lambda x: torch.as_tensor(x, dtype=torch.float32, device=cuda_device)  # noqa: E731
    A, B, F = dev(rng.standard_normal((M, K))), dev(rng.standard_normal((batch, K, J))), dev(
        rng.standard_normal((batch, M, J // 4)))
    two = torch.zeros(batch, M, J // 4, 4, device=cuda_device)
    two[..., 0] = F
    two = two.reshape(batch, M, J)
    # the accumulating product in its streaming (column-stationary) form, the one the single pass extends
    _lib.call("citrus_small_k_gemm_config", A.data_ptr(), K, B.data_ptr(), J, two.data_ptr(), J, M, K, J, batch,
              K * J, M * J, 1, 1, 0, _lib.stream_handle(two.device))
    one = torch.full((batch, M, J), float("nan"), device=cuda_device)
    kernels.source_expansion_first(A, B, one, F)
    assert torch.equal(one, two)
    expected = np.einsum("mk,bkj->bmj", A.cpu().numpy().astype(np.float64), B.cpu().numpy().astype(np.float64))
    expected.reshape(batch, M, J // 4, 4)[..., 0] += F.cpu().numpy()
    assert rel_err(one, expected) < 1e-5


@pytest.mark.parametrize("M, K, J, batch, accumulate", [(120, 36, 4096, 1, False), (36, 120, 1028, 1, True),
                                                        (5, 7, 64, 3, True), (1, 1, 4, 1, False),
                                                        (128, 128, 333, 2, True), (64, 36, 130, 1, False)])
def test_bf16x3_tensor_core_gemm_error_against_float64(cuda_device, M, K, J, batch, accumulate):
    """The bfloat16 hi/lo product on the tensor cores: its error against float64 stays at the split's ~1e-5 of the
    largest term, far below bfloat16's own."""
    rng = np.random.default_rng(M * 13 + K)
    A = rng.standard_normal((M, K))
    B = rng.standard_normal((batch, K, J))
    C0 = rng.standard_normal((batch, M, J))
    expected = np.einsum("mk,bkj->bmj", A, B) + (C0 if accumulate else 0)
    dev = lambda x: torch.as_tensor(x, dtype=torch.float32, device=cuda_device)  # noqa: E731
    C = dev(C0)
    err = torch.zeros(1, dtype=torch.int32, device=cuda_device)
    kernels.small_k_gemm(dev(A), dev(B), C, accumulate=accumulate, precision="bf16x3", error_word=err,
                         tensor_cores_only=True)
    torch.cuda.synchronize()
    assert int(err[0]) == 0
    scale = np.abs(A).max() * np.abs(B).max() * K
    assert np.abs(C.cpu().numpy() - expected).max() / scale < 3e-5


@pytest.mark.parametrize("M, K, J, batch", [(120, 36, 4096, 2), (240, 64, 1032, 1), (48, 16, 516, 3),
                                            (5, 7, 64, 1), (128, 36, 2052, 1)])
def test_tensor_core_source_expansion_with_means_against_float64(cuda_device, M, K, J, batch):
    """The source of an accumulator sweep in the mixed precision (tcgen05, bfloat16 hi/lo split, the first-collision
    means added in the epilogue): C = A B + (F, 0, 0, 0) against float64 within the split's ~1e-5 of the largest
    term, over 128-row launches (M = 240), row counts from 5 to 128 and partial column tiles."""
    rng = np.random.default_rng(M + 3 * K + J)
    A = rng.standard_normal((M, K))
    B = rng.standard_normal((batch, K, J))
    F = rng.standard_normal((batch, M, J // 4))
    expected = np.einsum("mk,bkj->bmj", A, B)
    expected.reshape(batch, M, J // 4, 4)[..., 0] += F
    dev = lambda x: torch.as_tensor(x, dtype=torch.float32, device=cuda_device)  # noqa: E731
    C = torch.full((batch, M, J), float("nan"), device=cuda_device)   # written, never read
    err = torch.zeros(1, dtype=torch.int32, device=cuda_device)
    kernels.source_expansion_first(dev(A), dev(B), C, dev(F), precision="bf16x3", error_word=err)
    torch.cuda.synchronize()
    assert int(err[0]) == 0
    scale = np.abs(A).max() * np.abs(B).max() * K
    assert np.abs(C.cpu().numpy() - expected).max() / scale < 3e-5
    fp32 = torch.empty_like(C)
    kernels.source_expansion_first(dev(A), dev(B), fp32, dev(F))
    assert float((C - fp32).abs().max()) / scale < 3e-5


@pytest.mark.parametrize("M, K, J, batch, accumulate, means", [(120, 36, 4096, 2, False, True),
                                                               (36, 64, 2052, 1, True, False),
                                                               (64, 36, 1024, 3, False, False),
                                                               (100, 48, 132, 1, False, True),
                                                               (17, 20, 260, 2, True, False)])
def test_warp_specialised_tensor_core_product_equals_single_stage(cuda_device, monkeypatch, M, K, J, batch,
                                                                  accumulate, means):
    """The warp-specialised tcgen05 product (tensor-copy loader, converters, MMA issuer, double-buffered accumulators,
    epilogue warps, the means by tensor copy where their strides allow a tensor map) performs the single-stage
    kernel's MMAs in the same order and the same epilogue: the same bits, for 17 to 120 rows, with accumulation, with
    the first-collision means (by tensor copy, and read directly where J / 4 is not a multiple of 4) and a partial last
    tile."""
    rng = np.random.default_rng(M * 5 + K + J)
    dev = lambda x: torch.as_tensor(x, dtype=torch.float32, device=cuda_device)  # noqa: E731
    A, B = dev(rng.standard_normal((M, K))), dev(rng.standard_normal((batch, K, J)))
    C0, F = dev(rng.standard_normal((batch, M, J))), dev(rng.standard_normal((batch, M, J // 4)))
    results = []
    for form in ("ws", "single"):
        if form == "single":
            monkeypatch.setenv("CITRUS_TC_FORM", "single")
        else:
            monkeypatch.delenv("CITRUS_TC_FORM", raising=False)
        C = C0.clone()
        err = torch.zeros(1, dtype=torch.int32, device=cuda_device)
        if means:
            kernels.source_expansion_first(A, B, C, F, precision="bf16x3", error_word=err)
        else:
            kernels.small_k_gemm(A, B, C, accumulate=accumulate, precision="bf16x3", error_word=err,
                                 tensor_cores_only=True)
        torch.cuda.synchronize()
        assert int(err[0]) == 0
        results.append(C)
    assert torch.equal(results[0], results[1])
    expected = np.einsum("mk,bkj->bmj", A.double().cpu().numpy(), B.double().cpu().numpy())
    if accumulate:
        expected += C0.double().cpu().numpy()
    if means:
        expected.reshape(batch, M, J // 4, 4)[..., 0] += F.double().cpu().numpy()
    scale = float(A.abs().max() * B.abs().max()) * K
    assert np.abs(results[0].double().cpu().numpy() - expected).max() / scale < 3e-5


def test_scattering_moments_match_reference_fixture(cuda_device):
    g = golden("scatter_moments_small")
    dev = lambda x: torch.as_tensor(x, dtype=torch.float32, device=cuda_device)  # noqa: E731
    for layout in kernels.LAYOUTS:
        assert rel_err(kernels.scattering_moments(dev(g["transfer"]), dev(g["phi4"]), layout), g["T4"]) < 1e-5
        assert rel_err(kernels.scattering_moments(dev(g["transfer"]), dev(g["phi1"]), layout), g["T1"]) < 1e-5
    # a strided view of cell-major storage, as the sweep returns it
    storage = dev(np.ascontiguousarray(np.moveaxis(g["phi4"], (0, 2), (4, 5))))  # [N, R, C, S, G, 4]
    view = kernels.cell_major_view(storage, 3)
    assert rel_err(scatter_moments(dev(g["transfer"]), view), g["T4"]) < 1e-5


def test_source_iteration_matches_oracle(cuda_device):
    rng = np.random.default_rng(8)
    shape, G, L = (5, 6, 4), 3, 3
    grid = Grid(shape, 0.6)
    q = product_quadrature(4, 8)
    ctx = make_sweep_context(grid, q, L, cuda_device)
    mu = rng.random((G, *shape)) * 1.0 + 0.5
    transfer = np.zeros((G, G, L + 1, *shape))
    for gi in range(G):
        for go in range(gi, G):
            transfer[gi, go, 0] = 0.2 * (0.5 ** (go - gi)) * mu[gi]
            transfer[gi, go, 1] = 0.05 * transfer[gi, go, 0]
    first = np.abs(rng.standard_normal((32, G, 4, *shape)))
    total, n, history = osweep.source_iteration(shape, grid.deltas, ctx.quadrature.omega, ctx.quadrature.weight, L,
                                                mu, transfer, first, 1e-3, 12)
    dev = lambda x: torch.as_tensor(x, dtype=torch.float32, device=cuda_device)  # noqa: E731
    result = source_iteration(ctx, dev(mu), dev(transfer), _direction_source(dev(first)), 1e-3, 12)
    assert result.num_iterations == n
    assert rel_err(result.phi_total, total) < 2e-5
    np.testing.assert_allclose(result.history, history, rtol=1e-3)
    # the cell-major source function of the scattering source against the oracle's expansion
    T = scatter_moments(dev(transfer), result.phi_total)
    source = scatter_source_function(ctx, T)
    idx = torch.arange(ctx.num_directions, device=cuda_device)
    got = source(idx).permute(0, 4, 5, 1, 2, 3)
    from citrus_gb300.quadrature import real_spherical_harmonics
    expected = osweep.scatter_source(real_spherical_harmonics(L, ctx.quadrature.omega),
                                     osweep.scatter_moments(transfer, result.phi_total.double().cpu().numpy()))
    assert rel_err(got, expected) < 1e-5


@pytest.mark.parametrize("M,K,acc", [(120, 36, True), (36, 120, False), (64, 36, False), (20, 36, True)])
def test_every_small_k_gemm_variant_matches(cuda_device, tmp_path, M, K, acc):
    """Each kernel the autotuner chooses between gives the product (float64 reference), and the tuned call too."""
    from citrus_gb300 import _lib
    from citrus_gb300.autotune import GEMM_CANDIDATES, Autotuner
    import citrus_gb300.autotune as autotune

    gen = torch.Generator().manual_seed(M + K)
    batch, J = 2, 4096 + 8
    A = torch.randn(M, K, generator=gen).to(cuda_device)
    B = torch.randn(batch, K, J, generator=gen).to(cuda_device)
    C0 = torch.randn(batch, M, J, generator=gen).to(cuda_device)
    ref = torch.einsum("mk,bkj->bmj", A.double(), B.double()) + (C0.double() if acc else 0)
    stream = _lib.stream_handle(cuda_device)
    ran = 0
    for variant, tile in GEMM_CANDIDATES:
        C = C0.clone()
        try:
            _lib.call("citrus_small_k_gemm_config", A.data_ptr(), K, B.data_ptr(), J, C.data_ptr(), J, M, K, J,
                      batch, K * J, M * J, int(acc), variant, tile, stream)
        except _lib.CitrusKernelError:
            continue        # a tile the shape does not admit (shared memory)
        ran += 1
        assert float((C.double() - ref).abs().max() / ref.abs().max()) < 1e-5, (variant, tile)
    assert ran >= 3
    saved = autotune._TUNER
    autotune._TUNER = Autotuner(path=tmp_path / "tuning.json", enabled=True)
    try:
        C = C0.clone()
        kernels.small_k_gemm(A, B, C, accumulate=acc)
        assert float((C.double() - ref).abs().max() / ref.abs().max()) < 1e-5
        assert len(autotune._TUNER.table) == 1
    finally:
        autotune._TUNER = saved
