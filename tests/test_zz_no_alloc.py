"""The allocation-free persistent sweep (``citrus_sweep_persistent_static``) against the caller-scratch one.

Collected last on purpose: the static scratch is shared by every call on a device, so this file also shows that the
entry point gives the same results after the rest of the suite has run on the same process and device.
"""

from __future__ import annotations

import ctypes

import numpy as np
import pytest
import torch

from citrus_gb300 import _lib, kernels
from citrus_gb300.geometry import Grid
from citrus_gb300.quadrature import product_quadrature
from citrus_gb300.transport_sweep import make_sweep_context

pytestmark = pytest.mark.gpu


def _problem(device, shape, G, views, seed):
    rng = np.random.default_rng(seed)
    ctx = make_sweep_context(Grid(shape, 0.5, 1.1, 0.9), product_quadrature(4, 8), 2, device)
    N = ctx.num_cells
    mu = torch.as_tensor(rng.random((N, G)) + 0.1, dtype=torch.float32, device=device)
    store = torch.as_tensor(rng.standard_normal((views, 8, ctx.directions_per_octant, N, 4 * G)),
                            dtype=torch.float32, device=device)
    return ctx, mu, store


def _static_sweep(ctx, store, mu, timeout_word):
    index = ctx.flat_index
    views, _, Dc, N, Q = store.shape
    offsets = np.ascontiguousarray(np.asarray(index.offsets, dtype=np.int32))
    c = ctx.c.contiguous()
    _lib.call("citrus_sweep_persistent_static", store.data_ptr(), mu.data_ptr(), c.data_ptr(),
              index.octant.data_ptr(), index.cell.data_ptr(), index.upstream.data_ptr(),
              offsets.ctypes.data_as(ctypes.c_void_p), index.num_planes, N, Q // 4, Dc, views,
              timeout_word.data_ptr(), kernels.DEFAULT_BARRIER_TIMEOUT_NS, _lib.stream_handle(store.device))


@pytest.mark.parametrize("shape, G, views", [((7, 6, 5), 8, 2), ((11, 4, 9), 3, 1)])
def test_static_scratch_sweep_matches_caller_scratch_sweep(cuda_device, shape, G, views):
    ctx, mu, store = _problem(cuda_device, shape, G, views, seed=sum(shape) + G)
    c = ctx.c.contiguous()
    timeout_word = torch.full((1,), 7, dtype=torch.int32, device=cuda_device)
    for call in range(2):  # two calls in a row through the same static scratch
        inputs = store * (1.0 + call) - 0.25 * call
        expected = inputs.clone()
        sync = kernels.sweep_planes(ctx.flat_index, expected, mu, c, method="persistent")
        got = inputs.clone()
        _static_sweep(ctx, got, mu, timeout_word)
        torch.cuda.synchronize()
        assert int(sync[2]) == 0
        assert int(timeout_word[0]) == 0, f"call {call}: barrier timeout reported"
        assert torch.equal(got, expected), f"call {call}"


def test_static_scratch_sweep_rejects_too_many_planes(cuda_device):
    ctx, mu, store = _problem(cuda_device, (3, 3, 3), 1, 1, seed=1)
    index = ctx.flat_index
    offsets = np.zeros(8193, dtype=np.int32)
    with pytest.raises(_lib.CitrusKernelError, match="exceed the static scratch"):
        _lib.call("citrus_sweep_persistent_static", store.data_ptr(), mu.data_ptr(), ctx.c.contiguous().data_ptr(),
                  index.octant.data_ptr(), index.cell.data_ptr(), index.upstream.data_ptr(),
                  offsets.ctypes.data_as(ctypes.c_void_p), 8192, ctx.num_cells, 1, ctx.directions_per_octant, 1,
                  None, kernels.DEFAULT_BARRIER_TIMEOUT_NS, _lib.stream_handle(store.device))
