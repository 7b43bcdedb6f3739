"""The per-view accumulator store (reference ``citrus/citrus.py:623-757``): scaled float16 cell means."""

from __future__ import annotations

import numpy as np
import pytest
import torch

from conftest import golden
from citrus_gb300.state_store import StateStore

SHAPE = (3, 16, 4, 4, 5, 6)  # [G, (L+1)^2 with L = 3, 4, Rc, Cc, Sc]


def test_location_and_sizes_without_a_gpu():
    """The storage decision is host arithmetic: the 0.5 cm WLAB accumulator with 1 cm cells is 17.6 MiB per view,
    36 views fit the default 2600 MiB GPU budget, 180 views go to pinned host memory."""
    shape = (6, 64, 4, 20, 30, 40)
    per = int(np.prod(shape)) * 4
    s36 = StateStore(36, shape, "cuda")
    assert s36.bytes_per_view < per / 7.9 and abs(s36.bytes_per_view / 2 ** 20 - 17.6) < 0.1
    assert s36.location == "gpu"
    s180 = StateStore(180, shape, "cuda")
    assert s180.location == "cpu" and s180.pinned
    assert StateStore(180, shape, "cuda", gpu_budget_mib=4000).location == "gpu"
    assert StateStore(2, shape, "cpu").location == "cpu" and not StateStore(2, shape, "cpu").pinned
    with pytest.raises(ValueError):
        StateStore(2, shape[:5], "cuda")
    with pytest.raises(ValueError):
        StateStore(2, shape, "cuda", location="disk")


def _phi(seed, device):
    g = torch.Generator().manual_seed(seed)
    # collided moments ~1e-6 per source photon: plain float16 would underflow, the scaled form does not
    phi = 1e-6 * torch.randn(SHAPE, generator=g) * torch.logspace(0, -3, SHAPE[1])[None, :, None, None, None, None]
    # the sweep's cell-major storage [N, Rc, Cc, Sc, G, 4] seen as [G, N, 4, Rc, Cc, Sc]
    return phi.permute(1, 3, 4, 5, 0, 2).contiguous().to(device).permute(4, 0, 5, 1, 2, 3)


@pytest.mark.gpu
@pytest.mark.parametrize("location", ["gpu", "cpu"])
def test_round_trip_is_the_reference_codec(cuda_device, location):
    store = StateStore(3, SHAPE, cuda_device, location=location)
    assert store.get(0) is None and store.location == location
    phis = [_phi(i, cuda_device) for i in range(3)]
    for i, p in enumerate(phis):
        store.put(i, p)
    for i, p in enumerate(phis):
        q = store.get(i)
        assert tuple(q.shape) == SHAPE and q.dtype == torch.float32 and q.device.type == "cuda"
        mean = p[:, :, :1]
        maximum = mean.abs().amax(dim=(2, 3, 4, 5), keepdim=True)
        scale = torch.where(maximum > 0, maximum / 2.0 ** 14, torch.ones_like(maximum))
        expected = (mean / scale).to(torch.float16).float() * scale  # the reference's float32 arithmetic
        assert torch.equal(q[:, :, :1], expected)
        assert float((q[:, :, 0] - p[:, :, 0]).norm() / p[:, :, 0].norm()) < 2e-4
        assert float(q[:, :, 1:].abs().max()) == 0.0
    assert store.bytes_per_view < int(np.prod(SHAPE)) * 4 / 7.5
    if location == "cpu":
        assert store._data[0].is_pinned() and store._data[0].device.type == "cpu"
    with pytest.raises(ValueError):
        store.put(0, phis[0][:, :9])
    store.close()
    assert store.get(1) is None


@pytest.mark.gpu
@pytest.mark.parametrize("location", ["gpu", "cpu"])
def test_codec_matches_the_reference_store(cuda_device, location):
    """The reference's own StateStore output (fixture): a seeded accumulator with a NaN cell in one (group, moment)
    plane and one all-zero plane. Stored float16 values, scales and the decoded accumulator bit for bit (NaN where
    the reference has NaN; the NaN plane takes the scale 1, as the reference's ``amax > 0`` test gives)."""
    g = golden("state_store_codec")
    shape = tuple(g["phi"].shape)
    storage = torch.as_tensor(g["phi"]).permute(1, 3, 4, 5, 0, 2).contiguous().to(cuda_device)
    phi = storage.permute(4, 0, 5, 1, 2, 3)                    # the sweep's cell-major storage, reference shape
    store = StateStore(1, shape, cuda_device, location=location)
    store.put(0, phi)
    np.testing.assert_array_equal(store._scale[0].cpu().numpy(), g["scale"])
    np.testing.assert_array_equal(store._data[0].float().cpu().numpy(), g["stored"])
    np.testing.assert_array_equal(store.get(0).cpu().numpy(), g["decoded"])
    assert float(g["scale"][1, 2].item()) == 1.0 and float(g["scale"][2, 5].item()) == 1.0
