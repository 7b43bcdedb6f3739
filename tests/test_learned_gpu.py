"""The learned proposal's network kernels on sm_103a against the float64 autograd oracle (``oracle/learned.py``):
single convolutions (3^3 and 1^3, the fused concatenation and upsampling, ReLU, ragged sizes), their input and weight
gradients, the whole U-Net's output, loss and every gradient, and the Adam step.

Tolerances: the kernels accumulate in float32 over at most C_in * 27 products per output and B * D * H * W per weight
gradient, so the tests ask for a relative error (max |a - b| / max |b|) of 1e-5 on outputs and 1e-4 on gradients of the
SIMT kernels. The tensor-core form multiplies the exact bfloat16 weights by a bfloat16 high + low split of each
input, which keeps the input to 2^-17 relative: 5e-5 on outputs and 3e-4 on gradients."""

from __future__ import annotations

import numpy as np
import pytest
import torch
import torch.nn.functional as F

from conftest import rel_err
from citrus_gb300 import _lib
from citrus_gb300.learned import Adam, ConvNet3D, mse
from oracle import learned as oracle

pytestmark = pytest.mark.gpu
OUT_TOL = {0: 5e-5, 1: 1e-5, 2: 5e-5}     # by convolution kernel: 0 autotuned, 1 SIMT, 2 tensor cores
GRAD_TOL = {0: 3e-4, 1: 1e-4, 2: 3e-4}


def _bf16(w: torch.Tensor, device) -> tuple:
    """(int16 bit patterns on the device, float64 CPU values) of the bfloat16 rounding of w."""
    b = w.to(torch.bfloat16)
    return b.view(torch.int16).to(device).contiguous(), b.double()


@pytest.mark.parametrize("variant", [1, 2])   # the FP32 SIMT kernel, the tcgen05 implicit GEMM
@pytest.mark.parametrize("k,ca,cb,up,co,shape,relu", [
    (3, 5, 0, False, 7, (6, 10, 12), True),
    (3, 3, 6, True, 18, (8, 8, 16), True),
    (3, 16, 16, True, 16, (4, 8, 8), False),
    (1, 33, 0, False, 5, (6, 9, 11), False),
    (3, 40, 0, False, 272, (2, 4, 6), True),      # two output-channel tiles, a voxel tile with few voxels
    (3, 24, 0, False, 192, (4, 4, 4), True),      # N = 192
    (3, 256, 0, False, 128, (2, 2, 2), True),     # the input gradient with N = 256
    (3, 64, 128, True, 64, (4, 4, 4), True),      # the input gradient split 64 + 128 (N = 192)
    (3, 128, 256, True, 128, (2, 2, 2), True),    # the input gradient over two tiles of 192
])
def test_conv_forward_and_gradients(cuda_device, variant, k, ca, cb, up, co, shape, relu):
    gen = torch.Generator().manual_seed(1)
    B = 2
    D, H, W = shape
    a = torch.randn(B, ca, D, H, W, generator=gen)
    bshape = (B, cb, D // 2, H // 2, W // 2) if up else (B, cb, D, H, W)
    b = torch.randn(*bshape, generator=gen) if cb else None
    w = torch.randn(co, ca + cb, k, k, k, generator=gen) / np.sqrt((ca + cb) * k ** 3)
    bias = torch.randn(co, generator=gen) * 0.1
    w_dev, w64 = _bf16(w, cuda_device)
    # device copies held for the whole test (a temporary's memory could be handed to the next allocation)
    a_d, bias_d = a.to(cuda_device).contiguous(), bias.to(cuda_device).contiguous()
    b_d = None if b is None else b.to(cuda_device).contiguous()
    out = torch.empty(B, co, D, H, W, device=cuda_device)
    stream = _lib.stream_handle(cuda_device)
    err = torch.zeros(1, dtype=torch.int32, device=cuda_device)
    _lib.call("citrus_conv3d_forward_config", a_d.data_ptr(), ca, _lib.ptr(b_d), cb, int(up), w_dev.data_ptr(),
              bias_d.data_ptr(), out.data_ptr(), co, B, D, H, W, k, int(relu), variant, err.data_ptr(), stream)

    a64 = a.double().requires_grad_(True)
    b64 = None if b is None else b.double().requires_grad_(True)
    w64 = w64.clone().requires_grad_(True)
    bias64 = bias.double().requires_grad_(True)
    parts = [a64]
    if b64 is not None:
        parts.append(F.interpolate(b64, scale_factor=2, mode="nearest") if up else b64)
    ref = F.conv3d(torch.cat(parts, 1), w64, bias64, padding=k // 2)
    if relu:
        ref = F.relu(ref)
    assert rel_err(out, ref) < OUT_TOL[variant]

    # gradients against an arbitrary upstream gradient; the A-part input gradient masked by a ReLU activation
    g = torch.randn(B, co, D, H, W, generator=gen)
    mask = torch.relu(torch.randn(B, ca, D, H, W, generator=gen))
    ref.backward(g.double())
    g_d, mask_d = g.to(cuda_device).contiguous(), mask.to(cuda_device).contiguous()
    ga = torch.empty(B, ca, D, H, W, device=cuda_device)
    gb = torch.empty(B, cb, D, H, W, device=cuda_device) if cb else None
    _lib.call("citrus_conv3d_backward_input_config", g_d.data_ptr(), co, w_dev.data_ptr(), ga.data_ptr(), ca,
              mask_d.data_ptr(), _lib.ptr(gb), cb, B, D, H, W, k, variant, err.data_ptr(), stream)
    # the kernel's input gradient is taken through the ReLU's output gradient, i.e. with respect to the
    # pre-activation input: compare against autograd of the linear convolution
    a_lin = a.double().requires_grad_(True)
    b_lin = None if b is None else b.double().requires_grad_(True)
    u_lin = None
    parts = [a_lin]
    if b_lin is not None:
        u_lin = (F.interpolate(b_lin, scale_factor=2, mode="nearest") if up else b_lin)
        u_lin.retain_grad()
        parts.append(u_lin)
    lin = F.conv3d(torch.cat(parts, 1), w64.detach(), None, padding=k // 2)
    lin.backward(g.double())
    assert rel_err(ga, a_lin.grad * (mask.double() > 0)) < OUT_TOL[variant]
    if cb:
        assert rel_err(gb, u_lin.grad) < OUT_TOL[variant]
        if up:
            coarse = torch.empty(*bshape, device=cuda_device)
            _lib.call("citrus_upsample2_backward", gb.data_ptr(), None, coarse.data_ptr(), B * cb, D // 2, H // 2,
                      W // 2, stream)
            assert rel_err(coarse, b_lin.grad) < OUT_TOL[variant]

    # weight gradients from the gradient of the pre-activation output (the ReLU's mask applied)
    g_pre = g.double() * (ref.detach() > 0) if relu else g.double()
    g_pre_d = g_pre.float().to(cuda_device).contiguous()
    assert int(err) == 0
    gw = torch.empty(co, ca + cb, k, k, k, device=cuda_device)
    gbias = torch.empty(co, device=cuda_device)
    lib = _lib.library()
    splits = int(lib.citrus_conv3d_weight_grad_splits(co, ca, cb, B, D, H, W, k))
    partial = torch.empty(max(1, splits) * gw.numel(), device=cuda_device)
    _lib.call("citrus_conv3d_backward_weight", g_pre_d.data_ptr(), co, a_d.data_ptr(), ca, _lib.ptr(b_d), cb,
              int(up), gw.data_ptr(), gbias.data_ptr(), B, D, H, W, k, partial.data_ptr(), partial.numel(), stream)
    w_req = w64.detach().clone().requires_grad_(True)
    x_cat = torch.cat([a.double()] + ([F.interpolate(b.double(), scale_factor=2, mode="nearest") if up
                                       else b.double()] if cb else []), 1)
    (gw_ref,) = torch.autograd.grad(F.conv3d(x_cat, w_req, None, padding=k // 2), [w_req], g_pre)
    assert rel_err(gw, gw_ref) < 1e-4
    assert rel_err(gbias, g_pre.sum(dim=(0, 2, 3, 4))) < 1e-4
    # the same gradient without the partial-sum workspace (one split)
    gw1 = torch.empty_like(gw)
    _lib.call("citrus_conv3d_backward_weight", g_pre_d.data_ptr(), co, a_d.data_ptr(), ca, _lib.ptr(b_d), cb,
              int(up), gw1.data_ptr(), None, B, D, H, W, k, None, 0, stream)
    assert rel_err(gw1, gw_ref) < 1e-4


def test_pooling_and_its_gradient(cuda_device):
    gen = torch.Generator().manual_seed(2)
    x = torch.randn(3, 4, 6, 8, 10, generator=gen)
    out = torch.empty(3, 4, 3, 4, 5, device=cuda_device)
    stream = _lib.stream_handle(cuda_device)
    xd = x.to(cuda_device)
    _lib.call("citrus_avg_pool2", xd.data_ptr(), out.data_ptr(), 12, 6, 8, 10, stream)
    assert rel_err(out, F.avg_pool3d(x.double(), 2)) < 1e-6
    g = torch.randn(3, 4, 3, 4, 5, generator=gen)
    prior = torch.randn(3, 4, 6, 8, 10, generator=gen)
    mask = torch.relu(torch.randn(3, 4, 6, 8, 10, generator=gen))
    gin, g_d, mask_d = prior.to(cuda_device), g.to(cuda_device), mask.to(cuda_device)
    _lib.call("citrus_avg_pool2_backward", g_d.data_ptr(), gin.data_ptr(), mask_d.data_ptr(), 1, 12, 6, 8, 10,
              stream)
    x64 = x.double().requires_grad_(True)
    F.avg_pool3d(x64, 2).backward(g.double())
    assert rel_err(gin, (prior.double() + x64.grad) * (mask > 0)) < 1e-6


def _net_and_oracle(cuda_device, channels, shape, B, seed, variant=0):
    net = ConvNet3D(5, 3, channels, seed=seed, device=cuda_device)
    net.variant = variant
    # non-zero biases so that every bias path is exercised
    gen = torch.Generator().manual_seed(seed + 10)
    for layer in net.layers.values():
        layer.bias.copy_(torch.randn(layer.c_out, generator=gen) * 0.05)
    x = torch.randn(B, 5, *shape, generator=gen)
    t = torch.randn(B, 3, *shape, generator=gen)
    w = {n: v.double().cpu() for n, v in net.bf16_weights().items()}
    b = {n: layer.bias.double().cpu() for n, layer in net.layers.items()}
    return net, x, t, oracle.loss_and_gradients(w, b, x, t, net.levels)


@pytest.mark.parametrize("variant", [0, 1, 2])   # autotuned per layer, all SIMT, all tensor cores
@pytest.mark.parametrize("channels,shape,B", [((4, 8, 8, 16), (16, 16, 8), 2), ((32, 64, 128, 256), (8, 8, 8), 1),
                                              ((6, 10), (6, 8, 4), 3)])
def test_unet_output_loss_and_gradients(cuda_device, channels, shape, B, variant):
    net, x, t, ref = _net_and_oracle(cuda_device, channels, shape, B, seed=3, variant=variant)
    y = net.forward(x.to(cuda_device).contiguous(), keep=True)
    assert rel_err(y, ref["y"]) < OUT_TOL[variant]
    if variant != 1:
        # the tensor-core form keeps inputs to 2^-17: a pre-activation that close to zero may take the other side of
        # its ReLU than in float64, which moves whole gradient terms; the oracle then takes the kernels' decisions
        acts = net._cache
        masks = {}
        for level in range(net.levels):
            masks[f"enc{level}a"], masks[f"enc{level}b"] = acts[f"a{level}"] > 0, acts[f"e{level}"] > 0
        for level in range(net.levels - 1):
            masks[f"dec{level}a"], masks[f"dec{level}b"] = acts[f"b{level}"] > 0, acts[f"d{level}"] > 0
        ref = oracle.loss_and_gradients({n: v.double().cpu() for n, v in net.bf16_weights().items()},
                                        {n: layer.bias.double().cpu() for n, layer in net.layers.items()}, x, t,
                                        net.levels, {n: m.cpu() for n, m in masks.items()})
        assert rel_err(y, ref["y"]) < OUT_TOL[variant]
    loss, grad = mse(y, t.to(cuda_device).contiguous())
    assert abs(float(loss) - ref["loss"]) <= OUT_TOL[variant] * ref["loss"]
    net.backward(grad)
    net.check_errors()
    grads = net.gradients()
    for name, g in grads.items():
        assert rel_err(g, ref[name]) < GRAD_TOL[variant], name


def test_adam_step_and_training(cuda_device):
    gen = torch.Generator().manual_seed(4)
    n = 1000
    p = torch.randn(n, generator=gen)
    g = torch.randn(n, generator=gen)
    pd, gd = p.to(cuda_device), g.to(cuda_device)
    m, v = torch.zeros(n, device=cuda_device), torch.zeros(n, device=cuda_device)
    bits = torch.empty(n, dtype=torch.int16, device=cuda_device)
    stream = _lib.stream_handle(cuda_device)
    p64, m64, v64 = p.double(), torch.zeros(n, dtype=torch.float64), torch.zeros(n, dtype=torch.float64)
    for step in (1, 2, 3):
        _lib.call("citrus_adam", pd.data_ptr(), gd.data_ptr(), m.data_ptr(), v.data_ptr(), bits.data_ptr(), n, 1e-2,
                  0.9, 0.999, 1e-8, step, stream)
        m64 = 0.9 * m64 + 0.1 * g.double()
        v64 = 0.999 * v64 + 0.001 * g.double() ** 2
        p64 = p64 - 1e-2 * (m64 / (1 - 0.9 ** step)) / ((v64 / (1 - 0.999 ** step)).sqrt() + 1e-8)
    assert rel_err(pd, p64) < 1e-5
    assert torch.equal(bits.view(torch.bfloat16).float(), pd.to(torch.bfloat16).float())

    # a few Adam steps on a fixed batch lower the loss of a small net
    net = ConvNet3D(2, 1, (4, 8), seed=0, device=cuda_device)
    x = torch.randn(2, 2, 8, 8, 8, generator=gen).to(cuda_device)
    target = (0.5 * x[:, :1] + 0.25 * x[:, 1:]).contiguous()
    opt = Adam(net, lr=3e-3)
    losses = []
    for _ in range(30):
        y = net.forward(x, keep=True)
        loss, grad = mse(y, target)
        net.backward(grad)
        opt.step()
        losses.append(float(loss))
    assert losses[-1] < 0.5 * losses[0]
