"""Oracle of the learned higher-order proposal's network: test infrastructure only.

The same 3D U-Net as ``citrus_gb300.learned.ConvNet3D`` (two 3^3 convolutions with ReLU per level, 2x average pooling,
nearest 2x upsampling with the skip connection concatenated first, a 1^3 output convolution), written with
``torch.nn.functional`` on the CPU in float64 and differentiated by autograd. It takes the bfloat16 weights the
kernels compute with, converted exactly to float64, so a comparison isolates the kernels' float32 arithmetic.

The reference has no learned part (its cold start is an empty accumulator, ``citrus/citrus.py:70-87``); this oracle
pins the network's forward values and gradients, not a reference computation.
"""

from __future__ import annotations

import torch
import torch.nn.functional as F


def forward(weights: dict, biases: dict, x: torch.Tensor, levels: int, masks: dict = None) -> torch.Tensor:
    """y [B, out, D, H, W] of x [B, in, D, H, W]; weights/biases by layer name (float64 CPU tensors). ``masks`` (by
    layer name, optional) replaces each ReLU's decision by a given one: the checked kernels' own, so that a
    pre-activation within rounding of zero takes the same side in both computations."""

    def conv(name, h, relu=True):
        w = weights[name]
        y = F.conv3d(h, w, biases[name], padding=w.shape[-1] // 2)
        if not relu:
            return y
        return F.relu(y) if masks is None else y * masks[name].to(y.dtype)

    skips = []
    h = x
    for level in range(levels):
        if level > 0:
            h = F.avg_pool3d(skips[-1], 2)
        h = conv(f"enc{level}b", conv(f"enc{level}a", h))
        skips.append(h)
    top = skips[-1]
    for level in reversed(range(levels - 1)):
        up = F.interpolate(top, scale_factor=2, mode="nearest")
        top = conv(f"dec{level}b", conv(f"dec{level}a", torch.cat([skips[level], up], 1)))
    return conv("out", top, relu=False)


def loss_and_gradients(weights: dict, biases: dict, x: torch.Tensor, target: torch.Tensor, levels: int,
                       masks: dict = None) -> dict:
    """Output, MSE loss and the gradient of every weight and bias, all float64 (``masks`` as in ``forward``)."""
    w = {k: v.detach().double().clone().requires_grad_(True) for k, v in weights.items()}
    b = {k: v.detach().double().clone().requires_grad_(True) for k, v in biases.items()}
    y = forward(w, b, x.double(), levels, masks)
    loss = ((y - target.double()) ** 2).mean()
    loss.backward()
    out = {"y": y.detach(), "loss": float(loss.detach())}
    for k in w:
        out[k + ".weight"] = w[k].grad.detach()
        out[k + ".bias"] = b[k].grad.detach()
    return out
