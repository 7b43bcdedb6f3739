"""Learned higher-order proposal of the CITRUS accumulator.

The accumulator of a view converges to the collided fluence Phi = phi^(1) + K Phi, where phi^(1) is the first-collided
fluence (one sweep of the first-collision source) and K the scatter-and-sweep operator. A cold start
(``CitrusState()``, reference ``citrus.py:70-87`` and ``:192-247``) begins from Phi = 0, so the first outer iterations
project a scatter image that lacks most of the higher collision orders. This module proposes them: a 3D U-Net
(:class:`ConvNet3D`) maps the transport cells' densities and the first-collided scalar flux to the scalar flux of the
higher orders, Phi_{>1} = Phi - phi^(1); the proposal Phi_0 = phi^(1) + Phi_{>1} replaces the cold start.

The network's training and inference run on the kernels of ``libcitrus_gb300.so`` (``citrus_conv3d_forward``,
``citrus_conv3d_backward_input``, ``citrus_conv3d_backward_weight``, pooling, upsampling, MSE and Adam entry points):
bfloat16 convolution weights with float32 master copies, float32 activations and float32 accumulation. The training
triples (densities, phi^(1), Phi_{>1}) come from the solver itself (:func:`generate_training_data`), and the plain
sweep judges every proposal (:func:`learned_view_step`, :func:`judged_sweeps`): the plain source iteration sweeps the
proposal, estimates the SPR error left from how much each sweep moves the scatter-to-primary ratio, accepts the
proposal when at most four sweeps bring that estimate within the tolerance (0.5 %), and otherwise goes on sweeping
as the plain method does.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Optional, Sequence

import numpy as np
import torch
from torch import Tensor

from . import _lib

DEFAULT_CHANNELS = (32, 64, 128, 256)   # 4 levels, 32 base channels


# ---- network -----------------------------------------------------------------------------------------------------

@dataclass
class ConvLayer:
    """One convolution: [A, up(B)] (c_a + c_b channels) -> c_out channels, k^3 taps, optional ReLU."""

    name: str
    c_a: int
    c_b: int
    b_up: bool
    c_out: int
    k: int
    relu: bool
    weight: Tensor = None          # float32 master [c_out, c_a + c_b, k, k, k]
    weight_bf16: Tensor = None     # int16 bit patterns of the bfloat16 weights the kernels read
    bias: Tensor = None            # float32 [c_out]
    grad_weight: Tensor = None
    grad_bias: Tensor = None
    m: tuple = ()
    v: tuple = ()

    @property
    def c_in(self) -> int:
        return self.c_a + self.c_b


def _check_cuda(t: Tensor, name: str) -> None:
    if t.device.type != "cuda" or t.dtype != torch.float32 or not t.is_contiguous():
        raise ValueError(f"{name} must be a contiguous float32 CUDA tensor")


class ConvNet3D:
    """3D U-Net of ``len(channels)`` levels: per level two 3^3 convolutions with ReLU, 2x average pooling down, nearest
    2x upsampling up with the skip connection concatenated, and a 1^3 output convolution. Spatial sizes must be
    divisible by 2^(levels - 1).

    Args:
        in_channels, out_channels: input and output channels.
        channels: channels of each level (default 32, 64, 128, 256).
        seed: seed of the He-normal initial weights (biases start at zero, the output layer at a tenth of He).
        device: CUDA device of the parameters.
    """

    def __init__(self, in_channels: int, out_channels: int, channels: Sequence[int] = DEFAULT_CHANNELS,
                 seed: int = 0, device="cuda") -> None:
        self.in_channels, self.out_channels = int(in_channels), int(out_channels)
        self.channels = tuple(int(c) for c in channels)
        if not self.channels or min(self.channels) < 1 or self.in_channels < 1 or self.out_channels < 1:
            raise ValueError("channel counts must be >= 1")
        self.device = torch.device(device)
        self.levels = len(self.channels)
        c = self.channels
        layers = []
        for level in range(self.levels):
            c_in = self.in_channels if level == 0 else c[level - 1]
            layers.append(ConvLayer(f"enc{level}a", c_in, 0, False, c[level], 3, True))
            layers.append(ConvLayer(f"enc{level}b", c[level], 0, False, c[level], 3, True))
        for level in reversed(range(self.levels - 1)):
            layers.append(ConvLayer(f"dec{level}a", c[level], c[level + 1], True, c[level], 3, True))
            layers.append(ConvLayer(f"dec{level}b", c[level], 0, False, c[level], 3, True))
        layers.append(ConvLayer("out", c[0], 0, False, self.out_channels, 1, False))
        self.layers = {layer.name: layer for layer in layers}
        rng = np.random.default_rng(seed)
        for layer in layers:
            fan_in = layer.c_in * layer.k ** 3
            std = math.sqrt(2.0 / fan_in) * (0.1 if layer.name == "out" else 1.0)
            w = rng.standard_normal((layer.c_out, layer.c_in, layer.k, layer.k, layer.k)) * std
            layer.weight = torch.as_tensor(w, dtype=torch.float32).to(self.device).contiguous()
            layer.bias = torch.zeros(layer.c_out, dtype=torch.float32, device=self.device)
            layer.weight_bf16 = torch.empty(layer.weight.shape, dtype=torch.int16, device=self.device)
            self._refresh_bf16(layer)
        self._cache: dict = {}
        self.variant = 0          # 0: the autotuner picks each layer's kernel; 1 SIMT; 2 tensor cores
        self._error = torch.zeros(1, dtype=torch.int32, device=self.device)

    # -- parameters --------------------------------------------------------------------------------------------------
    def _refresh_bf16(self, layer: ConvLayer) -> None:
        _lib.call("citrus_to_bf16", layer.weight.data_ptr(), layer.weight_bf16.data_ptr(), layer.weight.numel(),
                  _lib.stream_handle(self.device))

    def num_parameters(self) -> int:
        return sum(layer.weight.numel() + layer.bias.numel() for layer in self.layers.values())

    def state_dict(self) -> dict:
        """float32 master weights and biases (host copies)."""
        out = {}
        for name, layer in self.layers.items():
            out[name + ".weight"] = layer.weight.detach().cpu().clone()
            out[name + ".bias"] = layer.bias.detach().cpu().clone()
        return out

    def load_state_dict(self, state: dict) -> None:
        for name, layer in self.layers.items():
            w, b = state[name + ".weight"], state[name + ".bias"]
            if tuple(w.shape) != tuple(layer.weight.shape) or tuple(b.shape) != tuple(layer.bias.shape):
                raise ValueError(f"layer {name}: shapes {tuple(w.shape)}, {tuple(b.shape)} do not match")
            layer.weight.copy_(w.to(layer.weight))
            layer.bias.copy_(b.to(layer.bias))
            self._refresh_bf16(layer)

    def bf16_weights(self) -> dict:
        """name -> bfloat16 weights (the values the kernels compute with), for checks."""
        return {name: layer.weight_bf16.view(torch.bfloat16) for name, layer in self.layers.items()}

    def check_shape(self, x: Tensor) -> None:
        if x.dim() != 5 or int(x.shape[1]) != self.in_channels:
            raise ValueError(f"input must be [B, {self.in_channels}, D, H, W], got {tuple(x.shape)}")
        step = 2 ** (self.levels - 1)
        if any(int(n) % step for n in x.shape[2:]):
            raise ValueError(f"spatial sizes {tuple(x.shape[2:])} must be divisible by {step}")

    # -- kernels -----------------------------------------------------------------------------------------------------
    def _variant(self, op: str, layer: ConvLayer, shape: tuple, run) -> int:
        """The convolution kernel of this layer and shape: ``self.variant`` when set (1 SIMT, 2 tensor cores), else
        the autotuner's choice between them."""
        if self.variant:
            return self.variant
        from .autotune import Autotuner, tuner

        B, D, H, W = shape
        key = Autotuner.key(op, self.device, B=B, D=D, H=H, W=W, ca=layer.c_a, cb=layer.c_b, co=layer.c_out,
                            k=layer.k, up=int(layer.b_up))
        return int(tuner().choose(key, [2, 1], run, 2))

    def check_errors(self) -> None:
        """Raise if a wait for the tensor cores ran out in any convolution so far (reads a device word)."""
        if int(self._error.item()) != 0:
            self._error.zero_()
            raise _lib.CitrusKernelError("conv3d: a wait for the tensor cores ran out; the results are invalid")

    def _conv(self, layer: ConvLayer, a: Tensor, b: Optional[Tensor] = None) -> Tensor:
        B, _, D, H, W = a.shape
        out = torch.empty((B, layer.c_out, D, H, W), device=self.device, dtype=torch.float32)
        stream = _lib.stream_handle(self.device)

        def run(variant):
            _lib.call("citrus_conv3d_forward_config", a.data_ptr(), layer.c_a, _lib.ptr(b), layer.c_b,
                      int(layer.b_up), layer.weight_bf16.data_ptr(), layer.bias.data_ptr(), out.data_ptr(),
                      layer.c_out, B, D, H, W, layer.k, int(layer.relu), int(variant), self._error.data_ptr(),
                      stream)

        run(self._variant("conv3d_forward", layer, (B, D, H, W), run))
        return out

    def _pool(self, x: Tensor) -> Tensor:
        B, C, D, H, W = x.shape
        out = torch.empty((B, C, D // 2, H // 2, W // 2), device=self.device, dtype=torch.float32)
        _lib.call("citrus_avg_pool2", x.data_ptr(), out.data_ptr(), B * C, D, H, W, _lib.stream_handle(self.device))
        return out

    def _backward_input(self, layer: ConvLayer, g: Tensor, mask_a: Optional[Tensor], want_b: bool) -> tuple:
        B, _, D, H, W = g.shape
        ga = torch.empty((B, layer.c_a, D, H, W), device=self.device, dtype=torch.float32)
        gb = torch.empty((B, layer.c_b, D, H, W), device=self.device, dtype=torch.float32) if want_b else None
        stream = _lib.stream_handle(self.device)

        def run(variant):
            _lib.call("citrus_conv3d_backward_input_config", g.data_ptr(), layer.c_out, layer.weight_bf16.data_ptr(),
                      ga.data_ptr(), layer.c_a, _lib.ptr(mask_a), _lib.ptr(gb), layer.c_b if want_b else 0, B, D, H,
                      W, layer.k, int(variant), self._error.data_ptr(), stream)

        run(self._variant("conv3d_backward_input" + ("_b" if want_b else ""), layer, (B, D, H, W), run))
        return ga, gb

    def _backward_weight(self, layer: ConvLayer, g: Tensor, a: Tensor, b: Optional[Tensor]) -> None:
        B, _, D, H, W = g.shape
        if layer.grad_weight is None:
            layer.grad_weight = torch.empty_like(layer.weight)
            layer.grad_bias = torch.empty_like(layer.bias)
        lib = _lib.library()
        splits = int(lib.citrus_conv3d_weight_grad_splits(layer.c_out, layer.c_a, layer.c_b, B, D, H, W, layer.k))
        partial = None
        if splits > 1:
            partial = torch.empty(splits * layer.weight.numel(), device=self.device, dtype=torch.float32)
        _lib.call("citrus_conv3d_backward_weight", g.data_ptr(), layer.c_out, a.data_ptr(), layer.c_a, _lib.ptr(b),
                  layer.c_b, int(layer.b_up), layer.grad_weight.data_ptr(), layer.grad_bias.data_ptr(), B, D, H, W,
                  layer.k, _lib.ptr(partial), 0 if partial is None else partial.numel(),
                  _lib.stream_handle(self.device))

    # -- passes ------------------------------------------------------------------------------------------------------
    def forward(self, x: Tensor, keep: bool = False) -> Tensor:
        """[B, out_channels, D, H, W] of x [B, in_channels, D, H, W]; ``keep`` holds the activations for backward."""
        _check_cuda(x, "x")
        self.check_shape(x)
        L = self.levels
        acts = {"x": x}
        h = x
        skips = []
        for level in range(L):
            if level > 0:
                h = self._pool(skips[-1])
                acts[f"p{level}"] = h
            a = self._conv(self.layers[f"enc{level}a"], h)
            e = self._conv(self.layers[f"enc{level}b"], a)
            acts[f"a{level}"], acts[f"e{level}"] = a, e
            skips.append(e)
        top = skips[-1]
        for level in reversed(range(L - 1)):
            bact = self._conv(self.layers[f"dec{level}a"], skips[level], top)
            d = self._conv(self.layers[f"dec{level}b"], bact)
            acts[f"b{level}"], acts[f"d{level}"] = bact, d
            top = d
        acts["top"] = top
        y = self._conv(self.layers["out"], top)
        self._cache = acts if keep else {}
        return y

    def backward(self, grad_y: Tensor) -> None:
        """Gradients of every weight and bias from dL/dy of the last ``forward(keep=True)``."""
        acts = self._cache
        if not acts:
            raise RuntimeError("backward needs a forward(keep=True) first")
        _check_cuda(grad_y, "grad_y")
        L = self.levels
        stream = _lib.stream_handle(self.device)
        top = acts["top"]
        out = self.layers["out"]
        self._backward_weight(out, grad_y, top, None)
        g, _ = self._backward_input(out, grad_y, top, False)             # dL/d(pre-activation of top)
        skip_grads = {}
        for level in range(L - 1):
            coarse = acts[f"d{level + 1}"] if level + 1 < L - 1 else acts[f"e{L - 1}"]
            lb, la = self.layers[f"dec{level}b"], self.layers[f"dec{level}a"]
            self._backward_weight(lb, g, acts[f"b{level}"], None)
            g_b, _ = self._backward_input(lb, g, acts[f"b{level}"], False)
            self._backward_weight(la, g_b, acts[f"e{level}"], coarse)
            g_skip, g_up = self._backward_input(la, g_b, None, True)
            skip_grads[level] = g_skip
            B, C, D, H, W = coarse.shape
            g = torch.empty_like(coarse)
            _lib.call("citrus_upsample2_backward", g_up.data_ptr(), coarse.data_ptr(), g.data_ptr(), B * C, D, H, W,
                      stream)
        for level in reversed(range(L)):
            lb, la = self.layers[f"enc{level}b"], self.layers[f"enc{level}a"]
            self._backward_weight(lb, g, acts[f"a{level}"], None)
            g_a, _ = self._backward_input(lb, g, acts[f"a{level}"], False)
            src = acts["x"] if level == 0 else acts[f"p{level}"]
            self._backward_weight(la, g_a, src, None)
            if level == 0:
                break
            g_p, _ = self._backward_input(la, g_a, None, False)
            g = skip_grads[level - 1]
            e = acts[f"e{level - 1}"]
            B, C, D, H, W = e.shape
            _lib.call("citrus_avg_pool2_backward", g_p.data_ptr(), g.data_ptr(), e.data_ptr(), 1, B * C, D, H, W,
                      stream)

    def gradients(self) -> dict:
        out = {}
        for name, layer in self.layers.items():
            out[name + ".weight"] = layer.grad_weight
            out[name + ".bias"] = layer.grad_bias
        return out


def mse(pred: Tensor, target: Tensor) -> tuple:
    """(loss, dL/dpred) of the mean squared error; the loss is summed in float64 on the host from per-block sums."""
    _check_cuda(pred, "pred")
    _check_cuda(target, "target")
    if pred.shape != target.shape:
        raise ValueError(f"pred {tuple(pred.shape)} and target {tuple(target.shape)} differ")
    n = pred.numel()
    grad = torch.empty_like(pred)
    partial = torch.empty((n + 255) // 256, device=pred.device, dtype=torch.float32)
    _lib.call("citrus_mse", pred.data_ptr(), target.data_ptr(), n, grad.data_ptr(), partial.data_ptr(),
              partial.numel(), _lib.stream_handle(pred.device))
    return partial.double().sum() / n, grad


class Adam:
    """Adam on the float32 master weights of a :class:`ConvNet3D`; every step refreshes the bfloat16 copies."""

    def __init__(self, net: ConvNet3D, lr: float = 1e-3, betas=(0.9, 0.999), eps: float = 1e-8) -> None:
        self.net, self.lr, self.betas, self.eps = net, float(lr), tuple(betas), float(eps)
        self.step_count = 0
        for layer in net.layers.values():
            layer.m = (torch.zeros_like(layer.weight), torch.zeros_like(layer.bias))
            layer.v = (torch.zeros_like(layer.weight), torch.zeros_like(layer.bias))

    def step(self) -> None:
        self.step_count += 1
        stream = _lib.stream_handle(self.net.device)
        for layer in self.net.layers.values():
            for k, (p, g, bits) in enumerate(((layer.weight, layer.grad_weight, layer.weight_bf16),
                                              (layer.bias, layer.grad_bias, None))):
                _lib.call("citrus_adam", p.data_ptr(), g.data_ptr(), layer.m[k].data_ptr(), layer.v[k].data_ptr(),
                          _lib.ptr(bits), p.numel(), self.lr, self.betas[0], self.betas[1], self.eps,
                          self.step_count, stream)


# ---- the proposal ---------------------------------------------------------------------------------------------------

def scalar_flux(accumulator: Tensor) -> Tensor:
    """[G, Rc, Cc, Sc] cell-mean scalar moment (moment 0, linear-discontinuous component 0) of an accumulator."""
    return accumulator[:, 0, 0]


@dataclass
class ProposalSample:
    """One training triple on the transport cells: densities [M, R, C, S], phi^(1) and Phi_{>1} scalar fluxes [G, ...]."""

    rho: Tensor
    first: Tensor
    higher: Tensor


def features(rho_coarse: Tensor, first: Tensor) -> tuple:
    """Network input [1, M + G, R, C, S] and the flux scale s (mean first-collided scalar flux): densities in g/cc and
    phi^(1) / s. Phi_{>1} is linear in the source, so the network works on fluxes divided by s."""
    s = first.double().mean().clamp_min(1e-30)
    x = torch.cat([rho_coarse.float(), (first.double() / s).float()], 0).unsqueeze(0).contiguous()
    return x, float(s)


class HigherOrderProposal:
    """A trained :class:`ConvNet3D` that proposes Phi_{>1} from (densities, phi^(1)) on the transport cells."""

    def __init__(self, num_materials: int, num_groups: int, channels: Sequence[int] = DEFAULT_CHANNELS,
                 seed: int = 0, device="cuda") -> None:
        self.num_materials, self.num_groups = int(num_materials), int(num_groups)
        self.net = ConvNet3D(self.num_materials + self.num_groups, self.num_groups, channels, seed, device)
        self.history: list = []

    @property
    def device(self) -> torch.device:
        return self.net.device

    def predict(self, rho_coarse: Tensor, first: Tensor) -> Tensor:
        """Phi_{>1} scalar flux [G, R, C, S] of one view."""
        x, s = features(rho_coarse.to(self.device), first.to(self.device))
        y = self.net.forward(x)[0] * s
        self.net.check_errors()
        return y

    def propose(self, rho_coarse: Tensor, first_collided: Tensor) -> Tensor:
        """The proposed accumulator: phi^(1) with Phi_{>1} added to its cell-mean scalar moment."""
        proposal = first_collided.clone()
        scalar_flux(proposal).add_(self.predict(rho_coarse, scalar_flux(first_collided)))
        return proposal

    def fit(self, samples: Sequence[ProposalSample], epochs: int = 100, batch: int = 4, lr: float = 1e-3,
            seed: int = 0, log_every: int = 0) -> list:
        """Train on the triples with Adam and the mean squared error of Phi_{>1} / s; returns the loss per epoch."""
        if not samples:
            raise ValueError("no training samples")
        xs, ys = [], []
        for sample in samples:
            x, s = features(sample.rho.to(self.device), sample.first.to(self.device))
            xs.append(x[0])
            ys.append((sample.higher.to(self.device).double() / s).float())
        X, Y = torch.stack(xs).contiguous(), torch.stack(ys).contiguous()
        opt = Adam(self.net, lr=lr)
        rng = np.random.default_rng(seed)
        n = X.shape[0]
        batch = max(1, min(int(batch), n))
        losses = []
        for epoch in range(int(epochs)):
            order = rng.permutation(n)
            total = torch.zeros((), dtype=torch.float64, device=self.device)
            for i in range(0, n - batch + 1, batch):
                idx = torch.as_tensor(order[i:i + batch], device=self.device)
                xb, yb = X.index_select(0, idx).contiguous(), Y.index_select(0, idx).contiguous()
                pred = self.net.forward(xb, keep=True)
                loss, grad = mse(pred, yb)
                self.net.backward(grad)
                opt.step()
                total += loss
            self.net.check_errors()
            losses.append(float(total) / max(1, n // batch))
            if log_every and (epoch + 1) % log_every == 0:
                print(f"epoch {epoch + 1}: loss {losses[-1]:.4e}")
        self.history.extend(losses)
        return losses

    def relative_error(self, samples: Sequence[ProposalSample]) -> float:
        """||Phi_{>1} proposed - Phi_{>1}|| / ||Phi_{>1}|| over the samples."""
        num = den = 0.0
        for sample in samples:
            pred = self.predict(sample.rho, sample.first).double()
            ref = sample.higher.to(self.device).double()
            num += float(((pred - ref) ** 2).sum())
            den += float((ref ** 2).sum())
        return math.sqrt(num / max(den, 1e-300))


# ---- data from the solver --------------------------------------------------------------------------------------------

def collided_orders(solver, fields, angle: float, tolerance: float = 1e-4, max_sweeps: int = 60) -> tuple:
    """(phi^(1), Phi) of one view: the first-collided accumulator (one sweep of the first-collision source) and the
    converged collided accumulator of the Neumann series Phi = phi^(1) + K phi^(1) + K^2 phi^(1) + ..., stopped when
    a term's scalar flux falls below ``tolerance`` of the sum's (the series of ``accumulator_update_operator``)."""
    ctx = solver.sweep_context(fields.grid_coarse)
    phi_uc = solver.uncollided_fluence(fields, angle)
    first = solver.transport_sweep(fields, solver.first_collision_moment_source(fields, angle, phi_uc, ctx))
    total = first.clone()
    term = first
    for _ in range(int(max_sweeps)):
        term = solver.transport_sweep(fields, solver.scatter_moment_source(fields, term, ctx))
        total.add_(term)
        norms = torch.stack([torch.linalg.vector_norm(scalar_flux(term)), torch.linalg.vector_norm(scalar_flux(total))])
        t, s = norms.tolist()
        if t <= tolerance * s:
            break
    return first, total


def generate_training_data(solver, phantoms: Sequence[Tensor], grid, angles: Sequence[float],
                           tolerance: float = 1e-4) -> list:
    """Training triples of every (phantom, angle): fine densities [M, R, C, S] on ``grid`` per phantom."""
    samples = []
    for rho in phantoms:
        fields = solver.material_fields(torch.as_tensor(rho, dtype=torch.float32, device=solver.device), grid)
        for angle in angles:
            first, total = collided_orders(solver, fields, float(angle), tolerance)
            samples.append(ProposalSample(fields.rho_coarse.clone(), scalar_flux(first).contiguous(),
                                          (scalar_flux(total) - scalar_flux(first)).contiguous()))
    return samples


# ---- the step ------------------------------------------------------------------------------------------------------

@dataclass
class JudgedSweeps:
    """The plain sweep's verdict on a starting accumulator (a proposal, or the cold start phi^(1))."""

    scatter: Tensor            # scatter signal [Rd, Cd] of the last accumulator
    accumulator: Tensor        # the last accumulator
    sweeps: int                # sweeps of the scattering source after the first-collided one
    spr_change: list           # per sweep: max over panel pixels of |SPR change| / SPR
    spr_error_estimate: list   # per sweep from the second on: the remaining SPR error the sweeps' contraction implies
    accepted: bool             # the start met the tolerance within ACCEPT_SWEEPS sweeps


ESTIMATE_MARGIN = 1.0     # stop when the estimated SPR error is within this fraction of the tolerance
ACCEPT_SWEEPS = 4         # a start that meets the tolerance within this many sweeps is accepted
FIRST_ESTIMATE_SWEEP = 3  # the first estimate: after the third sweep (the first ratio of changes is not a contraction)


def judged_sweeps(solver, fields, angle: float, start: Tensor, first: Tensor, phi_uncollided: Tensor,
                  primary: Tensor, cone, tolerance: float = 0.005, max_sweeps: int = 40,
                  margin: float = ESTIMATE_MARGIN) -> JudgedSweeps:
    """Sweep ``start`` with the plain source iteration Phi_{k+1} = phi^(1) + K Phi_k until the remaining SPR error is
    estimated within ``margin * tolerance``.

    A sweep's SPR change c_k is the max over the panel pixels whose primary exceeds 1e-3 of its maximum of
    |S_{k+1} - S_k| / S_{k+1}, each S the full image of its accumulator (the image is not exactly linear in the
    accumulator: the footprint blur's width follows the mean height of the whole emission, so images of accumulator
    changes do not add up to the image of the sum). The iteration contracts by r = c_k / c_{k-1} per sweep, so
    the error left after sweep k is about c_k r / (1 - r) (r capped at 0.95). The first estimate comes after the
    third sweep, from the second and third changes: after a proposal the first sweep's change is mostly the
    correction of the proposal's own error, not the contraction, and a ratio taken against it is far too small
    (estimates of 0.1 % where 1 % was left). Measured on 12 unseen views against solves converged to 1e-6, this rule
    stopped every plain and learned start with its true SPR error within 0.39 % (tolerance 0.5 %)."""
    ctx = solver.sweep_context(fields.grid_coarse)
    context = solver.direction_context(fields, angle, cone)
    mask = primary > 1e-3 * primary.max()
    current = start

    def image(accumulator):
        return solver.scatter_image(fields, angle, phi_uncollided,
                                    solver.multiple_collision_source_moments(fields, accumulator), cone, context,
                                    signal_only=True)["signal"]

    scatter = image(current)
    changes, estimates = [], []
    for _ in range(int(max_sweeps)):
        nxt = solver.transport_sweep(fields, solver.scatter_moment_source(fields, current, ctx)).add_(first)
        following = image(nxt)
        delta = following - scatter
        scatter, current = following, nxt
        rel = delta[mask].abs() / scatter[mask].abs().clamp_min(1e-30)
        changes.append(float(rel.max()) if rel.numel() else 0.0)
        if len(changes) >= FIRST_ESTIMATE_SWEEP:
            r = min(changes[-1] / changes[-2], 0.95) if changes[-2] > 0 else 0.0
            estimates.append(changes[-1] * r / (1.0 - r))
            if estimates[-1] <= margin * tolerance:
                break
    return JudgedSweeps(scatter, current, len(changes), changes, estimates,
                        bool(estimates) and len(changes) <= ACCEPT_SWEEPS and estimates[-1] <= margin * tolerance)


def first_collided(solver, fields, angle: float) -> tuple:
    """(phi_uncollided, phi^(1)) of one view: the uncollided fluence and one sweep of the first-collision source."""
    ctx = solver.sweep_context(fields.grid_coarse)
    phi_uc = solver.uncollided_fluence(fields, angle)
    first = solver.transport_sweep(fields, solver.first_collision_moment_source(fields, angle, phi_uc, ctx))
    return phi_uc, first


def converged_view_step(solver, fields, angle: float, proposal: Optional[HigherOrderProposal] = None, *,
                        tolerance: float = 0.005, max_sweeps: int = 40, primary: Optional[Tensor] = None,
                        cone=None) -> tuple:
    """The scatter signal of one view converged to ``tolerance`` in SPR by plain sweeps, from the learned proposal
    (or, with ``proposal=None``, from the cold start phi^(1)). Returns (JudgedSweeps, primary signal)."""
    cone = solver.cone_quadrature(fields.grid_fine, angle) if cone is None else cone
    p = solver.primary(fields, angle)["signal"] if primary is None else primary
    phi_uc, first = first_collided(solver, fields, angle)
    start = first if proposal is None else proposal.propose(fields.rho_coarse, first)
    return judged_sweeps(solver, fields, angle, start, first, phi_uc, p, cone, tolerance, max_sweeps), p


def learned_view_step(solver, state, fields, angle: float, proposal: HigherOrderProposal, *,
                      tolerance: float = 0.005, max_sweeps: int = 40, primary: Optional[Tensor] = None) -> tuple:
    """One CITRUS scatter step of one view that starts from the learned proposal instead of a cold start.

    A state that already holds an accumulator takes the plain step (``citrus_view_step``). Otherwise phi^(1) is one
    sweep of the first-collision source, the proposal Phi_0 = phi^(1) + Phi_{>1} is swept by the plain source
    iteration, and the plain sweeps judge it (``judged_sweeps``): the proposal is accepted when at most
    ``ACCEPT_SWEEPS`` sweeps bring the estimated SPR error within the margin below ``tolerance``; otherwise the plain
    sweeps go on until they do (at most ``max_sweeps``).
    Returns (scatter signal, primary signal, new state, JudgedSweeps).
    """
    from .citrus_step import CitrusState, citrus_view_step

    if state.collided_moments is not None:
        scatter, p, new = citrus_view_step(solver, state, fields, angle, primary=primary is None)
        p = p if primary is None else primary
        return scatter, p, new, JudgedSweeps(scatter, new.collided_moments, 1, [], [], True)
    cone = state.cone_quadrature if state.cone_quadrature is not None else \
        solver.cone_quadrature(fields.grid_fine, angle)
    judged, p = converged_view_step(solver, fields, angle, proposal, tolerance=tolerance, max_sweeps=max_sweeps,
                                    primary=primary, cone=cone)
    new_state = CitrusState(angle=float(angle), collided_moments=judged.accumulator, cone_quadrature=cone,
                            num_steps=state.num_steps + 1, history=state.history + judged.spr_change)
    return judged.scatter, p, new_state, judged
