"""Direction sets and real spherical harmonics of the sweep and of the collapsed-cone image.

Follows ``citrus/scatter_solver/angular_quadrature.py``: the sweep uses a Gauss-Legendre (in cos theta) times
equal-azimuth product set (``:187-225``), the image a cone product set about the inward panel normal with gnomonic
cell widths (``:270-423``), and the real orthonormal harmonics are evaluated by the same normalized recurrences
(``:475-521``) so that the tables agree with the reference to float64 rounding. All tables are built in float64 on the
host and cast once.
"""

from __future__ import annotations

import math
from dataclasses import dataclass, replace
from typing import Optional

import numpy as np
import torch
from torch import Tensor


def octant_of(omega: np.ndarray) -> np.ndarray:
    """Octant code ``(x < 0) * 4 + (y < 0) * 2 + (z < 0)``; a zero component counts as non-negative."""
    neg = (np.asarray(omega) < 0).astype(np.int64)
    return neg[..., 0] * 4 + neg[..., 1] * 2 + neg[..., 2]


@dataclass(frozen=True, eq=False)
class Quadrature:
    """Directions [M, 3], weights [M] in sr, octant codes [M] and optional gnomonic cell widths [M, 2] (float64 numpy)."""

    omega: np.ndarray
    weight: np.ndarray
    octant: np.ndarray
    cell_width: Optional[np.ndarray] = None

    @staticmethod
    def from_directions(omega, weight) -> "Quadrature":
        omega = np.asarray(omega, dtype=np.float64).reshape(-1, 3)
        weight = np.asarray(weight, dtype=np.float64).reshape(-1)
        if weight.shape[0] != omega.shape[0]:
            raise ValueError("weight must have one entry per direction")
        return Quadrature(omega, weight, octant_of(omega))

    @property
    def num_directions(self) -> int:
        return int(self.omega.shape[0])

    @property
    def directions_per_octant(self) -> Optional[int]:
        counts = np.bincount(self.octant, minlength=8)
        return int(counts[0]) if np.all(counts == counts[0]) else None

    def by_octant(self) -> np.ndarray:
        """Stable permutation grouping the directions by octant (reference ``angular_quadrature.py:121-129``)."""
        return np.argsort(self.octant, kind="stable")

    def reordered(self, perm: np.ndarray) -> "Quadrature":
        cw = None if self.cell_width is None else self.cell_width[perm]
        return Quadrature(self.omega[perm], self.weight[perm], self.octant[perm], cw)


def product_quadrature(num_polar: int, num_azimuthal: int) -> Quadrature:
    """Gauss-Legendre x equal-azimuth product set on the sphere, flat index ``i * num_azimuthal + j``."""
    if num_azimuthal < 1 or num_polar < 1:
        raise ValueError("num_polar and num_azimuthal must be >= 1")
    mu, gw = np.polynomial.legendre.leggauss(num_polar)
    step = 2.0 * math.pi / num_azimuthal
    phi = (np.arange(num_azimuthal) + 0.5) * step
    st = np.sqrt(np.clip(1.0 - mu * mu, 0.0, None))
    omega = np.stack([st[:, None] * np.cos(phi)[None, :], st[:, None] * np.sin(phi)[None, :],
                      np.broadcast_to(mu[:, None], (num_polar, num_azimuthal))], axis=-1).reshape(-1, 3)
    weight = np.broadcast_to(gw[:, None] * step, (num_polar, num_azimuthal)).reshape(-1)
    return Quadrature.from_directions(omega, weight)


def _unit(v) -> np.ndarray:
    t = np.asarray(v, dtype=np.float64).reshape(-1)
    return t / np.linalg.norm(t)


def _local_frame(a: np.ndarray) -> tuple:
    """Right-handed frame (e1, e2, a): helper = least-aligned coordinate axis (reference ``:248-267``)."""
    helper = np.zeros(3)
    helper[int(np.argmin(np.abs(a)))] = 1.0
    e1 = helper - (helper @ a) * a
    e1 = e1 / np.linalg.norm(e1)
    return e1, np.cross(a, e1), a


def hemisphere_quadrature(axis, num_polar: int, num_azimuthal: int, max_polar_angle: float = math.pi / 2,
                          tangent_axes=None, subsamples: int = 16) -> Quadrature:
    """Cone product set about ``axis`` with gnomonic cell widths along ``tangent_axes`` (reference ``:309-423``)."""
    if not (0.0 < max_polar_angle <= math.pi):
        raise ValueError("max_polar_angle must be in (0, pi]")
    a = _unit(axis)
    cos_max = math.cos(max_polar_angle)
    nodes, gw = np.polynomial.legendre.leggauss(num_polar)
    half = 0.5 * (1.0 - cos_max)
    cos_t = (cos_max + half * (nodes + 1.0))[::-1]
    polar_w = (gw * half)[::-1]
    step = 2.0 * math.pi / num_azimuthal
    phi = (np.arange(num_azimuthal) + 0.5) * step
    e1, e2, _ = _local_frame(a)
    sin_t = np.sqrt(np.clip(1.0 - cos_t * cos_t, 0.0, None))
    local = ((sin_t[:, None] * np.cos(phi)[None, :])[..., None] * e1
             + (sin_t[:, None] * np.sin(phi)[None, :])[..., None] * e2 + cos_t[:, None, None] * a)
    omega = local.reshape(-1, 3)
    omega = omega / np.linalg.norm(omega, axis=-1, keepdims=True)
    weight = np.broadcast_to(polar_w[:, None] * step, (num_polar, num_azimuthal)).reshape(-1)
    q = Quadrature.from_directions(omega, weight)
    if tangent_axes is None:
        return q
    u = _unit(tangent_axes[0])
    u = u - (u @ a) * a
    u = u / np.linalg.norm(u)
    v = _unit(tangent_axes[1])
    v = v - (v @ a) * a - (v @ u) * u
    v = v / np.linalg.norm(v)
    # cell widths: sqrt(12) x standard deviation of the gnomonic coordinates over an equal-area lattice in each cell
    n = int(subsamples)
    frac = (np.arange(n) + 0.5) / n
    cos_edges = np.concatenate([[1.0], 1.0 - np.cumsum(polar_w)])
    cos_edges[-1] = cos_max
    cs = cos_edges[1:, None] + (cos_edges[:-1] - cos_edges[1:])[:, None] * frac[None, :]
    az = (np.arange(num_azimuthal)[:, None] + frac[None, :]) * step
    ss = np.sqrt(np.clip(1.0 - cs * cs, 0.0, None))
    lateral = np.cos(az)[..., None] * e1 + np.sin(az)[..., None] * e2
    d = ss[:, None, :, None, None] * lateral[None, :, None, :, :] + cs[:, None, :, None, None] * a
    normal = np.clip(d @ a, 1e-6, None)
    alpha, beta = (d @ u) / normal, (d @ v) / normal
    ns = float(n * n)

    def width(x):
        mean = x.sum(axis=(2, 3)) / ns
        var = np.clip((x * x).sum(axis=(2, 3)) / ns - mean * mean, 0.0, None)
        return np.sqrt(12.0 * var).reshape(-1)

    return replace(q, cell_width=np.stack([width(alpha), width(beta)], axis=-1))


def num_spherical_harmonics(L: int) -> int:
    return (L + 1) * (L + 1)


def degree_of_moment(L: int) -> np.ndarray:
    """Degree l of every flat harmonic index ``n = l*l + (k + l)``."""
    return np.concatenate([np.full(2 * l + 1, l, dtype=np.int64) for l in range(L + 1)])


def real_spherical_harmonics(L: int, omega: np.ndarray) -> np.ndarray:
    """Real orthonormal harmonics, polar axis +z, no Condon-Shortley phase, float64 [..., (L+1)^2].

    Normalized associated-Legendre recurrence in z times Re/Im of ``(x + i y)^k`` (reference ``:475-521``).
    """
    if L < 0:
        raise ValueError("L must be >= 0")
    omega = np.asarray(omega, dtype=np.float64)
    x, y, z = omega[..., 0], omega[..., 1], omega[..., 2]
    one = np.ones_like(z)
    Q = [dict() for _ in range(L + 1)]
    qkk = one * (1.0 / math.sqrt(4.0 * math.pi))
    for k in range(L + 1):
        if k > 0:
            qkk = qkk * math.sqrt((2 * k + 1) / (2.0 * k))
        Q[k][k] = qkk
        if k + 1 <= L:
            Q[k][k + 1] = math.sqrt(2 * k + 3) * z * qkk
        for l in range(k + 2, L + 1):
            a = math.sqrt((4.0 * l * l - 1.0) / (l * l - k * k))
            b = math.sqrt(((l - 1) ** 2 - k * k) / (4.0 * (l - 1) ** 2 - 1.0))
            Q[k][l] = a * (z * Q[k][l - 1] - b * Q[k][l - 2])
    C, S = [one], [np.zeros_like(z)]
    for k in range(1, L + 1):
        C.append(x * C[k - 1] - y * S[k - 1])
        S.append(x * S[k - 1] + y * C[k - 1])
    r2 = math.sqrt(2.0)
    cols = []
    for l in range(L + 1):
        for k in range(-l, l + 1):
            if k == 0:
                cols.append(Q[0][l])
            elif k > 0:
                cols.append(r2 * Q[k][l] * C[k])
            else:
                cols.append(r2 * Q[-k][l] * S[-k])
    return np.stack(cols, axis=-1)


@dataclass(frozen=True, eq=False)
class SphericalHarmonicBasis:
    """Y [M, N] and w Y [M, N] on a direction set (float64 numpy), with the degree of each moment."""

    L: int
    Y: np.ndarray
    Y_weighted: np.ndarray
    degree_of_moment: np.ndarray

    @property
    def num_moments(self) -> int:
        return int(self.Y.shape[1])


def spherical_harmonic_basis(L: int, quadrature: Quadrature) -> SphericalHarmonicBasis:
    Y = real_spherical_harmonics(L, quadrature.omega)
    return SphericalHarmonicBasis(L, Y, quadrature.weight[:, None] * Y, degree_of_moment(L))


def to_device(a: np.ndarray, device, dtype=torch.float32) -> Tensor:
    """A host table as a contiguous device tensor; a CUDA copy goes through pinned memory and is queued on the
    current stream without waiting for it (a copy from pageable memory blocks until the stream has drained)."""
    t = torch.tensor(np.ascontiguousarray(a), dtype=dtype)  # torch.tensor keeps a transposed array's strides
    if torch.device(device).type != "cuda":
        return t.to(device)
    return t.pin_memory().to(device, non_blocking=True)
