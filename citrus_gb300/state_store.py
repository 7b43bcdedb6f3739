"""Compact storage of one CITRUS accumulator per view (mirrors ``citrus/citrus.py:623-757``, ``StateStore``).

An accumulator ``[G, N, 4, Rc, Cc, Sc]`` is kept as its linear-discontinuous cell mean in scaled float16 with one
float32 scale per (group, moment): about an eighth of its float32 size. Encoding and decoding run as two kernels of
``libcitrus_gb300.so`` (``citrus_state_encode`` / ``citrus_state_decode``), bit-exact with the reference's float32
tensor arithmetic; the encoded slots live on the GPU, or in (pinned) host memory when the total does not fit the GPU
budget.
"""

from __future__ import annotations

import time
from typing import Optional, Sequence

import numpy as np
import torch
from torch import Tensor

from . import _lib


class StateStore:
    """Per-view accumulators as scaled float16 cell means (reference ``citrus.py:623-757``).

    Args:
        num_slots: number of stored accumulators (views).
        full_shape: accumulator shape ``[G, N, 4, Rc, Cc, Sc]``.
        device: device of the accumulators passed to ``put`` and returned by ``get``.
        location: ``"gpu"``, ``"cpu"`` (host memory) or ``"auto"`` (the GPU when the total fits ``gpu_budget_mib``
            on a CUDA device).
        gpu_budget_mib: largest total in MiB kept on the GPU by ``"auto"``.
        pinned_memory_limit_gib: largest total in GiB stored in pinned host memory.
    """

    def __init__(self, num_slots: int, full_shape: Sequence[int], device, location: str = "auto",
                 gpu_budget_mib: float = 2600.0, pinned_memory_limit_gib: float = 8.0) -> None:
        self.num_slots = int(num_slots)
        self.full_shape = tuple(int(n) for n in full_shape)
        if len(self.full_shape) != 6 or self.full_shape[2] != 4:
            raise ValueError(f"accumulator shape must be [G, N, 4, Rc, Cc, Sc], got {self.full_shape}")
        self.stored_shape = self.full_shape[:2] + (1,) + self.full_shape[3:]
        self.device = torch.device(device)
        if location == "auto":
            fits = self.total_bytes <= gpu_budget_mib * 2 ** 20
            location = "gpu" if self.device.type == "cuda" and fits else "cpu"
        if location not in ("gpu", "cpu"):
            raise ValueError(f"location must be 'auto', 'gpu' or 'cpu', got {location!r}")
        self.location = location
        self.pinned = (location == "cpu" and self.device.type == "cuda"
                       and self.total_bytes <= pinned_memory_limit_gib * 2 ** 30)
        self._data: list = [None] * self.num_slots
        self._scale: list = [None] * self.num_slots
        self.transfer_seconds = 0.0

    @property
    def cells(self) -> int:
        return int(np.prod(self.full_shape[3:]))

    @property
    def bytes_per_view(self) -> int:
        """Stored bytes of one accumulator, its scales included."""
        G, N = self.full_shape[:2]
        return int(np.prod(self.stored_shape)) * 2 + G * N * 4

    @property
    def total_bytes(self) -> int:
        return self.bytes_per_view * self.num_slots

    def _sync(self) -> None:
        if self.device.type == "cuda":
            torch.cuda.synchronize(self.device)

    def put(self, slot: int, accumulator: Tensor) -> None:
        """Store an accumulator ``[G, N, 4, Rc, Cc, Sc]`` (float32 CUDA, any strides with the cells of the trailing
        axes mergeable) in a slot as its cell mean in scaled float16."""
        if tuple(accumulator.shape) != self.full_shape:
            raise ValueError(f"accumulator must be {self.full_shape}, got {tuple(accumulator.shape)}")
        if accumulator.device.type != "cuda" or accumulator.dtype != torch.float32:
            raise ValueError("accumulator must be a float32 CUDA tensor")
        mean = accumulator.detach()[:, :, 0]                     # [G, N, Rc, Cc, Sc] view
        s_x = _cell_stride(mean)
        if s_x is None:
            mean = mean.contiguous()
            s_x = 1
        G, N = self.full_shape[:2]
        self._sync()
        t0 = time.perf_counter()
        data = torch.empty(self.stored_shape, dtype=torch.float16, device=accumulator.device)
        scale = torch.empty(G, N, 1, 1, 1, 1, dtype=torch.float32, device=accumulator.device)
        _lib.call("citrus_state_encode", mean.data_ptr(), G, N, self.cells, mean.stride(0), mean.stride(1), s_x,
                  data.data_ptr(), scale.data_ptr(), _lib.stream_handle(accumulator.device))
        if self.location == "gpu":
            self._data[slot], self._scale[slot] = data, scale
        else:
            buffer = self._data[slot]
            if buffer is None:
                buffer = torch.empty(self.stored_shape, dtype=torch.float16, pin_memory=self.pinned)
                self._data[slot] = buffer
            buffer.copy_(data)
            self._scale[slot] = scale.cpu()
        self._sync()
        self.transfer_seconds += time.perf_counter() - t0

    def get(self, slot: int) -> Optional[Tensor]:
        """The decoded accumulator of a slot (float32, zero slopes, in the sweep's cell-major storage), or None
        before its first ``put``."""
        if self._data[slot] is None:
            return None
        G, N = self.full_shape[:2]
        spatial = self.full_shape[3:]
        self._sync()
        t0 = time.perf_counter()
        data = self._data[slot].to(self.device, non_blocking=self.pinned)
        scale = self._scale[slot].to(self.device)
        storage = torch.empty((N,) + spatial + (G, 4), device=self.device, dtype=torch.float32)
        out = storage.permute(4, 0, 5, 1, 2, 3)                  # [G, N, 4, Rc, Cc, Sc]
        _lib.call("citrus_state_decode", data.data_ptr(), scale.data_ptr(), G, N, self.cells, out.data_ptr(),
                  out.stride(0), out.stride(1), out.stride(2), 4 * G, _lib.stream_handle(self.device))
        self._sync()
        self.transfer_seconds += time.perf_counter() - t0
        return out

    def close(self) -> None:
        self._data = [None] * self.num_slots
        self._scale = [None] * self.num_slots

    def describe(self) -> dict:
        return {"location": self.location, "pinned": self.pinned, "stored_shape": list(self.stored_shape),
                "full_shape": list(self.full_shape), "bytes_per_view": self.bytes_per_view,
                "num_views": self.num_slots, "total_gib": self.total_bytes / 2 ** 30}


def _cell_stride(t: Tensor) -> Optional[int]:
    """Element stride of the merged trailing three axes of ``t`` (None if they do not merge)."""
    sizes, strides = t.shape[-3:], t.stride()[-3:]
    if strides[1] == strides[2] * sizes[2] and strides[0] == strides[1] * sizes[1]:
        return strides[2]
    return None
