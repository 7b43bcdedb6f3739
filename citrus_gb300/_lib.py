"""ctypes binding of the C-ABI library ``libcitrus_gb300.so`` (declared in ``include/citrus_gb300.h``).

The library is loaded on first use from ``citrus_gb300/_lib``; a missing library or a failed call raises
``CitrusKernelError`` — there is no fallback path. Device tensors are passed as raw pointers, sizes as int64 and the
stream as the current torch stream's handle.
"""

from __future__ import annotations

import ctypes
from typing import Optional

import torch

from .build import LIBRARY_PATH

P = ctypes.c_void_p
I64 = ctypes.c_int64
I32 = ctypes.c_int32
F32 = ctypes.c_float
F64 = ctypes.c_double

# name -> argument types (every entry point returns int status)
SIGNATURES = {
    "citrus_abi_version": [],
    "citrus_launch_count": [],
    "citrus_sweep_planes": [P, P, P, P, P, P, P, I64, I64, I64, I64, I64, P],
    "citrus_sweep_persistent": [P, P, P, P, P, P, P, I64, I64, I64, I64, I64, P, I64, I64, I64, P],
    "citrus_sweep_persistent_config": [P, P, P, P, P, P, P, I64, I64, I64, I64, I64, P, I64, I32, I64, I64, P],
    "citrus_sweep_persistent_static": [P, P, P, P, P, P, P, I64, I64, I64, I64, I64, P, I64, P],
    "citrus_sweep_tiled": [P, P, P, P, P, P, P, P, I64, I64, I64, I64, I64, I64, I64, P, I64, I64, I64, I64, P],
    "citrus_small_k_gemm": [P, I64, P, I64, P, I64, I64, I64, I64, I64, I64, I64, I32, P],
    "citrus_small_k_gemm_config": [P, I64, P, I64, P, I64, I64, I64, I64, I64, I64, I64, I32, I32, I32, P],
    "citrus_source_expansion_first": [P, I64, P, I64, P, I64, P, I64, I64, I64, I64, I64, I64, I64, I64, P],
    "citrus_small_k_gemm_bf16x3": [P, I64, P, I64, P, I64, I64, I64, I64, I64, I64, I64, I32, P, P],
    "citrus_source_expansion_first_bf16x3": [P, I64, P, I64, P, I64, P, I64, I64, I64, I64, I64, I64, I64, I64, P, P],
    "citrus_state_encode": [P, I64, I64, I64, I64, I64, I64, P, P, P],
    "citrus_state_decode": [P, P, I64, I64, I64, P, I64, I64, I64, I64, P],
    "citrus_attenuation_to_density": [P, I64, P, P, P, I64, I64, P, P],
    "citrus_scattering_moments": [P, P, P] + [I64] * 14 + [P],
    "citrus_line_integrals": [P, I64, P, P, P, P, I64, P, P],
    "citrus_trace_from_source": [P, I64, P, P, P, P, P, P, P, P, I64, P, P],
    "citrus_downstream_cumulative": [P, I64, P, P, P, P, I64, P, F64, P, I64, I64, I64, P, I64, P],
    "citrus_crossing_tables": [P, P, P, I64, P, I64, P],
    "citrus_downstream_cumulative_tables": [P, I64, P, P, P, P, I64, P, F64, P, I64, I64, I64, P, I64, P],
    "citrus_oblique_project": [P, I64, I64, P, P, P, I64, P, I64, I64, P, I64, I64, I64, I64, P],
    "citrus_oblique_project_scratch": [P, I64, I64, P, P, P, I64, P, I64, I64, P, I64, I64, I64, I64, P, I64, P],
    "citrus_group_transmission": [P, I64, I64, P, P, P, I64, I64, P, P, P, P, P],
    "citrus_source_weight": [P, P, P, P, P, P, I64, I32, P, P],
    "citrus_source_field": [P, P, P, P, I64, F64, P, P, I64, P, P, P, P, P, I64, I32, P, P, P],
    "citrus_first_collision_source": [P, I64, P, I64, P, P, P, P, I64, F64, F64, P, I64, P, P],
    "citrus_first_collision_moments": [P, I64, P, I64, P, P, I64, P, P, I64, F64, F64, P, I64, P, P, P, P, P, I64,
                                       P],
    "citrus_first_collision_correction": [P, I64, P, I64, P, P, P, P, I64, F64, F64, P, P, I64, P, P, P, P, P, P],
    "citrus_first_collision_means": [I64, P, P, P, P, I64, P, P, P, P, P, I64, P],
    "citrus_attenuated_emission": [P, I64, P, I64, P, P, I64, P, P, P, I64, F64, F64, P, I64, P, P, I64, P, P, P, P,
                                   P, P, I64, P, P],
    "citrus_attenuated_emission_moments": [P, I64, P, I64, P, P, I64, P, P, P, I64, F64, F64, P, I64, P, P, I64, P, P,
                                           P, I64, P, P, P, P, I64, P, P],
    "citrus_box_blur": [P, P, I64, I64, I64, I64, I64, I64, I64, I64, I64, P, P, P, I32, F64, F64, P],
    "citrus_box_matrix": [P, I64, I64, P, P],
    "citrus_weighted_group_sum": [P, P, I64, I64, I64, I64, I64, P, P],
    "citrus_sum_directions": [P, I64, I64, I64, P, I32, P],
    "citrus_weighted_direction_sum": [P, I64, I64, I64, I64, I64, I64, I64, I64, P, I64, I64, P, I32, P],
    "citrus_grid_signal_sum": [P, I64, I64, I64, I64, I64, I64, I64, I64, P, I64, P, I64, P, P, P, P, P, P, P, P, I32, I32, P],
    "citrus_conv3d_forward": [P, I64, P, I64, I32, P, P, P, I64, I64, I64, I64, I64, I32, I32, P],
    "citrus_conv3d_backward_input": [P, I64, P, P, I64, P, P, I64, I64, I64, I64, I64, I32, P],
    "citrus_conv3d_forward_config": [P, I64, P, I64, I32, P, P, P, I64, I64, I64, I64, I64, I32, I32, I32, P, P],
    "citrus_conv3d_backward_input_config": [P, I64, P, P, I64, P, P, I64, I64, I64, I64, I64, I32, I32, P, P],
    "citrus_conv3d_weight_grad_splits": [I64, I64, I64, I64, I64, I64, I64, I32],
    "citrus_oblique_scratch_bytes": [I64],
    "citrus_conv3d_backward_weight": [P, I64, P, I64, P, I64, I32, P, P, I64, I64, I64, I64, I32, P, I64, P],
    "citrus_avg_pool2": [P, P, I64, I64, I64, I64, P],
    "citrus_avg_pool2_backward": [P, P, P, I32, I64, I64, I64, I64, P],
    "citrus_upsample2_backward": [P, P, P, I64, I64, I64, I64, P],
    "citrus_mse": [P, P, I64, P, P, I64, P],
    "citrus_adam": [P, P, P, P, P, I64, F64, F64, F64, F64, I64, P],
    "citrus_to_bf16": [P, P, I64, P],
}

_LIBRARY: Optional[ctypes.CDLL] = None


class CitrusKernelError(RuntimeError):
    """A citrus_gb300 entry point returned a non-zero status, or the library is unavailable."""


def library() -> ctypes.CDLL:
    """The loaded C-ABI library with its argument types declared (loaded once per process)."""
    global _LIBRARY
    if _LIBRARY is None:
        if not LIBRARY_PATH.exists():
            raise CitrusKernelError(f"{LIBRARY_PATH} is not built; run `python -m citrus_gb300.build` (or "
                                    f"__graft_entry__.build()) on this machine first")
        lib = ctypes.CDLL(str(LIBRARY_PATH))
        for name, argtypes in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.argtypes = argtypes
            fn.restype = ctypes.c_int
        lib.citrus_last_error_string.argtypes = []
        lib.citrus_last_error_string.restype = ctypes.c_char_p
        lib.citrus_launch_count.restype = ctypes.c_int64
        lib.citrus_conv3d_weight_grad_splits.restype = ctypes.c_int64
        lib.citrus_oblique_scratch_bytes.restype = ctypes.c_int64
        _LIBRARY = lib
    return _LIBRARY


_TIMED: Optional[dict] = None


class timed_calls:
    """Context manager that records CUDA events on the current stream around every call of the named entry points:
    ``records[name]`` is a list of (info, start event, end event), info = ``capture[name](args)`` evaluated during the
    call (while host arrays behind address arguments are alive), else None. A measurement aid for the benchmark."""

    def __init__(self, *names: str, capture: Optional[dict] = None):
        self.records = {n: [] for n in names}
        self.capture = dict(capture or {})

    def __enter__(self):
        global _TIMED
        _TIMED = self
        return self.records

    def __exit__(self, *exc):
        global _TIMED
        _TIMED = None


def call(name: str, *args) -> None:
    """Call an entry point and raise ``CitrusKernelError`` with the library's message on a non-zero status."""
    lib = library()
    if _TIMED is not None and name in _TIMED.records:
        stream = torch.cuda.current_stream()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        status = getattr(lib, name)(*args)
        e1.record(stream)
        fn = _TIMED.capture.get(name)
        _TIMED.records[name].append((fn(args) if fn is not None else None, e0, e1))
    else:
        status = getattr(lib, name)(*args)
    if status != 0:
        message = lib.citrus_last_error_string().decode(errors="replace")
        raise CitrusKernelError(f"{name} failed with status {status}: {message}")


def ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    """Device address of a tensor (None for None)."""
    return None if t is None else t.data_ptr()


def upload(a, device, dtype=None) -> torch.Tensor:
    """A host array on ``device`` through pinned memory, queued on the current stream without waiting for it (a copy
    from pageable memory would block until every earlier launch on the stream has finished)."""
    t = torch.as_tensor(a, dtype=dtype)
    if t.device.type != "cpu" or torch.device(device).type != "cuda":
        return t.to(device)
    return t.contiguous().pin_memory().to(device, non_blocking=True)


def stream_handle(device: torch.device) -> int:
    """Raw handle of the current torch stream of ``device``."""
    return torch.cuda.current_stream(device).cuda_stream


def launch_count() -> int:
    """Kernels the library has launched in this process so far."""
    return int(library().citrus_launch_count())
