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
    "citrus_sweep_planes": [P, P, P, P, P, P, P, I64, I64, I64, I64, I64, P],
    "citrus_sweep_persistent": [P, P, P, P, P, P, P, I64, I64, I64, I64, I64, P, I64, I64, I64, P],
    "citrus_sweep_persistent_static": [P, P, P, P, P, P, P, I64, I64, I64, I64, I64, P, I64, P],
    "citrus_small_k_gemm": [P, I64, P, I64, P, I64, I64, I64, I64, I64, I64, I64, I32, P],
    "citrus_scattering_moments": [P, P, P] + [I64] * 14 + [P],
    "citrus_line_integrals": [P, I64, P, P, P, P, I64, P, P],
    "citrus_trace_from_source": [P, I64, P, P, P, P, P, P, P, P, I64, P, P],
    "citrus_downstream_cumulative": [P, I64, P, P, P, P, I64, P, F64, P, P],
    "citrus_oblique_project": [P, I64, I64, P, P, P, I64, P, I64, I64, P, I64, I64, I64, I64, P],
    "citrus_group_transmission": [P, I64, I64, P, P, P, I64, I64, P, P, P, P, P],
    "citrus_source_weight": [P, P, P, P, P, P, I64, I32, P, P],
    "citrus_first_collision_source": [P, I64, P, I64, P, P, P, P, I64, F64, F64, P, I64, P, P],
    "citrus_first_collision_moments": [P, I64, P, I64, P, P, I64, P, P, I64, F64, F64, P, I64, P, P, P, I64, P],
    "citrus_first_collision_correction": [P, I64, P, I64, P, P, P, P, I64, F64, F64, P, P, I64, P, P, P, P, P],
    "citrus_attenuated_emission": [P, I64, P, I64, P, P, I64, P, P, P, I64, F64, F64, P, I64, P, P, P, P, P, P, P,
                                   I64, P, P],
    "citrus_box_blur": [P, P, I64, I64, I64, I64, I64, I64, I64, I64, I64, P, P, P, I32, F64, F64, P],
    "citrus_box_matrix": [P, I64, I64, P, P],
    "citrus_weighted_group_sum": [P, P, I64, I64, I64, I64, I64, P, P],
    "citrus_sum_directions": [P, I64, I64, I64, P, I32, P],
    "citrus_weighted_direction_sum": [P, I64, I64, I64, I64, I64, I64, I64, I64, P, I64, I64, P, I32, P],
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
        _LIBRARY = lib
    return _LIBRARY


def call(name: str, *args) -> None:
    """Call an entry point and raise ``CitrusKernelError`` with the library's message on a non-zero status."""
    lib = library()
    status = getattr(lib, name)(*args)
    if status != 0:
        message = lib.citrus_last_error_string().decode(errors="replace")
        raise CitrusKernelError(f"{name} failed with status {status}: {message}")


def ptr(t: Optional[torch.Tensor]) -> Optional[int]:
    """Device address of a tensor (None for None)."""
    return None if t is None else t.data_ptr()


def stream_handle(device: torch.device) -> int:
    """Raw handle of the current torch stream of ``device``."""
    return torch.cuda.current_stream(device).cuda_stream
