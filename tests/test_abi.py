"""The C-ABI library builds for sm_103a, loads, and exports every entry point that ``include/*.h`` declares (no GPU
needed: nothing is launched)."""

from __future__ import annotations

import ctypes
import re
from pathlib import Path

import pytest

from citrus_gb300 import _lib
from citrus_gb300.build import build

ROOT = Path(__file__).resolve().parent.parent


def _declared_functions() -> list:
    names = []
    for header in sorted((ROOT / "include").glob("*.h")):
        text = re.sub(r"/\*.*?\*/", "", header.read_text(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?(?:int64_t|int|char\s*\*|const char\s*\*)\s*\*?\s*(citrus_\w+)\s*\(", text,
                            flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def library():
    build()
    return ctypes.CDLL(str(_lib.LIBRARY_PATH))


def test_header_declares_entry_points():
    names = _declared_functions()
    assert "citrus_abi_version" in names and "citrus_sweep_persistent" in names
    assert len(names) >= 6


def test_library_exports_every_declared_symbol(library):
    missing = [n for n in _declared_functions() if not hasattr(library, n)]
    assert not missing, missing


def test_bindings_cover_the_header():
    declared = set(_declared_functions()) - {"citrus_last_error_string"}
    assert declared == set(_lib.SIGNATURES), declared ^ set(_lib.SIGNATURES)


def test_abi_version_and_error_string(library):
    library.citrus_abi_version.restype = ctypes.c_int
    assert library.citrus_abi_version() == 1
    library.citrus_last_error_string.restype = ctypes.c_char_p
    assert isinstance(library.citrus_last_error_string(), bytes)


def test_bad_arguments_are_rejected_before_any_launch(library):
    """Null pointers and bad sizes return CITRUS_EINVAL with a message; nothing touches a device."""
    lib = _lib.library()
    status = lib.citrus_small_k_gemm(None, 1, None, 4, None, 4, 1, 1, 4, 1, 0, 0, 0, None)
    assert status == 1
    assert b"null" in lib.citrus_last_error_string()
    status = lib.citrus_sweep_planes(None, None, None, None, None, None, None, 1, 1, 1, 1, 1, None)
    assert status == 1


def test_fused_source_entry_points_check_their_arguments(library):
    """The first-collision means and the one-pass source expansion reject null pointers, and the expansion columns
    that do not come in quadruples, with CITRUS_EINVAL before any launch."""
    lib = _lib.library()
    status = lib.citrus_source_expansion_first(None, 1, None, 4, None, 4, None, 1, 1, 1, 4, 1, 0, 0, 0, None)
    assert status == 1 and b"null" in lib.citrus_last_error_string()
    fake = 256  # never dereferenced: the sizes are refused first
    status = lib.citrus_source_expansion_first(fake, 1, fake, 6, fake, 6, fake, 2, 1, 1, 6, 1, 0, 0, 0, None)
    assert status == 1 and b"quadruples" in lib.citrus_last_error_string()
    status = lib.citrus_first_collision_means(8, None, None, None, None, 1, None, None, None, None, None, 8, None)
    assert status == 1 and b"null" in lib.citrus_last_error_string()


def test_allocation_free_sweep_checks_its_arguments(library):
    """citrus_sweep_persistent_static refuses null plane offsets, more planes than its static scratch holds, and a
    non-positive wait limit with CITRUS_EINVAL before any CUDA call (the pointers below are never dereferenced)."""
    import numpy as np
    lib = _lib.library()
    fake = 256
    offsets = np.zeros(9000, dtype=np.int32)
    args = (fake, fake, fake, fake, fake, fake)
    status = lib.citrus_sweep_persistent_static(*args, None, 4, 8, 1, 1, 1, None, 10 ** 9, None)
    assert status == 1 and b"null plane offsets" in lib.citrus_last_error_string()
    status = lib.citrus_sweep_persistent_static(*args, offsets.ctypes.data, 8192, 8, 1, 1, 1, None, 10 ** 9, None)
    assert status == 1 and b"8191" in lib.citrus_last_error_string()
    for timeout in (0, -5):
        status = lib.citrus_sweep_persistent_static(*args, offsets.ctypes.data, 4, 8, 1, 1, 1, None, timeout, None)
        assert status == 1 and b"timeout_ns" in lib.citrus_last_error_string()
