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


def test_grid_source_and_table_entry_points_check_their_arguments(library):
    """The anti-scatter-grid accumulation, the source field, the crossing tables, the tables' downstream trace and
    the oblique projection's scratch refuse bad arguments with CITRUS_EINVAL before any CUDA call (the fake
    addresses below are never dereferenced)."""
    import ctypes
    lib = _lib.library()
    fake = 256
    # more than 32 groups, more than two sets of septa, weights neither per channel nor shared
    status = lib.citrus_grid_signal_sum(fake, 2, 33, 4, 5, 1, 1, 1, 1, fake, 5, None, 0, None, None, None, None,
                                        None, None, None, fake, 1, 0, None)
    assert status == 1 and b"groups <= 32" in lib.citrus_last_error_string()
    status = lib.citrus_grid_signal_sum(fake, 2, 3, 4, 5, 1, 1, 1, 1, fake, 5, None, 3, None, None, None, None,
                                        None, None, None, fake, 1, 0, None)
    assert status == 1 and b"two sets" in lib.citrus_last_error_string()
    status = lib.citrus_grid_signal_sum(fake, 2, 3, 4, 5, 1, 1, 1, 1, fake, 4, None, 0, None, None, None, None,
                                        None, None, None, fake, 1, 0, None)
    assert status == 1 and b"cols | 1" in lib.citrus_last_error_string()
    status = lib.citrus_grid_signal_sum(fake, 2, 3, 4, 5, 1, 1, 1, 1, fake, 5, None, 1, None, None, None, None,
                                        None, None, None, fake, 1, 0, None)
    assert status == 1 and b"septa arrays" in lib.citrus_last_error_string()
    field = (ctypes.c_double * 23)()
    dims = (ctypes.c_int64 * 3)(2, 2, 2)
    # a profile without the panel; off-focal nodes without their count; a thickness without the path output
    status = lib.citrus_source_field(field, None, fake, None, 0, 0.0, None, None, 0, fake, None, None, None, None, 8,
                                     1, fake, None, None)
    assert status == 1 and b"needs the panel" in lib.citrus_last_error_string()
    status = lib.citrus_source_field(field, None, None, None, 0, 0.0, fake, fake, 0, fake, None, None, None, None, 8,
                                     1, fake, None, None)
    assert status == 1 and b"off-focal" in lib.citrus_last_error_string()
    status = lib.citrus_source_field(field, None, None, fake, 1, 2.7, None, None, 0, fake, None, None, None, None, 8,
                                     1, fake, None, None)
    assert status == 1 and b"filter-path output" in lib.citrus_last_error_string()
    box = (ctypes.c_double * 6)(0, 0, 0, 1, 1, 1)
    status = lib.citrus_crossing_tables(box, dims, fake, 4, fake, 4 * 3 * 6 - 1, None)
    assert status == 1 and b"needs 72" in lib.citrus_last_error_string()
    status = lib.citrus_downstream_cumulative_tables(fake, 2, box, dims, fake, fake, 4, fake, 1.0, fake, 1, 1, 1,
                                                     None, 0, None)
    assert status == 1 and b"null crossing tables" in lib.citrus_last_error_string()
    need = int(lib.citrus_oblique_scratch_bytes(7))
    assert need > 7 * 100 and int(lib.citrus_oblique_scratch_bytes(0)) == 0
    status = lib.citrus_oblique_project_scratch(fake, 1, 0, box, dims, fake, 7, fake, 4, 4, fake, 1, 1, 1, 1, fake,
                                                need - 1, None)
    assert status == 1 and b"direction scratch" in lib.citrus_last_error_string()
