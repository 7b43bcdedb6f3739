"""Build and bind the C restatements of the oracle (``oracle/c/*.c``): test infrastructure and the timed CPU baseline.

``build()`` compiles them with gcc (-O2, OpenMP, no machine-specific flags, so the same source builds on x86_64 and
aarch64) into ``oracle/_build/liboracle.so``.
"""

from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
SOURCES = sorted((HERE / "c").glob("*.c"))
LIBRARY = HERE / "_build" / "liboracle.so"
_LIB = None


def build(force: bool = False) -> Path:
    LIBRARY.parent.mkdir(exist_ok=True)
    newest = max(s.stat().st_mtime for s in SOURCES)
    if force or not LIBRARY.exists() or LIBRARY.stat().st_mtime < newest:
        cmd = ["gcc", "-O2", "-fopenmp", "-fPIC", "-shared", "-o", str(LIBRARY), *map(str, SOURCES), "-lm"]
        result = subprocess.run(cmd, capture_output=True, text=True)
        if result.returncode != 0:
            raise RuntimeError(f"oracle build failed:\n{result.stderr}")
    return LIBRARY


def library():
    global _LIB
    if _LIB is None:
        _LIB = ctypes.CDLL(str(build()))
        _LIB.oracle_ld_sweep_chunk.restype = ctypes.c_int
        _LIB.oracle_ld_sweep_chunk.argtypes = [ctypes.c_void_p] * 7 + [ctypes.c_int64] * 4
    return _LIB


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


def sweep_chunk(plan, c: np.ndarray, mu_cells: np.ndarray, source: np.ndarray) -> np.ndarray:
    """The C sweep of one chunk; same arguments and result as ``oracle.sweep.sweep_chunk``.

    plan: (offsets, octant, cell, upstream) of ``oracle.sweep.plan``; c [8, Dc, 3]; mu_cells [N, G];
    source [8, Dc, N, G, 4]. Returns psi [8, Dc, N, G, 4] float64.
    """
    offsets, octant, cell, upstream = (np.ascontiguousarray(a, dtype=np.int64) for a in plan)
    store = np.ascontiguousarray(source, dtype=np.float64).copy()
    c = np.ascontiguousarray(c, dtype=np.float64)
    mu = np.ascontiguousarray(mu_cells, dtype=np.float64)
    _, Dc, N, G, _ = store.shape
    library().oracle_ld_sweep_chunk(_p(store), _p(mu), _p(c), _p(octant), _p(cell), _p(upstream), _p(offsets),
                                    len(offsets) - 1, N, G, Dc)
    return store
