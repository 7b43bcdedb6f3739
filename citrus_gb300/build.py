"""Build recipe of the C-ABI library ``libcitrus_gb300.so`` (sm_103a only).

Each ``csrc/*.cu`` translation unit is compiled by nvcc in parallel into ``_build/`` and linked into
``citrus_gb300/_lib/libcitrus_gb300.so``; both folders are build outputs and stay out of version control. A unit is
recompiled only when it or a header is newer than its object.
"""

from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
from pathlib import Path

PACKAGE_DIR = Path(__file__).resolve().parent
SOURCE_DIR = PACKAGE_DIR / "csrc"
INCLUDE_DIR = PACKAGE_DIR.parent / "include"
BUILD_DIR = PACKAGE_DIR / "_build"
LIB_DIR = PACKAGE_DIR / "_lib"
LIBRARY_PATH = LIB_DIR / "libcitrus_gb300.so"
ARCH_FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3", "--expt-relaxed-constexpr"]


def nvcc_path() -> str:
    """The nvcc of the CUDA toolkit (CUDA_HOME, /usr/local/cuda or PATH)."""
    for root in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if root and (Path(root) / "bin" / "nvcc").exists():
            return str(Path(root) / "bin" / "nvcc")
    found = shutil.which("nvcc")
    if found is None:
        raise RuntimeError("nvcc not found: set CUDA_HOME or put nvcc on PATH")
    return found


def _headers_mtime() -> float:
    headers = list(SOURCE_DIR.glob("*.cuh")) + list(INCLUDE_DIR.glob("*.h"))
    return max((h.stat().st_mtime for h in headers), default=0.0)


def _compile(nvcc: str, source: Path, obj: Path, extra: list) -> None:
    cmd = [nvcc, *ARCH_FLAGS, *NVCC_FLAGS, *extra, "-I", str(INCLUDE_DIR), "-c", str(source), "-o", str(obj)]
    result = subprocess.run(cmd, capture_output=True, text=True)
    if result.returncode != 0:
        raise RuntimeError(f"nvcc failed on {source.name}:\n{result.stderr[-6000:]}")


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> Path:
    """Compile every translation unit for sm_103a and link the shared library; returns its path."""
    nvcc = nvcc_path()
    extra = list(extra_flags or [])
    BUILD_DIR.mkdir(exist_ok=True)
    LIB_DIR.mkdir(exist_ok=True)
    sources = sorted(SOURCE_DIR.glob("*.cu"))
    headers = _headers_mtime()
    jobs = []
    for source in sources:
        obj = BUILD_DIR / (source.stem + ".o")
        if force or not obj.exists() or obj.stat().st_mtime < max(source.stat().st_mtime, headers):
            jobs.append((source, obj))
    if jobs:
        workers = max(1, min(len(jobs), os.cpu_count() or 1))
        with concurrent.futures.ThreadPoolExecutor(workers) as pool:
            for future in [pool.submit(_compile, nvcc, s, o, extra) for s, o in jobs]:
                future.result()
    objects = [BUILD_DIR / (s.stem + ".o") for s in sources]
    if force or jobs or not LIBRARY_PATH.exists():
        tmp = LIB_DIR / (LIBRARY_PATH.name + ".tmp")
        cmd = [nvcc, *ARCH_FLAGS, "-shared", "-o", str(tmp), *map(str, objects), "-lcudart"]
        result = subprocess.run(cmd, capture_output=True, text=True)
        if result.returncode != 0:
            raise RuntimeError(f"link failed:\n{result.stderr[-4000:]}")
        os.replace(tmp, LIBRARY_PATH)
    if verbose:
        print(f"built {LIBRARY_PATH} ({len(jobs)} of {len(sources)} units compiled)")
    return LIBRARY_PATH


if __name__ == "__main__":
    build(verbose=True)
