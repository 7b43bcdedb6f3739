"""The project's autotuner: launch shapes picked by timing their candidates on the device, once per problem shape.

A choice is keyed by the tuned operation, the problem's shape and the device name. The first time a key is met
outside a CUDA-graph capture, every candidate runs once to warm up and then ``repeats`` times between CUDA events on
the current stream; the fastest (median) wins, a smaller candidate within ``slack`` of it when the candidates are
ordered by cost (fewer views per launch: less memory). Choices persist in a JSON table
(``$CITRUS_GB300_TUNING``, else ``~/.cache/citrus_gb300/tuning.json``); a key met during a capture without a choice
gets the caller's default, untimed.

Tuned here:

* ``small_k_gemm``: the small-K product's kernel — the float32 streaming forms against the shared-memory tiled
  kernel at each of its tile heights (``citrus_small_k_gemm_config``) and, in the bf16x3 precision, the tcgen05
  bf16 hi/lo product, timed into a scratch output;
* ``sweep``: views per persistent sweep launch of the batched step and the form of the sweep threads
  (``citrus_sweep_persistent_config``), timed on a store of ones of that many views (the sweep's memory traffic
  does not depend on the values; non-zero moments keep the divisions on their usual path), the per-view time
  compared.
"""

from __future__ import annotations

import json
import os
import statistics
import threading
from pathlib import Path
from typing import Callable, Optional, Sequence

import torch

from . import _lib

_LOCK = threading.Lock()


def _default_path() -> Path:
    env = os.environ.get("CITRUS_GB300_TUNING")
    return Path(env) if env else Path.home() / ".cache" / "citrus_gb300" / "tuning.json"


class Autotuner:
    """Timed choices between candidates, kept in memory and in a JSON file."""

    def __init__(self, path: Optional[os.PathLike] = None, repeats: int = 3, enabled: bool = True) -> None:
        self.path = Path(path) if path is not None else _default_path()
        self.repeats = max(1, int(repeats))
        self.enabled = enabled
        self.table: dict = {}
        self.timings: dict = {}
        try:
            self.table = json.loads(self.path.read_text())
        except (OSError, ValueError):
            self.table = {}

    @staticmethod
    def key(op: str, device: torch.device, **shape) -> str:
        name = torch.cuda.get_device_name(device) if device.type == "cuda" else device.type
        return f"{op}|{name}|" + ",".join(f"{k}={shape[k]}" for k in sorted(shape))

    def _save(self) -> None:
        try:
            self.path.parent.mkdir(parents=True, exist_ok=True)
            tmp = self.path.with_suffix(f".{os.getpid()}.tmp")
            tmp.write_text(json.dumps(self.table, indent=1, sort_keys=True))
            os.replace(tmp, self.path)
        except OSError:
            pass  # a read-only home keeps the choices in memory only

    def choose(self, key: str, candidates: Sequence, run: Callable, default, *, slack: float = 0.0,
               per_unit: Optional[Callable] = None):
        """The candidate ``run(c)`` runs fastest for ``key`` (``default`` while a graph is being captured or when
        tuning is off). ``per_unit(c)`` divides a candidate's time (e.g. per view); with ``slack`` > 0 the first
        candidate (in the given order) within ``slack`` of the fastest wins."""
        candidates = list(candidates)
        entry = self.table.get(key)
        if entry is not None and entry.get("choice") in candidates:
            return entry["choice"]
        if not self.enabled or not candidates or torch.cuda.is_current_stream_capturing():
            return default
        with _LOCK:
            stream = torch.cuda.current_stream()
            times = {}
            for c in candidates:
                try:
                    run(c)
                except _lib.CitrusKernelError:
                    continue                       # a candidate the shape does not admit
                samples = []
                for _ in range(self.repeats):
                    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                    e0.record(stream)
                    run(c)
                    e1.record(stream)
                    e1.synchronize()
                    samples.append(e0.elapsed_time(e1))
                t = statistics.median(samples)
                times[json.dumps(c)] = t / (per_unit(c) if per_unit else 1.0)
            if not times:
                return default
            best = min(times.values())
            choice = None
            for c in candidates:
                t = times.get(json.dumps(c))
                if t is not None and t <= best * (1.0 + slack):
                    choice = c
                    break
            self.table[key] = {"choice": choice, "ms": times}
            self.timings[key] = times
            self._save()
            return choice


_TUNER: Optional[Autotuner] = None


def tuner() -> Autotuner:
    """The process's autotuner (``CITRUS_GB300_AUTOTUNE=0`` turns timing off: defaults only)."""
    global _TUNER
    if _TUNER is None:
        _TUNER = Autotuner(enabled=os.environ.get("CITRUS_GB300_AUTOTUNE", "1") != "0")
    return _TUNER


GEMM_CANDIDATES = ([1, 0], [2, 1], [2, 2], [2, 4], [2, 8], [2, 16])   # (variant, tile row groups)


TENSOR_CORES = [3, 0]   # the tcgen05 bf16 hi/lo product, a candidate of the bf16x3 precision


def small_k_gemm_config(A, B, C, M: int, K: int, J: int, batch: int, sb: int, sc: int, accumulate: bool,
                        tensor_cores=None) -> list:
    """(variant, tile rows) of the small-K product for this shape, tuned into a scratch output: the float32 forms,
    and the tensor-core product ([3, 0]) when ``tensor_cores(out, ld_out, stride_out)`` runs it."""
    key = Autotuner.key("small_k_gemm" + ("_bf16x3" if tensor_cores else ""), A.device, M=M, K=K, J=J, batch=batch,
                        acc=int(bool(accumulate)),
                        aligned=int(J % 4 == 0 and B.stride(1) % 4 == 0 and C.stride(1) % 4 == 0))
    entry = tuner().table.get(key)
    if entry is not None:
        return entry["choice"]
    if torch.cuda.is_current_stream_capturing():
        return list(TENSOR_CORES) if tensor_cores else [0, 0]
    scratch = torch.empty((batch, M, J), device=A.device, dtype=torch.float32)
    stream = _lib.stream_handle(A.device)

    def run(c):
        if c == TENSOR_CORES:
            tensor_cores(scratch, J, M * J if batch > 1 else 0)
            return
        _lib.call("citrus_small_k_gemm_config", A.data_ptr(), A.stride(0), B.data_ptr(), B.stride(1),
                  scratch.data_ptr(), J, M, K, J, batch, sb, M * J if batch > 1 else 0, int(bool(accumulate)),
                  int(c[0]), int(c[1]), stream)

    candidates = list(GEMM_CANDIDATES) + ([list(TENSOR_CORES)] if tensor_cores and M <= 128 * 8 else [])
    choice = tuner().choose(key, candidates, run, list(TENSOR_CORES) if tensor_cores else [0, 0])
    del scratch
    return choice


VIEW_CANDIDATES = (1, 2, 4, 8)
# thread forms of the persistent sweep (each thread solves its lane in every view): one view at a time with the
# registers capped for 5 (form 1), 6 (form 3) or 4 (form 5) blocks of 256 threads per SM, or the loads of 2 (form 2)
# or 4 (form 4) views issued before their solves
UNROLL_CANDIDATES = (1, 3, 5, 2, 4)
# the tiled schedule (one grid barrier per tile diagonal) in the forms that came closest to the plane wavefront on the
# 64^3 x 120-direction grid: (thread form, tile edge, directions per task); directions per task are capped by the chunk
TILED_CANDIDATES = ((2, 4, 5), (2, 8, 3), (1, 4, 5), (1, 8, 3))


def sweep_config(ctx, mu_cells, num_groups: int, views: int, default=(4, 2, 0, 1), dc: int = 0) -> tuple:
    """(views per sweep launch, ``kernels.SweepForm``) for ``views`` views on this grid and chunks of ``dc``
    directions per octant (0: all): the per-view time of the sweep on a store of ones of 1, 2, 4 or 8 views (those
    whose store takes at most a quarter of the free device memory) in each form (the plane wavefront in each
    lanes-per-thread form, the tiled schedule per tile edge, thread form and directions per task); the first (fewest
    views) within 3 % of the fastest."""
    from . import kernels

    N, Q = ctx.num_cells, 4 * num_groups
    D8 = ctx.directions_per_octant if dc <= 0 else min(int(dc), ctx.directions_per_octant)
    c_chunk = ctx.c if D8 == ctx.directions_per_octant else ctx.c[:, :D8].contiguous()
    device = ctx.device
    # "form" names the forms' meaning: entries timed before the tiled schedule existed are not reused
    key = Autotuner.key("sweep", device, N=N, D8=D8, G=num_groups, shape="x".join(map(str, ctx.shape)),
                        form="views-per-thread+tiles")
    entry = tuner().table.get(key)
    if entry is None and not torch.cuda.is_current_stream_capturing():
        free, _ = torch.cuda.mem_get_info(device)
        per_view = 8 * D8 * N * Q * 4
        forms = [[u, 0, 1] for u in UNROLL_CANDIDATES] + [[u, t, min(d, D8)] for u, t, d in TILED_CANDIDATES]
        candidates = [[b, *f] for b in VIEW_CANDIDATES if b * per_view <= free // 4 for f in forms]
        candidates = candidates or [[1, *f] for f in forms]
        stores = {}

        def run(c):
            b, u, t, d = c
            if b not in stores:
                stores.clear()
                torch.cuda.empty_cache()
                stores[b] = torch.ones(b, 8, D8, N, Q, device=device)  # non-zero moments, as in a real step
            kernels.sweep_chunk(ctx, stores[b], mu_cells, c_chunk, kernels.SweepForm(u, t, d))

        tuner().choose(key, candidates, run, list(default), slack=0.03, per_unit=lambda c: float(c[0]))
        stores.clear()
        torch.cuda.empty_cache()
        entry = tuner().table.get(key)
    b, u, t, d = entry["choice"] if entry is not None else default
    return min(int(b), max(1, views)), kernels.SweepForm(int(u), int(t), int(d))
