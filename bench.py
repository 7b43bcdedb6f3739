"""Benchmark of the CITRUS scatter step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference] [--workload step|sweep]

Prints one JSON line. The default workload is the batched circular cone-beam scatter step: 64^3 cells of 0.4 cm,
8 groups (30-120 keV), P5, 120 sweep directions, a 256 x 192 curved panel, 60 views per outer iteration; one step
is the full scatter step of every view (uncollided fluence, one accumulator sweep, the signal-only collapsed-cone
image), with the accumulator sweeps of 4 views in one persistent launch (``--batch``) and float32 spherical-harmonic
products (``--precision bf16x3`` runs them on the tcgen05 tensor cores with a bfloat16 hi/lo split and reports the
scatter-to-primary error against float32). ``--workload sweep`` times the accumulator sweep alone (scattering
moments, source expansion, wavefront sweep, moment accumulation) of one view.

The reference arm (``--impl reference``) times the float64 CPU restatement of the same path on the host cores, on a
bounded sample of the same workload, and reports the same metric.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))


def _parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--workload", default="step", choices=["step", "sweep", "learned", "sweep-form", "mixed"],
                   help="step: the scatter step of every view (the headline); sweep: the accumulator sweep alone; "
                        "learned: the learned proposal alone (training and converged steps); sweep-form: one sweep "
                        "form on a store of ones of --views views at --cells (profiling); mixed: --views views "
                        "(default 4) of the 128x128x96, G=16, P7, 240-direction workload in float32 and bf16x3 "
                        "products")
    p.add_argument("--sweep-form", default="1,0,1",
                   help="sweep-form workload: thread form, tile edge (0: plane wavefront), directions per task")
    p.add_argument("--views", type=int, default=0, help="views per step (0: the workload's 60)")
    p.add_argument("--method", default="persistent", choices=["persistent", "planes"])
    p.add_argument("--dc", type=int, default=0, help="directions per octant per sweep chunk (0: all)")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    p.add_argument("--precision", default="fp32", choices=["fp32", "bf16x3"],
                   help="arithmetic of the spherical-harmonic products (bf16x3: tcgen05 tensor cores, hi/lo split)")
    p.add_argument("--no-mixed", action="store_true",
                   help="skip the second measurement of the step with the tensor-core bf16 hi/lo products")
    p.add_argument("--batch", type=int, default=0,
                   help="views per persistent sweep launch (0: the autotuner's choice; 1: citrus_view_step per view)")
    p.add_argument("--cells", type=int, default=64, help="cells per axis of the step workload (64; smaller for "
                                                         "profiling captures)")
    p.add_argument("--no-graph", dest="graph", action="store_false",
                   help="run every step eagerly instead of replaying the outer iteration from a CUDA graph")
    p.add_argument("--no-plain", action="store_true",
                   help="skip the measurement of the plain form (citrus_view_step per view, eager)")
    p.add_argument("--no-learned", action="store_true",
                   help="skip the learned higher-order proposal measurement (training and converged steps)")
    p.add_argument("--learned-cells", default="24,24,16",
                   help="cells of the learned-proposal workload (rows,cols,slices; 96,96,64 is the full size)")
    p.add_argument("--learned-phantoms", type=int, default=64, help="training phantoms (two views each)")
    p.add_argument("--learned-epochs", type=int, default=60)
    p.add_argument("--learned-views", type=int, default=6, help="unseen phantom views of the evaluation")
    return p.parse_args()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.samples = []
        self.window = (0.0, float("inf"))
        self._stop = threading.Event()
        self._thread = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                vals = [v.strip() for v in out.stdout.strip().split(",")]
                if len(vals) >= 7:
                    self.samples.append([time.monotonic()] + vals)
            except Exception:  # noqa: BLE001
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._thread = threading.Thread(target=self._run, daemon=True)
        self._thread.start()
        return self

    def __exit__(self, *exc):
        self._stop.set()
        self._thread.join(timeout=10)

    def mark(self, start: float, end: float) -> None:
        """The timed region, in time.monotonic() seconds: the summary uses the samples inside it."""
        self.window = (start, end)

    def summary(self) -> dict:
        lo, hi = self.window
        inside = [s[1:] for s in self.samples if lo <= s[0] <= hi] or [s[1:] for s in self.samples]
        sm = [float(s[0]) for s in inside if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in inside if s[1].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({n for s in inside for n, v in zip(names, s[3:7]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(inside)}


def _peaks() -> dict:
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        data = json.loads(path.read_text())
        return {"hbm_gbs": float(data["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


# =====================================================================================================================
# workloads
# =====================================================================================================================

def sweep_workload(device):
    """One view's accumulator sweep at 64^3, G = 8, P5, 120 directions."""
    import numpy as np
    import torch

    from citrus_gb300 import kernels
    from citrus_gb300.workloads import config2_sweep_problem

    prob = config2_sweep_problem(device)
    return prob


def run_gb300(args):
    import torch

    from citrus_gb300 import kernels
    from citrus_gb300.source_iteration import scatter_moments, scatter_source_function
    from citrus_gb300.transport_sweep import sweep
    from citrus_gb300.workloads import config2_sweep_problem

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=device)

    prob = config2_sweep_problem(device)
    ctx, mu_t, transfer, phi0 = prob["ctx"], prob["mu_t"], prob["transfer"], prob["phi"]
    N, G = ctx.num_cells, int(mu_t.shape[0])
    D8 = args.dc if 0 < args.dc < ctx.directions_per_octant else ctx.directions_per_octant
    updates = 8 * D8 * N * G

    # events around the sweep kernel itself, on the stream it runs on
    sweep_times = []
    stream = torch.cuda.current_stream(device)

    def one_step(phi, record):
        T = scatter_moments(transfer, phi)
        source = scatter_source_function(ctx, T)
        mu_cells = mu_t.reshape(G, N).t().contiguous()
        store = torch.empty(8, D8, N, 4 * G, device=device)
        idx = ctx.direction_indices(0, D8)
        source(idx, out=store.view(8 * D8, *ctx.shape, G, 4))
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        kernels.sweep_planes(ctx.flat_index, store, mu_cells, ctx.c[:, :D8].contiguous(), method=args.method)
        e1.record(stream)
        moments = torch.empty(ctx.num_moments, N * 4 * G, device=device)
        kernels.small_k_gemm(ctx.Y_weighted.index_select(0, idx).t().contiguous(), store.view(8 * D8, -1), moments)
        if record:
            sweep_times.append((e0, e1))
        return moments.view(ctx.num_moments, N, G, 4).permute(2, 0, 3, 1).reshape(G, ctx.num_moments, 4, *ctx.shape)

    phi = phi0
    for _ in range(args.warmup):
        one_step(phi, False)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    sampler = ClockSampler(local)
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with sampler:
        torch.cuda.synchronize()
        start.record(stream)
        for _ in range(args.steps):
            one_step(phi, True)
        end.record(stream)
        torch.cuda.synchronize()
    elapsed = start.elapsed_time(end) / 1e3
    if dist:
        t = torch.tensor([elapsed], device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t)
    kernel_s = statistics.mean(a.elapsed_time(b) / 1e3 for a, b in sweep_times)
    # e2e through host buffers: the accumulator moments in from pinned host memory, the new ones out
    host_phi = torch.empty(phi0.shape, dtype=torch.float32, pin_memory=True)
    host_phi.copy_(phi0.cpu())
    host_out = torch.empty(phi0.shape, dtype=torch.float32, pin_memory=True)
    torch.cuda.synchronize()
    e2e0, e2e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e2e0.record(stream)
    for _ in range(args.steps):
        dev_phi = host_phi.to(device, non_blocking=True).view(phi0.shape)
        new = one_step(dev_phi, False)
        host_out.copy_(new, non_blocking=True)
    e2e1.record(stream)
    torch.cuda.synchronize()
    e2e_s = e2e0.elapsed_time(e2e1) / 1e3
    peaks = _peaks()
    achieved = updates * 32 / kernel_s / 1e9
    line = {
        "metric": "accumulator sweep cell*dir*group updates/s (scatter-step sweep stage)",
        "value": updates * args.steps * world / elapsed, "unit": "updates/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": elapsed * 1e3 / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"64^3 cells x 0.4 cm, G=8, P5 (36 moments), {8 * D8} of 120 directions (6x20), one view "
                               f"per step",
                   "l2": "inputs larger than L2 (4.0 GB store)", "sweep_method": args.method},
        "e2e": {"value": updates * args.steps / e2e_s, "unit": "updates/s",
                "h2d_bytes_per_step": host_phi.numel() * 4, "d2h_bytes_per_step": host_out.numel() * 4},
        "gpu_launches": 4 * args.steps,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "traffic": None, "peak_source": peaks["source"],
                     "kernel": "sweep persistent wavefront", "kernel_ms": kernel_s * 1e3,
                     "algorithmic_bytes": updates * 32},
        "clocks": sampler.summary(),
    }
    if rank == 0:
        line["cpu_baseline"] = None if args.no_cpu else cpu_baseline_sweep()
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def cpu_baseline_sweep(budget_s: float = 20.0) -> dict:
    """The C restatement of the sweep (float64, OpenMP on every host core) on whole-grid chunks of one direction per
    octant, as many of the view's 15 chunks as fit the time budget."""
    import numpy as np

    from citrus_gb300.workloads import config2_sweep_problem_host
    from oracle import native
    from oracle import sweep as osweep

    prob = config2_sweep_problem_host()
    shape, G = prob["shape"], prob["G"]
    N = int(np.prod(shape))
    plan = osweep.plan(shape)
    rng = np.random.default_rng(0)
    mu_cells = np.ascontiguousarray(prob["mu_t"].reshape(G, N).T)
    source = rng.random((8, 1, N, G, 4))
    native.sweep_chunk(plan, prob["c"][:, :1], mu_cells, source)  # warm-up (threads, pages)
    done = 0
    t0 = time.perf_counter()
    while time.perf_counter() - t0 < budget_s and done < 15:
        native.sweep_chunk(plan, prob["c"][:, done:done + 1], mu_cells, source)
        done += 1
    elapsed = time.perf_counter() - t0
    return {"value": 8 * done * N * G / elapsed, "unit": "updates/s", "cores": os.cpu_count(), "kind": "port",
            "sample": f"{done} of 15 direction chunks (8 directions each) of one 64^3 x G=8 view sweep, float64 C "
                      f"restatement, OpenMP"}


def run_sweep_form(args):
    """One accumulator-sweep form (``kernels.SweepForm``) on the batched-views grid at --cells, a store of ones of
    --views views: CUDA-event time per launch and the algorithmic HBM fraction (32 B per update). For profiling."""
    import numpy as np
    import torch

    from citrus_gb300 import kernels
    from citrus_gb300.quadrature import product_quadrature
    from citrus_gb300.transport_sweep import make_sweep_context
    from citrus_gb300.workloads import batched_views

    device = torch.device("cuda")
    w = batched_views(cells=args.cells)
    ctx = make_sweep_context(w.grid, product_quadrature(w.num_polar, w.num_azimuthal), w.legendre_order, device)
    G, N, D8 = w.library.num_groups, ctx.num_cells, ctx.directions_per_octant
    mu = torch.as_tensor(np.einsum("mg,mijk->gijk", w.library.mu_t, w.rho).reshape(G, N).T.copy(),
                         dtype=torch.float32, device=device)
    V = max(1, args.views)
    form = kernels.SweepForm(*(int(x) for x in args.sweep_form.split(",")))
    store = torch.ones(V, 8, D8, N, 4 * G, device=device)
    for _ in range(args.warmup):
        kernels.sweep_chunk(ctx, store, mu, ctx.c, form)
    torch.cuda.synchronize()
    times = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        kernels.sweep_chunk(ctx, store, mu, ctx.c, form)
        e1.record()
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = statistics.median(times)
    algorithmic = 32 * V * 8 * D8 * N * G
    peaks = _peaks()
    print(json.dumps({"workload": f"sweep form {args.sweep_form} on {args.cells}^3 cells, G={G}, {8 * D8} directions, "
                                  f"{V} views per launch", "ms_per_launch": ms, "ms_per_view": ms / V,
                      "algorithmic_bytes": algorithmic, "frac": algorithmic / ms / 1e6 / peaks["hbm_gbs"]}),
          flush=True)


def run_mixed(args):
    """The mixed-precision workload (``workloads.mixed_precision_views``: 128 x 128 x 96 cells of 0.25 cm, G = 16,
    P7, 240 directions, curved 512 x 384 panel) on ``--views`` views (default 4) of the 90: two outer iterations (a
    cold start and a warm step) of ``batched_view_steps`` (eager) with float32 and with bf16x3 tensor-core products.
    Reports ms per view of the warm step (CUDA events) in each precision and, per view, the bf16x3 step's error
    against the float32 step: collided scalar flux (cells above 1e-3 of the maximum), scatter image and SPR (pixels
    whose primary exceeds 1e-3 of its maximum), element-wise maxima."""
    import dataclasses

    # one view's accumulator is 25.8 GB here: growable segments keep the allocator's free blocks reusable
    os.environ.setdefault("PYTORCH_CUDA_ALLOC_CONF", "expandable_segments:True")
    import torch

    from citrus_gb300.batched import batched_view_steps, direction_chunk
    from citrus_gb300.citrus_step import CitrusState
    from citrus_gb300.responses import ideal_counting_response, no_grid
    from citrus_gb300.scatter_solver import ScatterSolver, SolverConfig
    from citrus_gb300.workloads import mixed_precision_views

    device = torch.device("cuda")
    cells = (args.cells * 2, args.cells * 2, args.cells * 3 // 2) if args.cells != 64 else (128, 128, 96)
    w = mixed_precision_views(cells=cells)
    V = args.views if args.views > 0 else 4
    angles = [float(a) for a in w.angles()[:: max(1, w.num_views // V)][:V]]
    base = SolverConfig(num_groups=w.library.num_groups, legendre_order=w.legendre_order, num_polar=w.num_polar,
                        num_azimuthal=w.num_azimuthal, transport_cell_cm=w.transport_cell_cm,
                        quadrature_point_spacing_cm=0.5, cone_num_polar=w.cone_num_polar,
                        cone_num_azimuthal=w.cone_num_azimuthal)
    rho = torch.as_tensor(w.rho, dtype=torch.float32, device=device)
    results = {}
    for precision in ("fp32", "bf16x3"):
        solver = ScatterSolver(w.library, dataclasses.replace(base, moment_precision=precision), w.geometry,
                               detector=ideal_counting_response(), grid_response=no_grid(), device=device)
        fields = solver.material_fields(rho, w.grid)
        _, _, states = batched_view_steps(solver, [CitrusState() for _ in angles], fields, angles, batch=0)  # cold
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        signals, _, states = batched_view_steps(solver, states, fields, angles, batch=0)                 # warm
        e1.record()
        e1.synchronize()
        primaries = torch.stack([solver.primary(solver.material_fields(rho, w.grid), a)["signal"] for a in angles])
        results[precision] = {"ms_per_view": e0.elapsed_time(e1) / V, "signals": signals.clone(),
                              "scalar": [s.collided_moments[:, 0, 0].clone() for s in states],
                              "primary": primaries}
        ctx = solver.sweep_context(solver.material_fields(rho, w.grid).grid_coarse)
        results[precision]["chunk"] = direction_chunk(ctx.num_cells, w.library.num_groups, ctx.directions_per_octant)
        del states, signals, fields
        torch.cuda.empty_cache()
    a, b = results["fp32"], results["bf16x3"]
    per_view = []
    for v in range(V):
        p = a["primary"][v]
        mask = p > 1e-3 * p.max()
        s32, s16 = a["signals"][v], b["signals"][v]
        f32, f16 = a["scalar"][v], b["scalar"][v]
        cells_mask = f32.abs() > 1e-3 * f32.abs().max()
        per_view.append({
            "collided_scalar_max_rel": float(((f16 - f32).abs()[cells_mask] / f32.abs()[cells_mask]).max()),
            "scatter_max_rel": float(((s16 - s32).abs()[mask] / s32.abs()[mask]).max()),
            "spr_max_rel": float(((s16[mask] / p[mask]) / (s32[mask] / p[mask]) - 1).abs().max())})
    N = w.grid.num_voxels
    print(json.dumps({
        "workload": f"mixed_precision_views: {cells[0]}x{cells[1]}x{cells[2]} cells x {w.transport_cell_cm:g} cm, "
                    f"G=16 (20-140 keV), P7 (64 moments), 240 sweep directions (10x24), cone 16x32, curved 512x384 "
                    f"panel, {V} of the 90 views",
        "directions_per_octant_per_chunk": results["fp32"]["chunk"],
        "ms_per_view_warm_step": {"fp32": a["ms_per_view"], "bf16x3": b["ms_per_view"]},
        "updates_per_view": 240 * N * 16,
        "bf16x3_against_fp32_per_view": per_view,
        "note": "the float64 comparison of the mixed precision is the single-view workload's (the reference's own "
                "float64 run; mixed_precision_bf16x3.float64_reference_error of the step bench)"}), flush=True)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    if args.workload == "step":
        for _ in range(max(1, args.warmup)):   # imports, pages, OpenMP threads
            cpu_baseline_step(cells=args.cells, image_directions=1, fc_directions=1, sweep_chunks=1, points=1024,
                              slices=1)
        runs, wall = [], []
        for i in range(args.steps):
            t0 = time.perf_counter()
            runs.append(cpu_baseline_step(cells=args.cells, seed=i))
            wall.append(time.perf_counter() - t0)
        value = statistics.median(r["value"] for r in runs)
        base = dict(runs[0], value=value)
        base["sample"] = (f"median of {args.steps} steps, each a bounded sample of one view's stages timed and scaled "
                          f"to the whole view (the step's own duration is ms_per_step): " + base["sample"])
        line = {"metric": STEP_METRIC, "value": value, "unit": "ms/view", "impl": "reference", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * statistics.mean(wall),
                "higher_is_better": False, "dtype": "f64", "data": "synthetic (seeded phantom and library)",
                "config": step_config(args, 60, args.batch), "cpu_baseline": base, "extrapolated": True,
                "e2e": {"value": value, "unit": "ms/view", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    base = cpu_baseline_sweep(budget_s=max(5.0, 60.0 / max(1, args.steps + args.warmup)))
    line = {"metric": "accumulator sweep cell*dir*group updates/s (scatter-step sweep stage)", "value": base["value"],
            "unit": "updates/s", "impl": "reference", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "higher_is_better": True, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "64^3 cells x 0.4 cm, G=8, P5 (36 moments), 120 directions (6x20), one view"},
            "cpu_baseline": base, "e2e": {"value": base["value"], "unit": "updates/s", "h2d_bytes_per_step": 0,
                                          "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def cpu_baseline_step(cells: int = 64, image_directions: int = 1, fc_directions: int = 1, sweep_chunks: int = 1,
                      points: int = 4096, slices: int = 2, seed: int = 0) -> dict:
    """ms/view of the float64 restatement of one view's scatter step, each stage timed on a bounded sample and scaled
    linearly by its unit count to the whole view: the uncollided fluence (rays to ``points`` of the V quadrature
    points), the first-collision sampling correction and LD moments (``fc_directions`` of the sweep directions), the
    accumulator sweep (``sweep_chunks`` of the 15 eight-direction chunks, C with OpenMP, with the numpy source
    expansion and moment accumulation of those chunks), the two scattering-moment contractions (``slices`` of the
    z slices) and the collapsed-cone image (``image_directions`` of the panel-facing cone directions). The work does
    not depend on the values, so the fields between the stages are seeded stand-ins of the right shapes."""
    import numpy as np

    from citrus_gb300.quadrature import product_quadrature, real_spherical_harmonics
    from citrus_gb300.responses import ideal_counting_response
    from citrus_gb300.scatter_image import panel_direction_set
    from citrus_gb300.workloads import batched_views
    from oracle import image as oimage, native, physics, siddon, sweep as osweep

    w = batched_views(cells=cells)
    lib, geo, grid, rho = w.library, w.geometry, w.grid, w.rho
    G, L, angle = lib.num_groups, w.legendre_order, 0.0
    N_sh = (L + 1) ** 2
    V, shape = grid.num_voxels, grid.shape
    rng = np.random.default_rng(seed)
    stages = {}

    def timed(name, scale, fn):
        t0 = time.perf_counter()
        fn()
        stages[name] = (time.perf_counter() - t0) * scale

    src = np.asarray(geo.source_position(angle))
    pts = siddon.centers(grid).reshape(-1, 3)[rng.choice(V, points, replace=False)]

    def uncollided():
        path = siddon.upstream_to_points(rho, grid, src, pts)
        d = pts - src
        return physics.group_transmission(lib, path) * (physics.source_weight(geo, angle, pts) / (d * d).sum(-1))

    timed("uncollided", V / points, uncollided)
    phi_uc = 1e-4 * (1.0 + rng.random((G, *shape)))
    q = product_quadrature(w.num_polar, w.num_azimuthal)
    q = q.reordered(q.by_octant())
    K_s = q.omega.shape[0]
    om, wt = q.omega[:fc_directions], q.weight[:fc_directions]

    def first_collision():
        scale, beta, _, _ = physics.correction(lib, rho, phi_uc, grid, geo, angle, om, wt)
        physics.first_collision_moments(lib, rho, phi_uc, grid, geo, angle, om, scale, beta, 1)

    timed("first collision", K_s / fc_directions, first_collision)
    lib_t = lib.truncated(L)
    transfer = np.einsum("mabl,mijk->ablijk", lib_t.mu_s_l, rho[:, :, :, :slices])
    acc = 1e-3 * rng.random((G, N_sh, 4, shape[0], shape[1], slices))
    timed("scattering moments", 2 * shape[2] / slices,
          lambda: (osweep.scatter_moments(transfer, acc), osweep.scatter_moments(transfer, acc[:, :, 0])))
    del transfer, acc
    N = V
    plan = osweep.plan(shape)
    mu_cells = np.ascontiguousarray(np.einsum("mg,mijk->gijk", lib.mu_t, rho).reshape(G, N).T)
    c = (np.abs(q.omega) / np.asarray(grid.deltas)).reshape(8, -1, 3)
    Y = real_spherical_harmonics(L, q.omega).reshape(8, -1, N_sh)
    T_cells = 1e-3 * rng.random((N_sh, N * G * 4))
    moments = np.zeros((N_sh, N * G * 4))
    Dc = c.shape[1]

    def sweep():
        for j in range(sweep_chunks):
            Yc = Y[:, j]                                                   # one direction per octant
            source = (Yc @ T_cells).reshape(8, 1, N, G, 4)
            psi = native.sweep_chunk(plan, c[:, j:j + 1], mu_cells, source)
            moments[...] += Yc.T @ psi.reshape(8, -1)

    timed("sweep", Dc / sweep_chunks, sweep)
    del T_cells, moments
    cone = panel_direction_set(geo, angle, (w.cone_num_polar, w.cone_num_azimuthal), max_polar_angle=grid)
    keep, *_ = oimage.direction_weights(cone.omega, cone.weight, geo, angle, ideal_counting_response(),
                                        lib.group_energy)
    kept = np.flatnonzero(keep)
    pick = kept[:image_directions]
    T_img = 1e-3 * rng.random((G, N_sh, *shape))
    mu_t_coarse = np.einsum("mg,mijk->gijk", lib.mu_t, rho)
    timed("image", kept.size / image_directions,
          lambda: oimage.combined_image(lib, rho, phi_uc, grid, 1, T_img, L, geo, angle, cone.omega[pick],
                                        cone.weight[pick], cone.cell_width[pick], mu_t_coarse,
                                        ideal_counting_response()))
    total_ms = 1e3 * sum(stages.values())
    return {"value": total_ms, "unit": "ms/view", "cores": os.cpu_count(), "kind": "port",
            "stages_ms": {k: round(1e3 * v, 1) for k, v in stages.items()},
            "sample": (f"one view of batched_views at {cells}^3, float64 oracle: uncollided rays to {points} of {V} "
                       f"points, first collision at {fc_directions} of {K_s} sweep directions, sweep {sweep_chunks} of "
                       f"{Dc} chunks (C, OpenMP), moments on {slices} of {shape[2]} slices, image at "
                       f"{image_directions} of {kept.size} cone directions; each stage scaled linearly to the view "
                       f"(BLAS and OpenMP stages use every core, numpy elementwise stages one)")}


# =====================================================================================================================
# the scatter step of every view
# =====================================================================================================================

def make_step_solver(device, views: int = 0, cells: int = 64, precision: str = "fp32"):
    """The batched-views workload: solver, fields input, view angles (64^3, G = 8, P5, 120 directions, curved 256 x 192
    panel, cone 16 x 32, ideal counting detector, no grid)."""
    from citrus_gb300.responses import ideal_counting_response, no_grid
    from citrus_gb300.scatter_solver import ScatterSolver, SolverConfig
    from citrus_gb300.workloads import batched_views

    w = batched_views(cells=cells)
    config = SolverConfig(num_groups=w.library.num_groups, legendre_order=w.legendre_order, num_polar=w.num_polar,
                          num_azimuthal=w.num_azimuthal, transport_cell_cm=w.transport_cell_cm,
                          quadrature_point_spacing_cm=0.5, cone_num_polar=w.cone_num_polar,
                          cone_num_azimuthal=w.cone_num_azimuthal, moment_precision=precision)
    solver = ScatterSolver(w.library, config, w.geometry, detector=ideal_counting_response(), grid_response=no_grid(),
                           device=device)
    angles = w.angles()
    if views:
        angles = angles[:views]
    return w, solver, angles


STEP_METRIC = "scatter-step ms/view (all views of one outer iteration; cell*dir*group updates/s alongside)"


def step_config(args, views: int, batch: int) -> dict:
    """The ``config`` of the step's bench line, the same for both arms."""
    return {"workload": step_workload_name(args.cells, views, batch, args.graph),
            "l2": "inputs larger than L2 (4 GB sweep store per view)", "moment_precision": args.precision}


def sweep_form_name(solver, w, rho_dev) -> str:
    """The accumulator sweep's form the autotuner chose for this grid (plane wavefront or tiled schedule)."""
    from citrus_gb300.batched import sweep_launch_config
    fields = solver.material_fields(rho_dev, w.grid)
    _, form, dc = sweep_launch_config(solver, fields, 60, 0)
    chunks = f", {dc} directions per octant per chunk"
    if form.tile > 0:
        return (f"tiled: {form.tile}^3-cell tiles, {form.dirs_per_block} directions per task, thread form "
                f"{form.thread_form}{chunks}")
    return f"plane wavefront, thread form {form.thread_form}{chunks}"


def step_workload_name(cells: int, views: int, batch: int = 1, graph: bool = False) -> str:
    how = ("citrus_view_step per view" if batch == 1 else
           "batched_view_steps, the accumulator sweeps of several views per persistent launch (views per launch "
           "picked by the autotuner)" if batch <= 0 else
           f"batched_view_steps, the accumulator sweeps of {batch} views per persistent launch")
    if graph:
        how = f"GraphedOuterIteration: {how}, the outer iteration replayed from one CUDA graph"
    return (f"batched_views: {cells}^3 cells x {25.6 / cells:g} cm, G=8 (30-120 keV), P5, 120 sweep directions, cone "
            f"16x32, curved 256x192 panel, {views} views per rank per step, one accumulator sweep per view ({how}, "
            f"signal only)")


def _dims(address) -> tuple:
    """The three int64 sizes behind a host-array address handed to the library."""
    import ctypes
    arr = ctypes.cast(address, ctypes.POINTER(ctypes.c_int64))
    return int(arr[0]), int(arr[1]), int(arr[2])


def emission_bytes(args) -> int:
    """Algorithmic bytes of one citrus_attenuated_emission_moments call: every input read once (the densities and
    fluence of the points, the cells' attenuation, optical depths or material path lengths and scattering-source
    moments, the harmonics), the emission written once."""
    M, G, dims, f, k = int(args[1]), int(args[3]), _dims(args[5]), int(args[6]), int(args[14])
    TM, NS = int(args[17]), int(args[21])
    V = dims[0] * dims[1] * dims[2]
    NC = V // (f ** 3)
    C = 1 if args[23] is not None else G
    tau = k * NC * (TM if args[16] is not None else G)
    floats = (M + G + 1) * V + G * NC + tau + NS * G * NC + k * NS + k * G + k * V * C + 2 * k * (-(-V // 32))
    return 4 * floats


def product_emission_bytes(args) -> int:
    """Algorithmic bytes of one citrus_attenuated_emission call: as the fused form, with the multiple-collision
    source [K, NC, G] read in place of the moments and harmonics."""
    M, G, dims, f, k = int(args[1]), int(args[3]), _dims(args[5]), int(args[6]), int(args[14])
    TM = int(args[17])
    V = dims[0] * dims[1] * dims[2]
    NC = V // (f ** 3)
    C = 1 if args[21] is not None else G
    tau = k * NC * (TM if args[16] is not None else G)
    floats = (M + G + 1) * V + G * NC + tau + k * G * NC + k * G + k * V * C + 2 * k * (-(-V // 32))
    return 4 * floats


def downstream_bytes(args) -> int:
    """citrus_downstream_cumulative: the cell volume read once, the optical depths [K, C, V] written once."""
    C, dims, K = int(args[1]), _dims(args[3]), int(args[6])
    V = dims[0] * dims[1] * dims[2]
    return 4 * (C * V + K * C * V)


def sweep_bytes(args) -> int:
    """citrus_sweep_persistent: 32 B per cell x direction x group update (source moments in, fluence moments out)."""
    N, G, Dc, views = int(args[8]), int(args[9]), int(args[10]), int(args[11])
    return 32 * views * 8 * Dc * N * G


def tiled_sweep_bytes(args) -> int:
    """citrus_sweep_tiled: the same 32 B per update as the plane wavefront."""
    N, G, Dc, views = int(args[10]), int(args[11]), int(args[12]), int(args[13])
    return 32 * views * 8 * Dc * N * G


SWEEP_ENTRY_POINTS = ("citrus_sweep_tiled", "citrus_sweep_persistent_config", "citrus_sweep_persistent")
STEP_TIMED = {"citrus_attenuated_emission_moments": emission_bytes, "citrus_attenuated_emission": product_emission_bytes,
              "citrus_downstream_cumulative": downstream_bytes, "citrus_downstream_cumulative_tables": downstream_bytes,
              "citrus_sweep_persistent": sweep_bytes, "citrus_sweep_persistent_config": sweep_bytes,
              "citrus_sweep_tiled": tiled_sweep_bytes,
              "citrus_oblique_project": None, "citrus_oblique_project_scratch": None, "citrus_box_blur": None,
              "citrus_small_k_gemm": None,
              "citrus_small_k_gemm_config": None, "citrus_small_k_gemm_bf16x3": None, "citrus_first_collision_moments": None,
              "citrus_first_collision_means": None, "citrus_source_expansion_first": None,
              "citrus_source_expansion_first_bf16x3": None,
              "citrus_first_collision_correction": None, "citrus_scattering_moments": None}


def count_launches(fn) -> dict:
    """Kernels launched by ``fn()`` (one untimed step): this library's, from its own launch counter."""
    import torch

    from citrus_gb300 import _lib

    torch.cuda.synchronize()
    before = _lib.launch_count()
    fn()
    torch.cuda.synchronize()
    return {"citrus": _lib.launch_count() - before}


def spr_error(w, solver, angles, device) -> dict:
    """Scatter-to-primary ratio after two steps of a few views (the second one warm: the scattering-source expansion,
    the moment accumulation and the image product all run in the solver's moment precision) against the same steps
    with float32 products: max over panel pixels of |SPR - SPR_fp32| / SPR_fp32, and the scatter signal's error
    relative to its maximum."""
    import dataclasses

    import torch

    from citrus_gb300.citrus_step import CitrusState, citrus_view_step
    from citrus_gb300.view_sharding import gather_signals
    from citrus_gb300.scatter_solver import ScatterSolver

    ref_solver = ScatterSolver(solver.library, dataclasses.replace(solver.config, moment_precision="fp32"),
                               solver.geometry, detector=solver.detector, grid_response=solver.grid_response,
                               device=device)
    rho = torch.as_tensor(w.rho, dtype=torch.float32, device=device)
    fields, ref_fields = solver.material_fields(rho, w.grid), ref_solver.material_fields(rho, w.grid)
    worst_spr, worst_signal = 0.0, 0.0
    for angle in angles:
        _, _, state = citrus_view_step(solver, CitrusState(), fields, float(angle), primary=False)
        _, _, ref_state = citrus_view_step(ref_solver, CitrusState(), ref_fields, float(angle), primary=False)
        s, p, _ = citrus_view_step(solver, state, fields, float(angle), primary=True)
        s_ref, _, _ = citrus_view_step(ref_solver, ref_state, ref_fields, float(angle), primary=False)
        mask = p > 1e-3 * p.max()
        spr, spr_ref = s[mask] / p[mask], s_ref[mask] / p[mask]
        worst_spr = max(worst_spr, float(((spr - spr_ref).abs() / spr_ref.abs().clamp_min(1e-30)).max()))
        worst_signal = max(worst_signal, float((s - s_ref).abs().max() / s_ref.abs().max()))
    return {"against": "the same two steps with float32 spherical-harmonic products", "views": len(angles),
            "spr_max_rel": worst_spr, "signal_max_rel": worst_signal}


def float64_reference_error(device) -> dict:
    """The single-view workload (32^3 cells of 0.5 cm, one 60 keV group, P3, 48 sweep directions, cone 16 x 32, flat
    64 x 64 panel) stepped twice by ``citrus_view_step`` in float32 and in bf16x3 products, against the reference's
    own float64 run of the same two steps (the committed fixture ``tests/golden/config1_view.npz``, made by
    ``tests/golden/make_golden.py``): the worst per-pixel relative error of the scatter image and of the SPR over the
    pixels whose primary exceeds 1e-3 of its maximum, and of the collided scalar flux over the cells above 1e-3 of its
    maximum."""
    import numpy as np
    import torch

    from citrus_gb300.citrus_step import CitrusState, citrus_view_step
    from citrus_gb300.responses import ideal_counting_response, no_grid
    from citrus_gb300.scatter_solver import ScatterSolver, SolverConfig
    from citrus_gb300.workloads import single_view

    with np.load(ROOT / "tests" / "golden" / "config1_view.npz") as d:
        ref = {k: d[k] for k in d.files}
    w = single_view()
    out = {"workload": "single_view: 32^3 x 0.5 cm, G=1 (60 keV), P3, 48 sweep directions, cone 16x32, flat 64x64",
           "against": "the reference's float64 CPU run of the same two citrus_view_step calls"}
    for precision in ("fp32", "bf16x3"):
        config = SolverConfig(num_groups=1, legendre_order=w.legendre_order, num_polar=w.num_polar,
                              num_azimuthal=w.num_azimuthal, transport_cell_cm=w.transport_cell_cm,
                              quadrature_point_spacing_cm=0.5, cone_num_polar=w.cone_num_polar,
                              cone_num_azimuthal=w.cone_num_azimuthal, direction_chunk=6, moment_precision=precision)
        solver = ScatterSolver(w.library, config, w.geometry, detector=ideal_counting_response(),
                               grid_response=no_grid(), device=device)
        fields = solver.material_fields(torch.as_tensor(w.rho, dtype=torch.float32, device=device), w.grid)
        state = CitrusState()
        for _ in range(2):
            scatter, primary, state = citrus_view_step(solver, state, fields, 0.0, primary=True)
        s = scatter.double().cpu().numpy()
        p = primary.double().cpu().numpy()
        phi = state.collided_moments[:, 0, 0].double().cpu().numpy()
        s_ref, p_ref, phi_ref = ref["step2_scatter"], ref["primary"], ref["step2_scalar"][:, 0].astype(np.float64)
        mask = p_ref > 1e-3 * p_ref.max()
        cells = np.abs(phi_ref) > 1e-3 * np.abs(phi_ref).max()
        out[precision] = {
            "scatter_max_rel": float((np.abs(s - s_ref)[mask] / np.abs(s_ref)[mask]).max()),
            "spr_max_rel": float(np.abs((s[mask] / p[mask]) / (s_ref[mask] / p_ref[mask]) - 1).max()),
            "collided_scalar_max_rel": float((np.abs(phi - phi_ref)[cells] / np.abs(phi_ref)[cells]).max())}
    return out


def mixed_precision_step(args, w, solver, angles, rho_dev, device) -> dict:
    """The same step with the spherical-harmonic products on the tcgen05 tensor cores (bfloat16 hi/lo split, float32
    accumulation): ms/view over ``args.steps`` steps after one warm-up step, and its scatter-to-primary error against
    the float32 products."""
    import dataclasses

    import torch

    from citrus_gb300.batched import GraphedOuterIteration, batched_view_steps
    from citrus_gb300.citrus_step import CitrusState, citrus_view_step
    from citrus_gb300.scatter_solver import ScatterSolver

    mixed = ScatterSolver(solver.library, dataclasses.replace(solver.config, moment_precision="bf16x3"),
                          solver.geometry, detector=solver.detector, grid_response=solver.grid_response,
                          device=device)
    states = [CitrusState() for _ in angles]
    graphed = GraphedOuterIteration(mixed, w.grid, angles, batch=args.batch) if args.graph else None

    def step():
        if graphed is not None:
            graphed.step(rho_dev)
            return
        fields = mixed.material_fields(rho_dev, w.grid)
        if args.batch > 1:
            _, _, new = batched_view_steps(mixed, states, fields, [float(a) for a in angles], batch=args.batch)
            states[:] = new
        else:
            for v, a in enumerate(angles):
                _, _, states[v] = citrus_view_step(mixed, states[v], fields, float(a), primary=False)

    for _ in range(2 if graphed is not None else 1):   # the cold start, then the warm step and its capture
        step()
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream(device)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    torch.cuda.synchronize()
    value = e0.elapsed_time(e1) / (args.steps * len(angles))
    del graphed, states
    torch.cuda.empty_cache()
    return {"value": value, "unit": "ms/view", "steps": args.steps, "cuda_graph": bool(args.graph),
            "spr_error": spr_error(w, mixed, angles[:2], device),
            "float64_reference_error": float64_reference_error(device)}


def plain_single_view_step(w, solver, angles, rho_dev, device) -> dict:
    """The plain form of the same outer iteration: ``citrus_view_step`` per view, eagerly, one sweep launch per view
    (no batching, no graph), float32 products; ms/view over one warm step after the cold start."""
    import torch

    from citrus_gb300.citrus_step import CitrusState, citrus_view_step

    states = [CitrusState() for _ in angles]
    stream = torch.cuda.current_stream(device)

    def step():
        fields = solver.material_fields(rho_dev, w.grid)
        for v, a in enumerate(angles):
            _, _, states[v] = citrus_view_step(solver, states[v], fields, float(a), primary=False)

    step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    step()
    e1.record(stream)
    torch.cuda.synchronize()
    value = e0.elapsed_time(e1) / len(angles)
    states.clear()
    torch.cuda.empty_cache()
    return {"value": value, "unit": "ms/view", "steps": 1,
            "form": "citrus_view_step per view: one sweep launch per view, eager, float32 products"}


def learned_measurement(args, device) -> dict:
    """The learned higher-order proposal on the learned-proposal workload (random ellipsoid phantoms, 12 groups, P5,
    6 x 28 directions, cone 16 x 32, curved 256 x 192 panel) at ``--learned-cells``: the solver generates the
    training triples, the network (4 levels, 32 base channels) trains on the GPU, and on unseen phantom views the
    scatter signal is converged per sweep to an SPR change of 0.5 % from the proposal and from the cold start (the
    plain source iteration). ms/view from CUDA events around each view's converged step; SPR errors against a
    Neumann series converged to 1e-6."""
    import numpy as np
    import torch

    from citrus_gb300 import learned
    from citrus_gb300.citrus_step import CitrusState, citrus_view_step, project_scatter
    from citrus_gb300.responses import ideal_counting_response, no_grid
    from citrus_gb300.scatter_solver import ScatterSolver, SolverConfig
    from citrus_gb300.workloads import ellipsoid_phantom, learned_proposal

    cells = tuple(int(c) for c in args.learned_cells.split(","))
    w = learned_proposal(1, cells)
    config = SolverConfig(num_groups=w.library.num_groups, legendre_order=w.legendre_order, num_polar=w.num_polar,
                          num_azimuthal=w.num_azimuthal, transport_cell_cm=w.transport_cell_cm,
                          quadrature_point_spacing_cm=w.transport_cell_cm, cone_num_polar=w.cone_num_polar,
                          cone_num_azimuthal=w.cone_num_azimuthal)
    solver = ScatterSolver(w.library, config, w.geometry, detector=ideal_counting_response(), grid_response=no_grid(),
                           device=device)
    rng = np.random.default_rng(0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    samples = []
    for seed in range(args.learned_phantoms):
        samples += learned.generate_training_data(solver, [ellipsoid_phantom(w.grid, 1000 + seed)], w.grid,
                                                  [float(a) for a in rng.uniform(0, 2 * math.pi, 2)])
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    proposal = learned.HigherOrderProposal(w.library.num_materials, w.library.num_groups, seed=0, device=device)
    losses = proposal.fit(samples, epochs=args.learned_epochs, batch=4, lr=1e-3, seed=0)
    torch.cuda.synchronize()
    t2 = time.perf_counter()
    steps = len(samples) // 4 * args.learned_epochs
    results = {"plain": [], "learned": []}
    proposal_err, first_cold = [], []
    stream = torch.cuda.current_stream(device)
    for k in range(args.learned_views):
        seed = 5000 + k
        angle = float(np.random.default_rng(seed).uniform(0, 2 * math.pi))
        rho = torch.as_tensor(ellipsoid_phantom(w.grid, seed), dtype=torch.float32, device=device)
        fields = solver.material_fields(rho, w.grid)
        first, total = learned.collided_orders(solver, fields, angle, tolerance=1e-6)
        higher = learned.scalar_flux(total) - learned.scalar_flux(first)
        pred = proposal.predict(fields.rho_coarse, learned.scalar_flux(first))
        proposal_err.append(float(torch.linalg.vector_norm(pred - higher) / torch.linalg.vector_norm(higher)))
        phi_uc = solver.uncollided_fluence(fields, angle)
        cone = solver.cone_quadrature(w.grid, angle)
        ref = project_scatter(solver, None, w.grid, angle, phi_uc, total, fields, cone, signal_only=True)["signal"]
        primary = solver.primary(fields, angle)["signal"]
        mask = primary > 1e-3 * primary.max()

        def spr_err(scatter):
            return float(((scatter - ref)[mask].abs() / ref[mask].abs()).max())

        cold, _, _ = citrus_view_step(solver, CitrusState(cone_quadrature=cone), fields, angle, primary=False)
        first_cold.append(spr_err(cold))
        for name, prop in (("plain", None), ("learned", proposal)):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.synchronize()
            e0.record(stream)
            judged, _ = learned.converged_view_step(solver, fields, angle, prop, primary=primary, cone=cone)
            e1.record(stream)
            torch.cuda.synchronize()
            results[name].append((e0.elapsed_time(e1), judged.sweeps, spr_err(judged.scatter), judged.accepted))

    def summary(rows):
        return {"ms_per_view": statistics.mean(r[0] for r in rows), "sweeps_mean": statistics.mean(r[1] for r in rows),
                "spr_err_max": max(r[2] for r in rows), "accepted": sum(bool(r[3]) for r in rows)}

    return {
        "workload": f"learned_proposal: {cells[0]}x{cells[1]}x{cells[2]} cells x {w.transport_cell_cm:.2f} cm, G=12 "
                    f"(30-120 keV), P5, 168 sweep directions, cone 16x32, curved 256x192 panel; random ellipsoid "
                    f"phantoms (water 8-18 cm semi-axes, 0-4 air/soft-tissue/bone inserts)",
        "network": {"levels": 4, "base_channels": 32, "parameters": proposal.net.num_parameters(),
                    "weights": "bf16 (float32 master copies)", "accumulate": "f32"},
        "train": {"phantoms": args.learned_phantoms, "samples": len(samples), "epochs": args.learned_epochs,
                  "adam_steps": steps, "data_s": round(t1 - t0, 2), "train_s": round(t2 - t1, 2),
                  "ms_per_adam_step": round(1e3 * (t2 - t1) / max(1, steps), 3), "loss_first": losses[0],
                  "loss_last": losses[-1]},
        "eval_views": args.learned_views,
        "proposal_rel_err_max": max(proposal_err),
        "first_step_spr_err_max": {"cold_start": max(first_cold)},
        "converged_to_spr_error_estimate": 0.005,
        "plain": summary(results["plain"]),
        "learned": summary(results["learned"]),
        "combined_outer_iterations": combined_measurement(args, device, w, solver, proposal),
    }


def combined_measurement(args, device, w, solver, proposal, views: int = 12, seed: int = 5100,
                         tolerance: float = 0.005, max_iterations: int = 16) -> dict:
    """The scatter step of every view of one phantom (``views`` views over 360 degrees) iterated over outer iterations
    until every view's scatter-to-primary ratio is within ``tolerance`` of its converged value (a Neumann series to
    1e-6, computed before the timing), in two forms: the plain one, ``citrus_view_step`` per view from a cold start,
    eager, float32 products; and the combined one, every view seeded with the learned proposal (one sweep of the
    first-collision source and the network, timed) and stepped by ``GraphedOuterIteration`` (the views' sweeps
    batched per persistent launch, the outer iteration replayed from a CUDA graph) with the bf16x3 tensor-core
    products. CUDA-event times of every step; the error is checked between steps, outside the timed spans."""
    import dataclasses

    import numpy as np
    import torch

    from citrus_gb300 import learned
    from citrus_gb300.batched import GraphedOuterIteration, resolve_batch
    from citrus_gb300.citrus_step import CitrusState, citrus_view_step, project_scatter
    from citrus_gb300.scatter_solver import ScatterSolver
    from citrus_gb300.workloads import ellipsoid_phantom

    angles = [2 * math.pi * v / views for v in range(views)]
    rho = torch.as_tensor(ellipsoid_phantom(w.grid, seed), dtype=torch.float32, device=device)
    fields = solver.material_fields(rho, w.grid)
    refs, masks = [], []
    for a in angles:
        _, total = learned.collided_orders(solver, fields, a, tolerance=1e-6)
        phi_uc = solver.uncollided_fluence(fields, a)
        cone = solver.cone_quadrature(w.grid, a)
        refs.append(project_scatter(solver, None, w.grid, a, phi_uc, total, fields, cone, signal_only=True)["signal"])
        p = solver.primary(fields, a)["signal"]
        masks.append(p > 1e-3 * p.max())

    def worst(signals) -> float:
        return max(float(((s - r)[m].abs() / r[m].abs()).max()) for s, r, m in zip(signals, refs, masks))

    stream = torch.cuda.current_stream(device)

    def timed(fn):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = fn()
        e1.record(stream)
        e1.synchronize()
        return out, e0.elapsed_time(e1)

    # plain: cold start, one eager citrus_view_step per view and outer iteration
    states = [CitrusState() for _ in angles]
    plain_ms, plain_errors = [], []

    def plain_step():
        out = []
        for v, a in enumerate(angles):
            s, _, states[v] = citrus_view_step(solver, states[v], fields, a, primary=False)
            out.append(s)
        return out

    plain_step()                                       # warm-up of tables and contexts, not counted
    states = [CitrusState() for _ in angles]
    for _ in range(max_iterations):
        signals, ms = timed(plain_step)
        plain_ms.append(ms)
        plain_errors.append(worst(signals))
        if plain_errors[-1] <= tolerance:
            break
    # combined: learned seeds, batched sweeps, graph replays, bf16x3 products
    mixed = ScatterSolver(solver.library, dataclasses.replace(solver.config, moment_precision="bf16x3"),
                          solver.geometry, detector=solver.detector, grid_response=solver.grid_response, device=device)
    mixed.direction_context_cache_size = max(mixed.direction_context_cache_size, views)
    mfields = mixed.material_fields(rho, w.grid)
    batch = resolve_batch(mixed, mfields, views, 0)

    def seeds():
        out = []
        for a in angles:
            _, first = learned.first_collided(mixed, mfields, a)
            out.append(proposal.propose(mfields.rho_coarse, first))
        return out

    seeds()                                            # warm-up, not counted
    graphed = GraphedOuterIteration(mixed, w.grid, angles, batch=batch)
    accumulators, seed_ms = timed(seeds)
    graphed.seed(rho, accumulators)
    combined_ms, combined_errors = [], []
    for _ in range(max_iterations):
        (signals, _), ms = timed(lambda: graphed.step(rho))
        combined_ms.append(ms)
        combined_errors.append(worst(list(signals)))
        if combined_errors[-1] <= tolerance:
            break
    plain_total, combined_total = sum(plain_ms), seed_ms + sum(combined_ms)
    # the first combined iteration also records the CUDA graph (once per run of outer iterations); its replays are
    # what every further outer iteration costs
    replay = statistics.mean(combined_ms[1:]) if len(combined_ms) > 1 else combined_ms[0]
    steady_total = seed_ms + replay * len(combined_ms)
    return {"views": views, "phantom_seed": seed, "spr_tolerance": tolerance,
            "plain": {"outer_iterations": len(plain_ms), "ms_per_view": plain_total / views,
                      "ms_per_view_per_iteration": [round(m / views, 3) for m in plain_ms],
                      "spr_err_per_iteration": [round(e, 5) for e in plain_errors]},
            "combined": {"outer_iterations": len(combined_ms), "ms_per_view": combined_total / views,
                         "seed_ms_per_view": seed_ms / views, "views_per_sweep_launch": batch,
                         "ms_per_view_per_iteration": [round(m / views, 3) for m in combined_ms],
                         "spr_err_per_iteration": [round(e, 5) for e in combined_errors],
                         "form": "learned seeds + GraphedOuterIteration (batched sweeps, CUDA graph) + bf16x3"},
            "speedup": plain_total / combined_total,
            "speedup_graph_recorded": plain_total / steady_total,
            "note": "the combined form's first iteration includes recording the CUDA graph; speedup_graph_recorded "
                    "counts every iteration at the replay time (the graph is recorded once per run)"}


def run_step(args):
    import torch

    from citrus_gb300 import _lib
    from citrus_gb300.batched import GraphedOuterIteration, batched_view_steps, resolve_batch
    from citrus_gb300.citrus_step import CitrusState, citrus_view_step

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    device = torch.device("cuda", local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=device)
    w, solver, angles = make_step_solver(device, args.views, args.cells, args.precision)
    # weak scaling: every rank owns V views of the V x world views of the outer iteration, round-robin (views rank,
    # rank + world, ...: the angles of the first V views offset by the rank), as view_sharding.owned_views assigns
    angles = angles + rank * (2 * math.pi / len(angles)) / max(1, world)
    V = len(angles)
    rho_host = torch.as_tensor(w.rho, dtype=torch.float32).pin_memory()
    rho_dev = rho_host.to(device)
    requested_batch = args.batch
    if args.batch <= 0:
        args.batch = resolve_batch(solver, solver.material_fields(rho_dev, w.grid), V, 0)
    states = [CitrusState() for _ in angles]
    stream = torch.cuda.current_stream(device)
    graphed = GraphedOuterIteration(solver, w.grid, angles, batch=args.batch) if args.graph else None

    def eager_step(rho, signals=None):
        fields = solver.material_fields(rho, w.grid)
        if args.batch > 1:
            out, _, new_states = batched_view_steps(solver, states, fields, [float(a) for a in angles],
                                                    batch=args.batch)
            states[:] = new_states
        else:
            outs = []
            for v, angle in enumerate(angles):
                scatter, _, states[v] = citrus_view_step(solver, states[v], fields, float(angle), primary=False)
                outs.append(scatter)
            out = torch.stack(outs)
        finish(out, signals)

    def finish(out, signals):
        # with several ranks, every rank's views (round-robin shares of the V x world views) are all-gathered in view
        # order, the outer iteration's one collective (view_sharding.gather_signals); rank 0 copies them out
        if dist:
            out = gather_signals(out, V * world)
        if signals is not None:
            signals.copy_(out[:V] if dist else out, non_blocking=True)

    def one_step(rho, signals=None):
        if graphed is None:
            return eager_step(rho, signals)
        out, _ = graphed.step(rho)
        finish(out, signals)

    sampler = ClockSampler(local)  # started before the warm-up: its first nvidia-smi call is slow
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with sampler:
        for _ in range(args.warmup):
            one_step(rho_dev)
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        t_start = time.monotonic()
        torch.cuda.nvtx.range_push("citrus_timed_steps")   # the range a profiler's launch list is filtered to
        start.record(stream)
        for _ in range(args.steps):
            one_step(rho_dev)
        end.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        sampler.mark(t_start, time.monotonic())
    elapsed = start.elapsed_time(end) / 1e3
    if dist:
        t = torch.tensor([elapsed], device=device)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        elapsed = float(t)
    # e2e: the densities in from pinned host memory, every view's scatter signal out to pinned host memory
    Rd, Cd = w.geometry.image_shape
    host_signals = torch.empty(V, Rd, Cd, dtype=torch.float32).pin_memory()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        one_step(rho_host.to(device, non_blocking=True), host_signals)
    e1.record(stream)
    torch.cuda.synchronize()
    e2e = e0.elapsed_time(e1) / 1e3
    graph_replays = 0 if graphed is None else graphed.replays
    del graphed, one_step
    torch.cuda.empty_cache()
    # the entry points of one eager step of the same views (CUDA events on the launch stream around every call;
    # a graph replay has no calls to time), outside the timed region
    if args.graph:
        for _ in range(2):
            eager_step(rho_dev)
    torch.cuda.synchronize()
    with _lib.timed_calls(*STEP_TIMED, capture={n: f for n, f in STEP_TIMED.items() if f}) as calls:
        eager_step(rho_dev)
        torch.cuda.synchronize()
    breakdown_steps = 1
    per_entry = {}
    for name, recs in calls.items():
        if recs:
            per_entry[name] = [a.elapsed_time(b) / 1e3 for _, a, b in recs]
    # the roofline is reported for the entry point with the largest share among those with an algorithmic byte count
    ranked = sorted((n for n in per_entry if STEP_TIMED[n] is not None), key=lambda n: -sum(per_entry[n]))
    top = ranked[0] if ranked else None
    top_s = per_entry[top] if top else []
    top_bytes = [info for info, _, _ in calls[top]] if top else []
    launches = count_launches(lambda: eager_step(rho_dev))   # a replay launches the same kernels as the eager step
    states.clear()
    torch.cuda.empty_cache()
    plain = None if args.no_plain else plain_single_view_step(w, solver, angles, rho_dev, device)
    spr = spr_error(w, solver, angles[:2], device) if args.precision != "fp32" else None
    mixed = None
    if args.precision == "fp32" and not args.no_mixed:
        mixed = mixed_precision_step(args, w, solver, angles, rho_dev, device)
    ms_per_view = elapsed * 1e3 / (args.steps * V)
    N = w.grid.num_voxels
    updates = 8 * (w.num_polar * w.num_azimuthal // 8) * N * w.library.num_groups
    peaks = _peaks()
    achieved = sum(top_bytes) / sum(top_s) / 1e9 if top_s else None
    line = {
        "metric": STEP_METRIC,
        "value": ms_per_view / max(1, world), "unit": "ms/view", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": elapsed * 1e3 / args.steps, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded phantom and library)",
        "config": step_config(args, V, requested_batch),
        "sweep_launch": {"views_per_launch": args.batch, "autotuned": requested_batch <= 0,
                         "form": sweep_form_name(solver, w, rho_dev)},
        "updates_per_s": updates * V * args.steps * world / elapsed,
        "e2e": {"value": e2e * 1e3 / (args.steps * V) / max(1, world), "unit": "ms/view",
                "h2d_bytes_per_step": rho_host.numel() * 4, "d2h_bytes_per_step": host_signals.numel() * 4},
        "gpu_launches": launches["citrus"] * args.steps,
        "cuda_graph": {"outer_iteration_replayed": bool(args.graph), "replays": graph_replays},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": None if achieved is None else achieved / peaks["hbm_gbs"], "traffic": None,
                     "peak_source": peaks["source"],
                     "entry_point": top, "launches": len(top_s),
                     "kernel_ms_mean": 1e3 * statistics.mean(top_s) if top_s else None,
                     "algorithmic_bytes_per_launch": statistics.mean(top_bytes) if top_bytes else None},
        "entry_point_ms_per_view": {n: round(1e3 * sum(t) / (breakdown_steps * V), 3)
                                    for n, t in sorted(per_entry.items(), key=lambda x: -sum(x[1]))},
        "clocks": sampler.summary(),
    }
    sweep_name = next((n for n in SWEEP_ENTRY_POINTS if calls.get(n)), None)
    sweep_recs = calls.get(sweep_name) or [] if sweep_name else []
    if sweep_recs:
        sweep_s = sum(per_entry[sweep_name])
        sweep_gbs = sum(info for info, _, _ in sweep_recs) / sweep_s / 1e9
        line["sweep_roofline"] = {"entry_point": sweep_name, "bound": "hbm", "achieved": sweep_gbs,
                                  "peak": peaks["hbm_gbs"], "unit": "GB/s",
                                  "frac": sweep_gbs / peaks["hbm_gbs"], "launches": len(sweep_recs),
                                  "kernel_ms_mean": 1e3 * sweep_s / len(sweep_recs),
                                  "algorithmic_bytes_per_launch": statistics.mean(i for i, _, _ in sweep_recs)}
    if spr is not None:
        line["spr_error"] = spr
    if mixed is not None:
        line["mixed_precision_bf16x3"] = mixed
    if plain is not None:
        line["plain_single_view_step"] = plain
    if not args.no_learned and rank == 0:
        line["learned_proposal"] = learned_measurement(args, device)
    if rank == 0:
        line["cpu_baseline"] = None if args.no_cpu else cpu_baseline_step(cells=args.cells)
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_learned(args) -> None:
    """The learned-proposal measurement on its own (one JSON line; the profile captures of the network's kernels)."""
    import torch

    device = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
    torch.cuda.set_device(device)
    result = learned_measurement(args, device)
    print(json.dumps({"metric": "learned proposal: ms/view to an estimated SPR error of 0.5 % (plain sweeps judge)",
                      "value": result["learned"]["ms_per_view"], "unit": "ms/view", "n_gpus": 1,
                      "higher_is_better": False, "data": "synthetic (seeded random ellipsoid phantoms)",
                      "dtype": "f32", "config": {"workload": result["workload"]}, "learned_proposal": result}),
          flush=True)


if __name__ == "__main__":
    a = _parse()
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "step":
        run_step(a)
    elif a.workload == "learned":
        run_learned(a)
    elif a.workload == "sweep-form":
        run_sweep_form(a)
    elif a.workload == "mixed":
        run_mixed(a)
    else:
        run_gb300(a)
