#!/usr/bin/env python3
"""Benchmark: rays/s of the Monte Carlo view-factor tracer on one GB300.

Workload: the 64-surface mixed scene from seed 2 (16 cylinders, 16 frusta,
12 discs, 10 annuli, 10 spheres; radii U[0.05,1], lengths U[0.1,2], random
axes, centres U[-3,3]^3), 1e8 rays per step spread over the emitters by area.
A step is one pass of the tracer over those 1e8 rays.

* value   -- rays/s of the timed kernel path with the scene resident on the
             device (CUDA events on the library's stream around each step).
* e2e     -- the same through the C ABI with host buffers: scene upload,
             trace, FP64 normalisation and read-back of the tallies and F.
* roofline -- FP32 issue roofline of the tracing kernel: algorithmic FP32
             operations per ray (per-type costs, FMA = 1) / kernel time,
             against the device's measured dependent-FMA issue rate.
* cpu_baseline -- the CPU restatement of the reference kernel on all host
             cores over a bounded sample of the same workload.

``--impl reference`` times that CPU restatement alone on the same workload
(the reference's OpenCL kernel cannot run without an OpenCL runtime).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

# FP32 operations per call from the source of RayFactorGPU.cl (FMA/mad = 1, MUFU not counted).
TEST_OPS = {0: 33, 1: 39, 2: 33, 3: 23, 4: 21, 5: 23}      # per ray x surface test, by type
EMIT_OPS = {0: 52, 1: 58, 2: 55, 3: 52, 4: 48, 5: 50}      # per emitted ray, by emitter type
SPHERE_CHECK_OPS = 12                                          # per ray x bounding-sphere check
METRIC = "rays/s on 1 GB300: batched mixed-precision vs plain kernel at equal F error"


def algorithmic_ops(scene, rays) -> float:
    types = scene.primitives["type"].astype(int)
    per_ray_tests = float(sum(TEST_OPS[t] for t in types))
    return float(sum(int(r) * (EMIT_OPS[int(t)] + per_ray_tests) for r, t in zip(rays, types)))


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 25 ms (the headline's
    timed region is a few tens of ms); entering waits for the first sample so that
    the region is covered."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int = 0):
        self.rows = []
        self.proc = None
        self.device = device
        self.thread = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "25"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            t0 = time.perf_counter()
            while not self.rows and time.perf_counter() - t0 < 5.0 and self.proc.poll() is None:
                time.sleep(0.005)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 8:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc is not None:
            n = len(self.rows)  # one more sample, taken at the end of the region
            t0 = time.perf_counter()
            while len(self.rows) == n and time.perf_counter() - t0 < 1.0 and self.proc.poll() is None:
                time.sleep(0.005)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            if self.thread:
                self.thread.join(timeout=2)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[4 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(self.rows)}


def dist_info():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


WORKLOADS = {
    "enclosure3": "3-surface closed enclosure (coaxial discs r=0.5 h=1, inward cylinder), 1e7 rays per surface",
    "furnace": "furnace-like enclosure: 180 wall rings, 2x20 annuli, fibre, 30-frustum neck-down, one bounding "
               "cylinder; 1e9 rays spread by area (plain kernel: bounding-surface path)",
    "stress": "precision stress: thin annuli (0.999), 89.9 degree frusta, unit primitives 1e4 from the origin; "
              "1e8 rays spread by area",
    "ref-furnace": "the reference's own furnace model (sample-geometries input-furnace.xml as its Scene loader "
                   "reads it: 360 cylinder rings, 52 annuli, no bounding surfaces); 1e9 rays spread by area",
}


def workload_label(args) -> str:
    if args.workload in WORKLOADS:
        return WORKLOADS[args.workload]
    if args.surfaces == 64:
        return ("mixed64 seed 2: 64 surfaces (16 cyl, 16 frustum, 12 disc, 10 annulus, 10 sphere), "
                "1e8 rays/step spread by area")
    return (f"mixed scene seed 2: {args.surfaces} surfaces (mixed64 type mix), {args.rays:.0e} rays/step "
            "spread by area")


def workload(args):
    from rayfactorcl_gb300 import generators
    if args.workload == "enclosure3":
        return generators.enclosure3()
    if args.workload == "furnace":
        return generators.furnace_scene()
    if args.workload == "stress":
        return generators.precision_stress()
    if args.workload == "ref-furnace":  # tables the reference's loader wrote (tests/golden)
        from rayfactorcl_gb300.scene import Scene
        from rayfactorcl_gb300.tracer import budgets_by_area, surface_areas
        sc = Scene.from_bytes((ROOT / "tests" / "golden" / "scenes" / "input-furnace.bin").read_bytes())
        return generators.Workload("ref-furnace", "", sc, budgets_by_area(sc, 1_000_000_000, use_density=False),
                                   surface_areas(sc))
    if args.surfaces == 64:
        return generators.mixed_scene(seed=2, total_rays=args.rays)
    frac = np.array([16, 16, 12, 10, 10], float) / 64.0
    counts = np.floor(frac * args.surfaces).astype(int)
    counts[0] += args.surfaces - counts.sum()
    return generators.mixed_scene(seed=2, total_rays=args.rays, counts=tuple(int(c) for c in counts))


def flipped_rows(scene) -> np.ndarray:
    """Planar emitters (rectangle, disc, annulus) whose FP32 world normal is -z
    to within rounding."""
    out = np.zeros(scene.n, bool)
    for i, pr in enumerate(scene.primitives):
        if int(pr["type"]) not in (3, 4, 5):
            continue
        im = pr["invm"].astype(np.float32).reshape(3, 4)
        nrm = im[2, :3] / np.float32(np.sqrt(np.sum(im[2, :3].astype(np.float64) ** 2)))  # invm^T (0,0,1)
        out[i] = float(nrm[2]) < -1.0 + 1e-6
    return out


def cpu_rate(w, seconds: float, threads: int = 0):
    """Oracle rays/s on host cores over a bounded, area-weighted sample."""
    from oracle import oracle as O
    p = O.params(compat=0, key1=w.key1)
    frac = 1e-4
    while True:
        probe = np.maximum((w.rays * frac).astype(np.int64) // 4 * 4, 4)
        t0 = time.perf_counter()
        O.tally(w.scene, p, probe, threads=threads)
        dt = time.perf_counter() - t0
        if dt > 0.5 or frac >= 1.0:
            break
        frac *= 8
    scale = seconds / max(dt, 1e-3)
    sample = np.maximum((probe * scale).astype(np.int64) // 4 * 4, 4)
    t0 = time.perf_counter()
    O.tally(w.scene, p, sample, threads=threads)
    dt = time.perf_counter() - t0
    nthreads = threads if threads > 0 else O.max_threads()
    return float(sample.sum()) / dt, sample, nthreads, dt


def run_reference(args):
    """The reference method on the host cores: the CPU restatement of runGPU
    (RayFactorGPU.cl:481-527) with OpenMP over all cores.  Every step traces the
    same bounded, area-weighted sample of the workload (sized once, about
    --ref-seconds of CPU work), timed on its own; value = sample rays / mean step
    time.  Under torchrun only rank 0 works."""
    rank, world, _ = dist_info()
    if rank != 0:
        return 0
    w = workload(args)
    from oracle import oracle as O
    O.lib()
    _, sample, nthreads, _ = cpu_rate(w, seconds=args.ref_seconds)
    p = O.params(compat=0, key1=w.key1)
    step_s = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        O.tally(w.scene, p, sample)
        if i >= args.warmup:
            step_s.append(time.perf_counter() - t0)
    rays = int(sample.sum())
    value = rays / float(np.mean(step_s))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * float(np.mean(step_s)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic", "config": {"workload": workload_label(args),
                                        "kernel": "CPU restatement of RayFactorGPU.cl runGPU",
                                        "rays_per_step": rays,
                                        "step": f"a {rays}-ray area-weighted sample of the workload"},
        "cpu_baseline": {"value": value, "unit": "rays/s", "cores": nthreads, "kind": "port",
                         "sample": f"{rays} rays of the workload per step, area-weighted"},
        "e2e": {"value": value, "unit": "rays/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def time_trace(t, rays, steps, warmup, l2_flush, stream, use_bv=False):
    """Per-step device time (CUDA events on the library's stream, L2 flushed
    before each step) and the tracing kernel's own time."""
    import torch
    for _ in range(warmup):
        t.trace_async(rays, use_bv)
        torch.cuda.synchronize()
    step_ms, kern_ms = [], []
    for _ in range(steps):
        with torch.cuda.stream(stream):
            l2_flush.zero_()  # inputs are smaller than L2: flush it between steps
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
        t.trace_async(rays, use_bv)
        with torch.cuda.stream(stream):
            e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        kern_ms.append(t.last_stats()[0])
    return float(np.mean(step_ms)), float(np.mean(kern_ms))


def time_sharded(t, rays, rank, world, steps, warmup, dev, use_bv, l2_flush, with_upload=None):
    """N ranks, weak scaling: rank r traces its share of a run of world x rays per
    emitter (ray ranges split on Philox draws, rayfactorcl_gb300.shard), reads its
    int64 tallies and joins one all_reduce of them -- the path's only exchange
    step (the reference sums per-device tallies on the host, main.cpp:224-234).
    Wall time per step, max over ranks; with_upload(): re-upload the scene first
    (the end-to-end variant)."""
    import torch
    import torch.distributed as dist

    from rayfactorcl_gb300 import shard
    first, count = shard.shard_ranges(np.asarray(rays, np.int64) * world, rank, world)
    n = len(rays)
    hits = np.zeros((n, n), np.uint64)
    out = torch.zeros(n * n, dtype=torch.int64, device=dev)

    def step():
        if with_upload is not None:
            with_upload()
        t.trace_range(first, count, use_bv)
        t.read_results(hits, None)
        out.copy_(torch.from_numpy(hits.view(np.int64).reshape(-1)))
        dist.all_reduce(out, op=dist.ReduceOp.SUM)

    for _ in range(warmup):
        step()
    total = 0.0
    for _ in range(steps):
        l2_flush.zero_()
        torch.cuda.synchronize()
        dist.barrier()
        t0 = time.perf_counter()
        step()
        torch.cuda.synchronize()
        total += time.perf_counter() - t0
    m = torch.tensor([1e3 * total / steps], device=dev)
    dist.all_reduce(m, op=dist.ReduceOp.MAX)
    return float(m.item()), t.last_stats()[0]


def run_ours(args):
    import ctypes

    import torch

    from rayfactorcl_gb300 import _lib
    from rayfactorcl_gb300.tracer import PREC_EXACT, PREC_FAST, PREC_FP64, PREC_MIXED, Tracer

    rank, world, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = f"cuda:{local}"
    _lib.load()
    w = workload(args)
    sc = w.scene
    rays = w.rays
    total_rays = int(rays.sum())
    ref_ops = algorithmic_ops(sc, rays)
    headline = {"mixed": PREC_MIXED, "exact": PREC_EXACT, "fast": PREC_FAST}[args.precision]
    # the reference traces a scene with bounding surfaces through runBVGPU; every
    # kernel here follows it (the mixed kernel culls inside each bounding surface's
    # range with its own masks and spheres)
    plain_bv = bool(sc.use_bounding_volumes) and sc.bounding_volumes is not None and len(sc.bounding_volumes) > 0

    fma = ctypes.c_double()
    _lib.check(_lib.load().rf_measure_fp32_peak(local, fma))
    peak_ops = fma.value
    l2_flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    def tracer(prec, tally_mode=0):
        t = Tracer(precision=prec, key1=w.key1, device=local, rays_per_thread=args.rays_per_thread,
                   tally_mode=tally_mode)
        t.set_scene(sc)
        return t, torch.cuda.ExternalStream(t.stream_handle, device=dev)

    # -- headline kernel: scene resident, per-step device time ------------
    t, stream = tracer(headline, args.tally_mode)
    head_bv = plain_bv
    # launch shape (plain kernels) or kernel choice (mixed: small-scene vs batched) for these budgets
    t.trace_async(rays, head_bv)
    t.read_results(None, None)
    if not args.tally_mode:  # a fixed tally mode is measured as chosen
        t.autotune(head_bv)
    head_launch = t.launch_config()
    mixed_small = headline == PREC_MIXED and not head_bv and head_launch["block"] == 256
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        if world > 1:  # sharded ray ranges + one tally sum
            ms_step, kernel_ms = time_sharded(t, rays, rank, world, args.steps, args.warmup, dev, head_bv, l2_flush)
        else:
            ms_step, kernel_ms = time_trace(t, rays, args.steps, args.warmup, l2_flush, stream, head_bv)
        torch.cuda.synchronize()
    barrier()
    hits = np.zeros((sc.n, sc.n), np.uint64)
    t.read_results(hits, None)
    assert int(hits.sum()) <= total_rays * world
    refined = t.refined_count() if headline == PREC_MIXED else 0
    work = None
    if headline == PREC_MIXED and not mixed_small:  # the timed kernel does not count; one more run that does
        with Tracer(precision=headline, key1=w.key1, device=local, work_counts=True) as tc:
            tc.set_scene(sc)
            tc.trace(rays, head_bv)
            work = tc.work_counts()
    value = world * total_rays / (ms_step * 1e-3)

    # -- e2e: host buffers through the C ABI (scene upload, trace, FP64 F, read-back)
    e2e_ms = []
    if world > 1:  # the sharded step with the scene uploaded each time
        e2e_ms.append(time_sharded(t, rays, rank, world, args.steps, args.warmup, dev, head_bv, l2_flush,
                                   with_upload=lambda: t.set_scene(sc))[0])
    else:
        for i in range(args.warmup + args.steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            t.set_scene(sc)
            t.trace(rays, head_bv)
            e2e_ms.append((time.perf_counter() - t0) * 1e3)
        e2e_ms = e2e_ms[args.warmup:]
    h2d = sc.primitives.nbytes + sc.n * 64 + rays.nbytes + 32 * sc.n + 8 * sc.n
    if headline == PREC_MIXED:
        # re-centred records, hit records, spheres, patch balls, sphere chains, planes,
        # emission frames, mask rows and offsets; the cones of the direction cells
        h2d += sc.n * (112 + 64 + 16 + 16 * 16 + 8 * 16 + 16 + 5 * 16 + 8 + 16) + 512 * 16
    d2h = sc.n * sc.n * (16 if world == 1 else 8)
    t.close()

    # roofline of the headline kernel: FP32 work it performed / its time
    if mixed_small:  # every ray against every surface but a planar emitter itself
        types = sc.primitives["type"].astype(int)
        emit = float(sum(int(r) * EMIT_OPS[int(ty)] for r, ty in zip(rays, types)))
        per_ray = float(sum(TEST_OPS[int(ty)] for ty in types))
        tests = float(sum(int(r) * (per_ray - (TEST_OPS[int(ty)] if int(ty) in (3, 4, 5) else 0))
                          for r, ty in zip(rays, types)))
        if head_bv:
            tests += float(total_rays) * sum(TEST_OPS[int(b["type"])] for b in sc.bounding_volumes)
        done_ops = emit + tests
        n_tests = sum(int(r) * (sc.n - (1 if int(ty) in (3, 4, 5) else 0)) for r, ty in zip(rays, types))
        culled = 1.0 - n_tests / (float(total_rays) * sc.n)
    elif work is not None:
        types = sc.primitives["type"].astype(int)
        emit = float(sum(int(r) * EMIT_OPS[int(ty)] for r, ty in zip(rays, types)))
        tests = float(sum(int(work[k]) * TEST_OPS[k] for k in range(6)))
        if head_bv:  # every ray also tests each bounding surface (not in the counters)
            tests += float(total_rays) * sum(TEST_OPS[int(b["type"])] for b in sc.bounding_volumes)
        # every candidate of a packet gets a ray/bounding-sphere check in each of the
        # 32 lanes (12 FP32 operations: three differences, two dot products, the
        # clamp, the closest-approach product and its fma)
        checks = SPHERE_CHECK_OPS * 32.0 * float(work[6])
        done_ops = emit + tests + checks
        all_pairs = float(total_rays) * sc.n
        culled = 1.0 - float(sum(int(work[k]) for k in range(6))) / all_pairs
    else:
        done_ops, culled = ref_ops, 0.0
    achieved = done_ops / (kernel_ms * 1e-3)

    # -- the plain kernel (reference method, bit-exact) on the same rays -----
    plain = None
    if headline != PREC_EXACT and not args.no_plain:
        tp, sp = tracer(PREC_EXACT)
        tp.trace_async(rays, plain_bv)  # the workload's budgets, which the autotuner then tunes for
        tp.read_results(None, None)
        plain_cfg = tp.autotune(plain_bv)  # the plain kernel at its best launch shape
        p_step, p_kern = time_trace(tp, rays, args.steps, args.warmup, l2_flush, sp, plain_bv)
        tp.close()
        plain = {"value": world * total_rays / (p_step * 1e-3), "unit": "rays/s", "ms_per_step": p_step,
                 "kernel_ms": p_kern, "roofline_frac": ref_ops / (p_kern * 1e-3) / peak_ops,
                 "launch": plain_cfg, "arithmetic": "bit-exact with the CPU restatement (IEEE rcp/sqrt)"}
    # the same plain kernel with hardware approximations (the analogue of the
    # reference's native_* functions): no longer bit-exact, same method
    plain_fast = None
    if headline != PREC_FAST and not args.no_plain:
        tp, sp = tracer(PREC_FAST)
        tp.trace_async(rays, plain_bv)
        tp.read_results(None, None)
        fast_cfg = tp.autotune(plain_bv)
        f_step, f_kern = time_trace(tp, rays, args.steps, args.warmup, l2_flush, sp, plain_bv)
        tp.close()
        plain_fast = {"value": world * total_rays / (f_step * 1e-3), "unit": "rays/s", "ms_per_step": f_step,
                      "kernel_ms": f_kern, "roofline_frac": ref_ops / (f_kern * 1e-3) / peak_ops,
                      "launch": fast_cfg, "arithmetic": "FP32 hardware approximations (rcp/sqrt/rsqrt.approx)"}

    # -- F error at equal rays against the FP64 tracer (identical streams) ----
    ferr = None
    if not args.no_ferr:
        sub = np.maximum((rays // args.ferr_div) // 4 * 4, 4)
        Fs = {}
        for name, prec in (("fp64", PREC_FP64), ("mixed", PREC_MIXED), ("exact", PREC_EXACT), ("fast", PREC_FAST)):
            tt, _ = tracer(prec)
            Fs[name] = tt.trace(sub, plain_bv)[1]
            tt.close()
        sig = np.sqrt(np.clip(Fs["fp64"] * (1 - Fs["fp64"]), 0, None) / sub[:, None])
        # planar emitters facing -z to FP32 precision: the reference's alignRayDirection
        # switches to its d = 0.5 branch there in FP32 but not in FP64, so the two
        # trace different (equally valid) rays and their rows differ statistically
        flip = flipped_rows(sc)
        keep = ~flip
        ferr = {"rays": int(sub.sum()),
                "max_abs_mixed_vs_fp64": float(np.max(np.abs(Fs["mixed"] - Fs["fp64"])[keep])) if keep.any() else None,
                "max_abs_plain_vs_fp64": float(np.max(np.abs(Fs["exact"] - Fs["fp64"])[keep])) if keep.any() else None,
                "max_abs_plain_fast_vs_fp64": float(np.max(np.abs(Fs["fast"] - Fs["fp64"])[keep])) if keep.any() else None,
                "max_binomial_sigma": float(sig.max()),
                "rows_excluded_minus_z_emitters": int(flip.sum()),
                "max_abs_mixed_vs_fp64_all_rows": float(np.max(np.abs(Fs["mixed"] - Fs["fp64"])))}

    # -- the reference's absolute EPS against a scale-relative one (furnace: the
    #    fibre's radius, 6.25e-5, is far below EPS = 1e-3)
    eps_cmp = None
    if args.workload == "furnace" and ferr is not None:
        tt = Tracer(precision=PREC_MIXED, key1=w.key1, device=local, eps=-1e-6)
        tt.set_scene(sc)
        Frel = tt.trace(sub)[1]
        tt.close()
        dF = np.abs(Frel - Fs["mixed"])
        i, j = np.unravel_index(int(np.argmax(dF)), dF.shape)
        eps_cmp = {"eps_relative": -1e-6, "max_abs_dF_vs_eps_1e-3": float(dF.max()),
                   "at": [int(i), int(j)], "F_eps_1e-3": float(Fs["mixed"][i, j]), "F_relative": float(Frel[i, j]),
                   "sigma": float(sig[i, j])}

    # -- CPU baseline -----------------------------------------------------
    cpu = None
    if rank == 0 and not args.no_cpu:
        rate, sample, nthreads, dt = cpu_rate(w, seconds=args.cpu_seconds)
        rate1, sample1, _, dt1 = cpu_rate(w, seconds=args.cpu_seconds / 3, threads=1)
        cpu = {"value": rate, "unit": "rays/s", "cores": nthreads, "kind": "port",
               "sample": f"{int(sample.sum())} rays of the workload, area-weighted, {dt:.1f} s",
               "single_thread": {"value": rate1, "unit": "rays/s", "cores": 1,
                                 "sample": f"{int(sample1.sum())} rays of the workload, area-weighted, {dt1:.1f} s"}}

    hbm_peak = None
    try:
        hbm_peak = float(json.loads((ROOT / "MEASURED_PEAKS.json").read_text())["hbm_gbs"])
    except (OSError, ValueError, KeyError):
        hbm_peak = None
    # DRAM bytes per launch of the timed kernel from an ncu capture of this workload
    # (profiles/traffic.json, key "<workload>:<precision>"); null when none was made
    traffic = None
    prof = ROOT / "profiles" / "traffic.json"
    if prof.exists() and args.surfaces == 64 and args.rays == 100_000_000:
        try:
            traffic = json.loads(prof.read_text()).get(f"{args.workload}:{args.precision}")
        except (ValueError, OSError):
            traffic = None

    kname = {"mixed": ("small-scene mixed-precision kernel (rf::mixed_small_kernel)" if mixed_small else
                       "batched mixed-precision persistent kernel (rf::batched_kernel)"),
             "exact": "plain bit-exact kernel (rf::trace_kernel<MExact>)",
             "fast": "plain FP32-approximation kernel (rf::trace_kernel<MFast>)"}[args.precision]
    line = {
        "metric": METRIC, "value": value, "unit": "rays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload_label(args),
                   "kernel": kname, "l2": "flushed between steps (256 MB write)",
                   "rays_per_step": total_rays * world,
                   "parallelism": ("one GPU" if world == 1 else
                                   f"{world} GPUs: ray ranges of each emitter's stream split on Philox draws, "
                                   "one int64 all_reduce of the tallies per step")},
        "e2e": {"value": world * total_rays / (float(np.mean(e2e_ms)) * 1e-3), "unit": "rays/s",
                "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "roofline": {"bound": "fp32-issue", "achieved": achieved / 1e12, "peak": peak_ops / 1e12,
                     "unit": "Top/s (FP32 ops performed, FMA = 1 op)", "frac": achieved / peak_ops,
                     "traffic": traffic,
                     "peak_source": "measured in-run: dependent-FMA issue probe (rf_measure_fp32_peak)",
                     # the brute-force work the rays represent (every ray against every
                     # surface, as the plain kernel does it) per second, against the same peak
                     "brute_force_equivalent_frac": ref_ops / (kernel_ms * 1e-3) / peak_ops,
                     # DRAM: the per-launch traffic from ncu over the kernel time, against
                     # the measured HBM copy bandwidth (the path does not use HBM)
                     "hbm": ({"achieved_gbs": traffic / (kernel_ms * 1e-3) / 1e9, "peak_gbs": hbm_peak,
                              "frac": traffic / (kernel_ms * 1e-3) / 1e9 / hbm_peak}
                             if traffic and hbm_peak else None)},
        "kernel_ms": kernel_ms,
        "launch": head_launch,
        "plain_kernel": plain,
        "speedup_vs_plain": (value / plain["value"]) if plain else None,
        "plain_kernel_fast": plain_fast,
        "speedup_vs_plain_fast": (value / plain_fast["value"]) if plain_fast else None,
        "culled_test_fraction": culled,
        "work_counts": [int(x) for x in work] if work is not None else None,
        "fp64_refined_tests": refined,
        "f_error": ferr,
        "eps_comparison": eps_cmp,
        "cpu_baseline": cpu,
        "clocks": clocks.summary(),
        "gpu_launches": args.steps,
    }
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def run_sweep(args):
    """Configuration 4: independent scenes with log-uniform surface counts and
    budgets, traced by one persistent launch per round of the graph-driven
    convergence loop until every row's binomial standard error is <= tol."""
    import torch

    from rayfactorcl_gb300 import _lib, generators
    from rayfactorcl_gb300.tracer import PREC_EXACT, PREC_FAST, PREC_MIXED, Tracer

    rank, world, local = dist_info()
    torch.cuda.set_device(local)
    ws = generators.batched_sweep(n_scenes=args.sweep_scenes, seed=4)
    scenes = [w.scene for w in ws]
    init = [w.rays for w in ws]
    with Tracer(precision=PREC_MIXED, device=local) as t:
        t.trace_batch(scenes[:2], init[:2])  # warm up
        torch.cuda.synchronize()
        with ClockSampler(local) as clocks:
            t0 = time.perf_counter()
            hits, F, rays, rounds = t.converge_batch(scenes, init, tol=args.sweep_tol,
                                                     round_rays=args.sweep_round, max_rounds=args.sweep_max_rounds)
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
        ms, launches = t.last_stats()
        refined = t.refined_count()
        # the plain kernel against the batched kernel on identical rays: every
        # 16th scene with 1/64 of its converged budgets
        sub = list(range(0, len(scenes), 16))
        sub_rays = [np.maximum(rays[i] // 64 // 4 * 4, 4) for i in sub]
        sub_scenes = [scenes[i] for i in sub]
        n_sub = int(sum(int(r.sum()) for r in sub_rays))
        t.trace_batch(sub_scenes, sub_rays)
        b_ms = t.last_stats()[0]
    # the plain kernel, bit-exact and with hardware approximations, each autotuned per
    # scene on these budgets
    p_ms = {PREC_EXACT: 0.0, PREC_FAST: 0.0}
    for sc, r in zip(sub_scenes, sub_rays):
        for prec in p_ms:
            with Tracer(precision=prec, device=local) as tp:
                tp.set_scene(sc)
                tp.trace(r)  # the budgets the autotuner tunes for
                tp.autotune()
                tp.trace(r)  # warm-up
                tp.trace(r)
                p_ms[prec] += tp.last_stats()[0]
    total = int(sum(int(r.sum()) for r in rays))
    worst = max(float(np.sqrt(np.clip(f * (1 - f), 0, None) / r[:, None]).max()) for f, r in zip(F, rays))
    line = {"metric": METRIC, "value": total / (ms * 1e-3), "unit": "rays/s", "n_gpus": 1, "steps": 1,
            "warmup": 1, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic",
            "config": {"workload": f"sweep of {len(scenes)} scenes, 10-400 surfaces (log-uniform), "
                                   f"budgets 1e5-1e7, convergence to std err <= {args.sweep_tol}",
                       "kernel": "batched mixed-precision persistent kernel in a CUDA-graph while loop"},
            "rays_total": total, "rounds": rounds, "max_std_err": worst, "wall_s": dt,
            "plain_subset": {"scenes": len(sub), "rays": n_sub, "surfaces": [int(sc.n) for sc in sub_scenes],
                             "batched_rays_per_s": n_sub / (b_ms * 1e-3),
                             "plain_rays_per_s": n_sub / (p_ms[PREC_EXACT] * 1e-3),
                             "speedup": p_ms[PREC_EXACT] / b_ms,
                             "plain_fast_rays_per_s": n_sub / (p_ms[PREC_FAST] * 1e-3),
                             "speedup_vs_plain_fast": p_ms[PREC_FAST] / b_ms},
            "gpu_launches": launches, "fp64_refined_tests": refined, "clocks": clocks.summary()}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="mixed", choices=["mixed", "exact", "fast"])
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--no-ferr", action="store_true")
    ap.add_argument("--ferr-div", type=int, default=10)
    ap.add_argument("--rays", type=int, default=100_000_000)
    ap.add_argument("--surfaces", type=int, default=64, help="surfaces of the mixed scene (same type mix)")
    ap.add_argument("--rays-per-thread", type=int, default=0, choices=[0, 4, 8])
    ap.add_argument("--tally-mode", type=int, default=0, choices=[0, 1, 2],
                    help="plain headline kernel: 1 shared-memory row histogram, 2 global atomics per ray "
                         "(as runGPU's atomic_inc, RayFactorGPU.cl:524); 0 autotuned")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--ref-seconds", type=float, default=4.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--workload", default="mixed64", choices=["mixed64", "sweep", *WORKLOADS])
    ap.add_argument("--sweep-scenes", type=int, default=256)
    ap.add_argument("--sweep-tol", type=float, default=1e-4)
    ap.add_argument("--sweep-round", type=int, default=1 << 26)
    ap.add_argument("--sweep-max-rounds", type=int, default=64)
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "sweep":
        return run_sweep(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
