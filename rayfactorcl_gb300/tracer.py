"""Host-side interface over the C ABI, mirroring the reference's host driver.

:func:`run_cl_gpurng` has the signature and the behaviour of
``runCL_GPURNG(int n_samples, Scene &scene)`` (RayFactorCL/main.cpp:54-272):
it sizes each emitter's ray budget (main.cpp:172-173), chooses the
bounding-surface kernel when the scene asks for it (main.cpp:68-75), traces,
normalises the tallies by the rays shot (main.cpp:178, 241-249) and writes
``output.txt`` (main.cpp:236-249).  :class:`Tracer` exposes the individual
steps.  All work runs in the CUDA library; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import _lib
from ._lib import (COMPAT_ALL, COMPAT_BUDGET, COMPAT_BV_STALE, COMPAT_SPHERE, COMPAT_STREAMS,  # noqa: F401
                   PREC_EXACT, PREC_FAST, PREC_MIXED, PREC_FP64, RfError, check, ptr)
from .scene import BV_DTYPE, PRIM_DTYPE, Scene

REF_KEY1 = 0xDECAFBAD


class Tracer:
    """One CUDA context (stream, device buffers) holding one scene."""

    def __init__(self, precision: int = PREC_EXACT, compat: int = 0, key1: int = REF_KEY1,
                 eps: float = 1e-3, device: int = 0, block_size: int = 0, rays_per_thread: int = 0,
                 scene_id: int = 0, tally_mode: int = 0, table_mode: int = 0, test_order: int = 0,
                 work_counts: bool = False, batched_grid: int = 0, split_stacks: bool = False):
        L = _lib.load()
        cfg = _lib.RfConfig()
        L.rf_config_default(ctypes.byref(cfg))
        cfg.compat = compat
        cfg.precision = precision
        cfg.key1 = key1 & 0xFFFFFFFF
        cfg.eps = eps
        cfg.device = device
        cfg.block_size = block_size
        cfg.rays_per_thread = rays_per_thread
        cfg.scene_id = scene_id & 0xFFFFFFFF
        cfg.tally_mode = tally_mode
        cfg.table_mode = table_mode
        cfg.test_order = test_order
        cfg.work_counts = 1 if work_counts else 0
        cfg.batched_grid = batched_grid
        cfg.split_stacks = 1 if split_stacks else 0
        h = ctypes.c_void_p()
        check(L.rf_create(ctypes.byref(h), ctypes.byref(cfg)))
        self._h = h
        self._L = L
        self.cfg = cfg
        self.precision = precision
        self.n = 0
        self.scene: Scene | None = None

    # -- lifetime --------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            self._L.rf_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, status):
        check(status, self._h)

    # -- scene -----------------------------------------------------------
    def set_scene(self, scene: Scene):
        prims = np.ascontiguousarray(scene.primitives, PRIM_DTYPE)
        bvs = np.ascontiguousarray(scene.bounding_volumes, BV_DTYPE)
        self._check(self._L.rf_set_scene(self._h, ptr(prims), prims.shape[0],
                                         ptr(bvs) if bvs.shape[0] else None, bvs.shape[0]))
        self.n = prims.shape[0]
        self.scene = scene

    # -- tracing ---------------------------------------------------------
    def _rays(self, rays) -> np.ndarray:
        r = np.asarray(rays, np.int64)
        if self.n and r.ndim == 0:
            r = np.broadcast_to(r, (self.n,))
        if self.n and r.shape != (self.n,):
            raise ValueError(f"rays_per_emitter needs {self.n} entries, got {r.shape}")
        return np.ascontiguousarray(r, np.int64)

    def trace(self, rays, use_bv: bool = False, want_F: bool = True):
        """Tally matrix (int64 n x n) and F (float64 n x n, or None)."""
        r = self._rays(rays)
        hits = np.zeros((self.n, self.n), np.uint64)
        F = np.zeros((self.n, self.n), np.float64) if want_F else None
        self._check(self._L.rf_trace(self._h, ptr(r), 1 if use_bv else 0, ptr(hits), ptr(F)))
        return hits.astype(np.int64), F

    def trace_async(self, rays, use_bv: bool = False):
        self._keep = self._rays(rays)
        self._check(self._L.rf_trace_async(self._h, ptr(self._keep), 1 if use_bv else 0))

    def trace_range(self, first_ray, count, use_bv: bool = False, accumulate: bool = False):
        """Trace rays [first, first+count) of every emitter into the running tallies."""
        f, c = self._rays(first_ray), self._rays(count)
        self._keep = (f, c)
        self._check(self._L.rf_trace_range(self._h, ptr(f), ptr(c), 1 if use_bv else 0,
                                           1 if accumulate else 0))

    def set_tallies(self, hits: np.ndarray, rays):
        """Restore a checkpoint (tallies and rays traced per emitter)."""
        h = np.ascontiguousarray(hits, np.uint64)
        r = self._rays(rays)
        self._check(self._L.rf_set_tallies(self._h, ptr(h), ptr(r)))

    def results(self):
        """(int64 tallies, F) of everything traced so far."""
        hits = np.zeros((self.n, self.n), np.uint64)
        F = np.zeros((self.n, self.n), np.float64)
        self._check(self._L.rf_read_results(self._h, ptr(hits), ptr(F)))
        return hits.astype(np.int64), F

    def read_results(self, hits: np.ndarray | None = None, F: np.ndarray | None = None):
        self._check(self._L.rf_read_results(self._h, ptr(hits), ptr(F)))
        return hits, F

    @property
    def stream_handle(self) -> int:
        """The context's cudaStream_t as an integer."""
        return int(self._L.rf_stream(self._h) or 0)

    def last_stats(self):
        ms = ctypes.c_double()
        launches = ctypes.c_int32()
        self._check(self._L.rf_last_trace_stats(self._h, ctypes.byref(ms), ctypes.byref(launches)))
        return ms.value, launches.value

    def trace_rays(self, emitter: int, first_ray: int, n_rays: int, use_bv: bool = False) -> np.ndarray:
        out = np.empty(n_rays, np.int32)
        self._check(self._L.rf_trace_rays(self._h, emitter, first_ray, n_rays, 1 if use_bv else 0,
                                          ptr(out)))
        return out

    def run_gpurng(self, n_samples: int, use_bv: bool = False):
        rays = np.zeros(self.n, np.int64)
        hits = np.zeros((self.n, self.n), np.uint64)
        F = np.zeros((self.n, self.n), np.float64)
        self._check(self._L.rf_run_gpurng(self._h, int(n_samples), 1 if use_bv else 0, ptr(rays),
                                          ptr(hits), ptr(F)))
        return rays, hits.astype(np.int64), F

    def autotune(self, use_bv: bool = False, cache_path: str | None = None):
        """Time the launch shapes of the current scene and keep the fastest."""
        self._check(self._L.rf_autotune(self._h, 1 if use_bv else 0,
                                        None if cache_path is None else str(cache_path).encode()))
        return self.launch_config()

    def launch_config(self) -> dict:
        v = [ctypes.c_int32() for _ in range(5)]
        self._check(self._L.rf_get_launch_config(self._h, *[ctypes.byref(x) for x in v]))
        return {"block": v[0].value, "rays_per_thread": v[1].value, "smem_hist": v[2].value,
                "smem_table": v[3].value, "one_ray_at_a_time": v[4].value}

    def refined_count(self) -> int:
        """Quadric tests re-evaluated in FP64 by the last mixed-precision run."""
        v = ctypes.c_uint64()
        self._check(self._L.rf_last_refine_count(self._h, ctypes.byref(v)))
        return int(v.value)

    def work_counts(self) -> np.ndarray:
        """[tests by type x6, cone tests, packets] of the last mixed-precision run."""
        out = np.zeros(8, np.uint64)
        self._check(self._L.rf_last_work_counts(self._h, ptr(out)))
        return out

    def _descs(self, scenes, rays_list):
        keep, descs = [], (_lib.RfSceneDesc * len(scenes))()
        for i, (sc, r) in enumerate(zip(scenes, rays_list)):
            prims = np.ascontiguousarray(sc.primitives, PRIM_DTYPE)
            rr = np.ascontiguousarray(np.broadcast_to(np.asarray(r, np.int64), (prims.shape[0],)), np.int64)
            keep += [prims, rr]
            descs[i].prims = prims.ctypes.data
            descs[i].n_prims = prims.shape[0]
            descs[i].rays_per_emitter = rr.ctypes.data
        return descs, keep

    def _split(self, scenes, flat):
        out, off = [], 0
        for sc in scenes:
            n = sc.primitives.shape[0]
            out.append(flat[off:off + n * n].reshape(n, n))
            off += n * n
        return out

    def trace_batch(self, scenes, rays_list):
        """One persistent launch over many scenes (mixed precision).  Lists of
        per-scene tally and F matrices."""
        descs, keep = self._descs(scenes, rays_list)
        tot = sum(int(sc.primitives.shape[0]) ** 2 for sc in scenes)
        hits = np.zeros(tot, np.uint64)
        F = np.zeros(tot, np.float64)
        self._check(self._L.rf_trace_batch(self._h, descs, len(scenes), ptr(hits), ptr(F)))
        del keep
        return self._split(scenes, hits.astype(np.int64)), self._split(scenes, F)

    def converge_batch(self, scenes, rays_list, tol: float, round_rays: int, max_rounds: int):
        """Add rays until every row's binomial standard error is <= tol (CUDA-graph
        loop on the device).  Returns (hits list, F list, rays list, rounds)."""
        descs, keep = self._descs(scenes, rays_list)
        tot = sum(int(sc.primitives.shape[0]) ** 2 for sc in scenes)
        nrows = sum(int(sc.primitives.shape[0]) for sc in scenes)
        hits = np.zeros(tot, np.uint64)
        F = np.zeros(tot, np.float64)
        rays = np.zeros(nrows, np.int64)
        rounds = ctypes.c_int32()
        self._check(self._L.rf_converge_batch(self._h, descs, len(scenes), float(tol), int(round_rays),
                                              int(max_rounds), ptr(hits), ptr(F), ptr(rays),
                                              ctypes.byref(rounds)))
        del keep
        rl, off = [], 0
        for sc in scenes:
            n = sc.primitives.shape[0]
            rl.append(rays[off:off + n].copy())
            off += n
        return self._split(scenes, hits.astype(np.int64)), self._split(scenes, F), rl, rounds.value

    def smooth_F(self, F: np.ndarray, areas: np.ndarray, closed: bool = True):
        """Reciprocity (and, for a closed enclosure, summation) enforced in FP64."""
        F = np.ascontiguousarray(F, np.float64)
        a = np.ascontiguousarray(areas, np.float64)
        out = np.zeros_like(F)
        it, res = ctypes.c_int32(), ctypes.c_double()
        self._check(self._L.rf_smooth_F(self._h, ptr(F), ptr(a), F.shape[0], 1 if closed else 0, ptr(out),
                                        ctypes.byref(it), ctypes.byref(res)))
        return out, it.value, res.value

    def check_F(self, F: np.ndarray, areas: np.ndarray | None = None):
        F = np.ascontiguousarray(F, np.float64)
        a = None if areas is None else np.ascontiguousarray(areas, np.float64)
        s, r = ctypes.c_double(), ctypes.c_double()
        self._check(self._L.rf_check_F(self._h, ptr(F), ptr(a), F.shape[0], ctypes.byref(s),
                                       ctypes.byref(r)))
        return s.value, r.value


def ray_budgets(scene: Scene, n_samples: int, compat: int = 0) -> np.ndarray:
    """main.cpp:172-173 budgets (rays, int64) for every emitter; no GPU needed."""
    L = _lib.load()
    prims = np.ascontiguousarray(scene.primitives, PRIM_DTYPE)
    out = np.zeros(prims.shape[0], np.int64)
    check(L.rf_ray_budgets(ptr(prims), prims.shape[0], int(n_samples), compat, ptr(out)))
    return out


def surface_areas(scene: Scene) -> np.ndarray:
    """FP64 area of every primitive under its transform (no GPU needed)."""
    prims = np.ascontiguousarray(scene.primitives, PRIM_DTYPE)
    out = np.zeros(prims.shape[0], np.float64)
    check(_lib.load().rf_surface_areas(ptr(prims), prims.shape[0], ptr(out)))
    return out


def budgets_by_area(scene: Scene, total_rays: int, use_density: bool = True) -> np.ndarray:
    """total_rays spread over the emitters by area, multiples of four; weighted by
    each primitive's <rayDensity> from the scene file when the scene has them."""
    prims = np.ascontiguousarray(scene.primitives, PRIM_DTYPE)
    out = np.zeros(prims.shape[0], np.int64)
    dens = getattr(scene, "density", None)
    if use_density and dens is not None and len(dens) == prims.shape[0]:
        d = np.ascontiguousarray(dens, np.float64)
        check(_lib.load().rf_budgets_by_density(ptr(prims), prims.shape[0], ptr(d), int(total_rays), ptr(out)))
    else:
        check(_lib.load().rf_budgets_by_area(ptr(prims), prims.shape[0], int(total_rays), ptr(out)))
    return out


def segment_stacks(scene: Scene, use_bv: bool = True) -> list[tuple[int, int]]:
    """(first surface, number of surfaces) of every segment stack the mixed
    kernels trace as one cylinder; with use_bv, none crosses a bounding
    surface's child range."""
    prims = np.ascontiguousarray(scene.primitives, PRIM_DTYPE)
    bvs = getattr(scene, "bounding_volumes", None)
    nb = len(bvs) if (use_bv and bvs is not None) else 0
    bv = np.ascontiguousarray(bvs, BV_DTYPE) if nb else None
    n = prims.shape[0]
    first = np.zeros(max(n, 1), np.int32)
    count = np.zeros(max(n, 1), np.int32)
    k = ctypes.c_int32()
    check(_lib.load().rf_segment_stacks(ptr(prims), n, ptr(bv) if nb else None, nb, ptr(first), ptr(count),
                                        first.shape[0], ctypes.byref(k)))
    return [(int(first[i]), int(count[i])) for i in range(k.value)]


def write_output_txt(path: str | Path, F: np.ndarray):
    """main.cpp:236-249 format: rows of '%.8g,' values."""
    F = np.ascontiguousarray(F, np.float64)
    check(_lib.load().rf_write_output_txt(str(path).encode(), ptr(F), F.shape[0]))


def run_cl_gpurng(n_samples: int, scene: Scene, output: str | Path | None = "output.txt",
                  stats: dict | None = None, **tracer_kw):
    """runCL_GPURNG(n_samples, scene) (main.cpp:54-272) on the GPU.

    Returns (rays per emitter, int64 tallies, F).  Writes ``output`` unless it is None.
    ``stats``, if given, receives the tracing kernel's time, its launch count and (mixed
    precision) the quadric tests re-evaluated in FP64.
    """
    with Tracer(**tracer_kw) as t:
        t.set_scene(scene)
        # runBVGPU when the scene asks for it (main.cpp:68-70), in every precision; the
        # mixed kernel takes up to 64 bounding surfaces over 512 surfaces (else an error)
        bvs = scene.bounding_volumes
        use_bv = bool(scene.use_bounding_volumes) and bvs is not None and len(bvs) > 0
        rays, hits, F = t.run_gpurng(n_samples, use_bv=use_bv)
        if stats is not None:
            ms, launches = t.last_stats()
            stats.update(kernel_ms=ms, launches=launches,
                         fp64_refined_tests=t.refined_count() if t.precision == PREC_MIXED else 0)
    if output is not None:
        write_output_txt(output, F)
    return rays, hits, F
