"""ctypes front end of the C oracle (test infrastructure).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module; the product never does.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import build as _build

COMPAT_BUDGET = 1 << 0
COMPAT_SPHERE = 1 << 1
COMPAT_BV_STALE = 1 << 2
COMPAT_STREAMS = 1 << 3
COMPAT_ALL = COMPAT_BUDGET | COMPAT_SPHERE | COMPAT_BV_STALE | COMPAT_STREAMS
REF_KEY1 = 0xDECAFBAD


class Params(ctypes.Structure):
    _fields_ = [("compat", ctypes.c_uint32), ("key1", ctypes.c_uint32), ("eps", ctypes.c_float),
                ("use_bv", ctypes.c_int32), ("scene_id", ctypes.c_uint32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = _bind(ctypes.CDLL(str(_build.build_oracle())))
    return _lib


def _bind(L):
    P = ctypes.c_void_p
    L.rfo_philox4x32_10.argtypes = [P, P, P]
    L.rfo_sincosf_array.argtypes = [P, ctypes.c_int64, P, P]
    L.rfo_stream_uniforms.argtypes = [ctypes.POINTER(Params), ctypes.c_int32, ctypes.c_int64, P]
    L.rfo_emit_ray.argtypes = [P, ctypes.c_int32, ctypes.POINTER(Params), ctypes.c_int64, P, P]
    for name in ("rfo_trace_rays", "rfo_trace_rays_f64"):
        getattr(L, name).argtypes = [P, ctypes.c_int32, P, ctypes.c_int32, ctypes.POINTER(Params),
                                     ctypes.c_int32, ctypes.c_int64, ctypes.c_int64, P,
                                     ctypes.c_int32]
        getattr(L, name).restype = ctypes.c_int
    for name in ("rfo_tally", "rfo_tally_f64"):
        getattr(L, name).argtypes = [P, ctypes.c_int32, P, ctypes.c_int32, ctypes.POINTER(Params),
                                     ctypes.c_int32, ctypes.c_int64, P, ctypes.c_int32]
        getattr(L, name).restype = ctypes.c_int
    L.rfo_ref_nthreads.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]
    L.rfo_ref_nthreads.restype = ctypes.c_int64
    L.rfo_max_threads.restype = ctypes.c_int32
    return L


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(ctypes.c_void_p)


def params(compat: int = COMPAT_ALL, key1: int = REF_KEY1, eps: float = 1e-3,
           use_bv: bool = False, scene_id: int = 0) -> Params:
    return Params(compat, key1 & 0xFFFFFFFF, eps, 1 if use_bv else 0, scene_id & 0xFFFFFFFF)


def philox(ctr, key) -> np.ndarray:
    c = np.ascontiguousarray(ctr, np.uint32)
    k = np.ascontiguousarray(key, np.uint32)
    out = np.zeros(4, np.uint32)
    lib().rfo_philox4x32_10(_ptr(c), _ptr(k), _ptr(out))
    return out


def sincos(x: np.ndarray):
    x = np.ascontiguousarray(x, np.float32)
    s = np.empty_like(x)
    c = np.empty_like(x)
    lib().rfo_sincosf_array(_ptr(x), x.size, _ptr(s), _ptr(c))
    return s, c


def uniforms(p: Params, emitter: int, gid: int) -> np.ndarray:
    out = np.zeros(4, np.float32)
    lib().rfo_stream_uniforms(ctypes.byref(p), emitter, gid, _ptr(out))
    return out


def emit_ray(prims: np.ndarray, emitter: int, p: Params, ray: int):
    s = np.zeros(3, np.float32)
    c = np.zeros(3, np.float32)
    lib().rfo_emit_ray(_ptr(prims), emitter, ctypes.byref(p), ray, _ptr(s), _ptr(c))
    return s, c


def _tables(scene):
    prims = np.ascontiguousarray(scene.primitives)
    bvs = np.ascontiguousarray(scene.bounding_volumes)
    return prims, bvs


def trace_rays(scene, p: Params, emitter: int, ray_begin: int, ray_end: int,
               f64: bool = False, threads: int = 0, lib_=None) -> np.ndarray:
    prims, bvs = _tables(scene)
    out = np.full(ray_end - ray_begin, -7, np.int32)
    L = lib_ if lib_ is not None else lib()
    fn = L.rfo_trace_rays_f64 if f64 else L.rfo_trace_rays
    rc = fn(_ptr(prims), prims.shape[0], _ptr(bvs), bvs.shape[0], ctypes.byref(p), emitter,
            ray_begin, ray_end, _ptr(out), threads)
    if rc != 0:
        raise ValueError(f"oracle trace_rays failed ({rc})")
    return out


def tally(scene, p: Params, rays: np.ndarray, f64: bool = False, threads: int = 0,
          emitters=None) -> np.ndarray:
    """int64 N x N tally matrix, row e = rays[e] rays from emitter e."""
    prims, bvs = _tables(scene)
    n = prims.shape[0]
    hits = np.zeros((n, n), np.int64)
    fn = lib().rfo_tally_f64 if f64 else lib().rfo_tally
    for e in (range(n) if emitters is None else emitters):
        if int(rays[e]) <= 0:
            continue
        row = np.zeros(n, np.int64)
        rc = fn(_ptr(prims), n, _ptr(bvs), bvs.shape[0], ctypes.byref(p), e, int(rays[e]),
                _ptr(row), threads)
        if rc != 0:
            raise ValueError(f"oracle tally failed ({rc})")
        hits[e] = row
    return hits


def ref_nthreads(ray_density: int, n_samples: int, wg: int = 128) -> int:
    return int(lib().rfo_ref_nthreads(ray_density, n_samples, wg))


def max_threads() -> int:
    return int(lib().rfo_max_threads())


def load_variant(path) -> ctypes.CDLL:
    """Bind an oracle build made by build.build_oracle_variant (tests only)."""
    return _bind(ctypes.CDLL(str(path)))


# Per-ray fixture written by the reference's own kernel (tests/golden/make_golden.py)
REF_WINDOWS = ((0, 8), (1048573, 1048581))


def window_rays(windows=REF_WINDOWS):
    """(ray_begin, ray_end) of each work-item window of the per-ray fixture."""
    return [(4 * g0, 4 * g1) for g0, g1 in windows]


GOLDEN = Path(__file__).resolve().parent.parent / "tests" / "golden"
