"""ctypes binding of ``librayfactor_gb300.so`` (include/rayfactor_gb300.h).

Loading fails loudly when the library has not been built: the tracer has no
CPU path.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

import os

# RF_LIB_PATH selects another build of the library (for example one installed elsewhere)
LIB_PATH = Path(os.environ.get("RF_LIB_PATH", str(Path(__file__).resolve().parent / "librayfactor_gb300.so")))

RF_OK = 0
STATUS = {0: "RF_OK", 1: "RF_ERR_INVALID_ARG", 2: "RF_ERR_BAD_SCENE", 3: "RF_ERR_OOM",
          4: "RF_ERR_CUDA", 5: "RF_ERR_TIMEOUT", 6: "RF_ERR_OVERFLOW", 7: "RF_ERR_NO_DEVICE",
          8: "RF_ERR_UNSUPPORTED", 9: "RF_ERR_STATE"}

COMPAT_BUDGET = 1 << 0
COMPAT_SPHERE = 1 << 1
COMPAT_BV_STALE = 1 << 2
COMPAT_STREAMS = 1 << 3
COMPAT_ALL = COMPAT_BUDGET | COMPAT_SPHERE | COMPAT_BV_STALE | COMPAT_STREAMS

PREC_EXACT, PREC_FAST, PREC_MIXED, PREC_FP64 = 0, 1, 2, 3

# every symbol declared in include/rayfactor_gb300.h
EXPORTS = ("rf_config_default", "rf_create", "rf_destroy", "rf_last_error", "rf_status_string",
           "rf_abi_version", "rf_set_scene", "rf_trace", "rf_trace_async", "rf_read_results",
           "rf_last_trace_stats", "rf_stream", "rf_trace_rays", "rf_run_gpurng", "rf_ray_budgets",
           "rf_write_output_txt", "rf_trace_batch", "rf_converge_batch", "rf_check_F",
           "rf_autotune", "rf_last_refine_count", "rf_last_work_counts", "rf_measure_fp32_peak",
           "rf_trace_mixed_noalloc", "rf_get_launch_config", "rf_trace_range", "rf_set_tallies",
           "rf_surface_areas", "rf_budgets_by_area", "rf_budgets_by_density", "rf_smooth_F",
           "rf_segment_stacks")


class RfConfig(ctypes.Structure):
    _fields_ = [("struct_size", ctypes.c_uint32), ("compat", ctypes.c_uint32),
                ("precision", ctypes.c_uint32), ("key1", ctypes.c_uint32), ("eps", ctypes.c_float),
                ("device", ctypes.c_int32), ("block_size", ctypes.c_int32),
                ("rays_per_thread", ctypes.c_int32), ("scene_id", ctypes.c_uint32),
                ("tally_mode", ctypes.c_int32), ("table_mode", ctypes.c_int32),
                ("test_order", ctypes.c_int32), ("work_counts", ctypes.c_int32),
                ("batched_grid", ctypes.c_int32), ("split_stacks", ctypes.c_int32),
                ("reserved", ctypes.c_uint32)]


class RfSceneDesc(ctypes.Structure):
    _fields_ = [("prims", ctypes.c_void_p), ("n_prims", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("rays_per_emitter", ctypes.c_void_p)]


class RfError(RuntimeError):
    def __init__(self, status: int, msg: str = ""):
        self.status = status
        super().__init__(f"{STATUS.get(status, status)}: {msg}")


_lib = None


def load() -> ctypes.CDLL:
    """Load the library once; raise if it is missing (run build() first)."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        raise RuntimeError(f"{LIB_PATH.name} is not built; run rayfactorcl_gb300.build.build()")
    L = ctypes.CDLL(str(LIB_PATH))
    P, I32, I64, U32 = ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_uint32
    sig = {
        "rf_config_default": (None, [ctypes.POINTER(RfConfig)]),
        "rf_create": (ctypes.c_int, [ctypes.POINTER(P), ctypes.POINTER(RfConfig)]),
        "rf_destroy": (None, [P]),
        "rf_last_error": (ctypes.c_char_p, [P]),
        "rf_status_string": (ctypes.c_char_p, [ctypes.c_int]),
        "rf_abi_version": (I32, []),
        "rf_set_scene": (ctypes.c_int, [P, P, I32, P, I32]),
        "rf_trace": (ctypes.c_int, [P, P, I32, P, P]),
        "rf_trace_async": (ctypes.c_int, [P, P, I32]),
        "rf_read_results": (ctypes.c_int, [P, P, P]),
        "rf_stream": (P, [P]),
        "rf_last_trace_stats": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(I32)]),
        "rf_trace_rays": (ctypes.c_int, [P, I32, I64, I64, I32, P]),
        "rf_run_gpurng": (ctypes.c_int, [P, I32, I32, P, P, P]),
        "rf_ray_budgets": (ctypes.c_int, [P, I32, I32, U32, P]),
        "rf_write_output_txt": (ctypes.c_int, [ctypes.c_char_p, P, I32]),
        "rf_trace_batch": (ctypes.c_int, [P, P, I32, P, P]),
        "rf_converge_batch": (ctypes.c_int, [P, P, I32, ctypes.c_double, I64, I32, P, P, P, P]),
        "rf_check_F": (ctypes.c_int, [P, P, P, I32, ctypes.POINTER(ctypes.c_double),
                                      ctypes.POINTER(ctypes.c_double)]),
        "rf_autotune": (ctypes.c_int, [P, I32, ctypes.c_char_p]),
        "rf_get_launch_config": (ctypes.c_int, [P, P, P, P, P, P]),
        "rf_trace_range": (ctypes.c_int, [P, P, P, I32, I32]),
        "rf_set_tallies": (ctypes.c_int, [P, P, P]),
        "rf_surface_areas": (ctypes.c_int, [P, I32, P]),
        "rf_smooth_F": (ctypes.c_int, [P, P, P, I32, I32, P, ctypes.POINTER(I32), ctypes.POINTER(ctypes.c_double)]),
        "rf_budgets_by_area": (ctypes.c_int, [P, I32, I64, P]),
        "rf_budgets_by_density": (ctypes.c_int, [P, I32, P, I64, P]),
        "rf_segment_stacks": (ctypes.c_int, [P, I32, P, I32, P, P, I32, ctypes.POINTER(I32)]),
        "rf_last_refine_count": (ctypes.c_int, [P, ctypes.POINTER(ctypes.c_uint64)]),
        "rf_last_work_counts": (ctypes.c_int, [P, P]),
        "rf_measure_fp32_peak": (ctypes.c_int, [I32, ctypes.POINTER(ctypes.c_double)]),
        "rf_trace_mixed_noalloc": (ctypes.c_int, [P, I32, P, U32, U32, ctypes.c_float, P, P]),
    }
    for name, (res, args) in sig.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def ptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def check(status: int, ctx=None):
    if status != RF_OK:
        msg = ""
        if ctx is not None:
            raw = load().rf_last_error(ctx)
            msg = raw.decode() if raw else ""
        raise RfError(status, msg)
