"""GPU test of rf_trace_mixed_noalloc, the entry point for hosts that cannot let
a library allocate device memory (their GPU memory is already reserved in
their own pool, or a cudaMalloc's device-wide synchronisation would stall
them).  The test owns the only device buffer (the tally matrix, allocated
here by the test itself) and checks that two calls in a row, through the
C ABI, give exactly the tallies of the allocating rf_trace path with the same
mixed-precision kernel and streams; the second call also shows that the
shared scratch array is cleared between calls.  Further cases: a non-default
stream with the reference's streams (RF_COMPAT_STREAMS), a scale-relative
eps, the host-side size checks, and that a call leaves the device's free
memory and the caller's allocator untouched.  This file is collected last.
"""
import ctypes

import numpy as np
import pytest

from helpers import golden_scene
from rayfactorcl_gb300 import _lib
from rayfactorcl_gb300.scene import PRIM_DTYPE
from rayfactorcl_gb300.tracer import PREC_MIXED, REF_KEY1, Tracer

pytestmark = pytest.mark.gpu


def _noalloc(prims, rays, hits_dev_ptr, compat=0, key1=REF_KEY1, eps=1e-3, stream=None):
    L = _lib.load()
    return L.rf_trace_mixed_noalloc(_lib.ptr(prims), prims.shape[0], _lib.ptr(rays), compat, key1,
                                    ctypes.c_float(eps), ctypes.c_void_p(hits_dev_ptr),
                                    None if stream is None else ctypes.c_void_p(stream))


def _reference(sc, rays, compat=0, eps=1e-3):
    with Tracer(precision=PREC_MIXED, compat=compat, eps=eps) as t:
        t.set_scene(sc)
        ref, _ = t.trace(rays)
    return ref


def test_no_alloc_matches_allocating_path(built_lib):
    torch = pytest.importorskip("torch")
    sc = golden_scene("gen_mixed64")
    prims = np.ascontiguousarray(sc.primitives, PRIM_DTYPE)
    n = prims.shape[0]
    rng = np.random.default_rng(11)
    budgets = [rng.integers(0, 60000, n).astype(np.int64), np.full(n, 30001, np.int64)]
    hits_dev = torch.zeros(n * n, dtype=torch.int64, device="cuda:0")
    for rays in budgets:  # two calls in a row on the same scratch array
        status = _noalloc(prims, rays, hits_dev.data_ptr())
        assert status == _lib.RF_OK, _lib.STATUS.get(status)
        torch.cuda.synchronize()
        got = hits_dev.cpu().numpy().reshape(n, n)
        assert np.array_equal(got, _reference(sc, rays))
        assert got.sum() > 0


def test_no_alloc_on_a_caller_stream_with_reference_streams(built_lib):
    """A torch stream of the caller, the reference's stream words (RF_COMPAT_STREAMS)
    and a scale-relative eps: still the allocating path's tallies."""
    torch = pytest.importorskip("torch")
    sc = golden_scene("gen_furnace")
    prims = np.ascontiguousarray(sc.primitives, PRIM_DTYPE)
    n = prims.shape[0]
    rays = np.full(n, 4 * 3001, np.int64)
    rays[::7] = 0
    hits_dev = torch.zeros(n * n, dtype=torch.int64, device="cuda:0")
    st = torch.cuda.Stream()
    for compat, eps in ((_lib.COMPAT_STREAMS, 1e-3), (0, -1e-6)):
        with torch.cuda.stream(st):
            status = _noalloc(prims, rays, hits_dev.data_ptr(), compat=compat, eps=eps, stream=st.cuda_stream)
        assert status == _lib.RF_OK, _lib.STATUS.get(status)
        st.synchronize()
        got = hits_dev.cpu().numpy().reshape(n, n)
        assert np.array_equal(got, _reference(sc, rays, compat=compat, eps=eps)), (compat, eps)


def test_no_alloc_leaves_device_memory_alone(built_lib):
    """The property the entry point exists for: across a call (after the first,
    which loads the kernels), the device's free memory and the caller's torch
    allocator are unchanged."""
    torch = pytest.importorskip("torch")
    sc = golden_scene("gen_mixed64")
    prims = np.ascontiguousarray(sc.primitives, PRIM_DTYPE)
    n = prims.shape[0]
    rays = np.full(n, 200_000, np.int64)
    hits_dev = torch.zeros(n * n, dtype=torch.int64, device="cuda:0")
    assert _noalloc(prims, rays, hits_dev.data_ptr()) == _lib.RF_OK
    torch.cuda.synchronize()
    for _ in range(3):
        free0, _total = torch.cuda.mem_get_info()
        stats0 = torch.cuda.memory_stats()
        assert _noalloc(prims, rays, hits_dev.data_ptr()) == _lib.RF_OK
        torch.cuda.synchronize()
        free1, _total = torch.cuda.mem_get_info()
        stats1 = torch.cuda.memory_stats()
        assert free1 == free0
        for key in ("allocation.all.allocated", "segment.all.allocated", "reserved_bytes.all.current"):
            assert stats1.get(key, 0) == stats0.get(key, 0), key
    assert int(hits_dev.sum().item()) > 0


def test_no_alloc_rejects_oversized_and_bad_input(built_lib):
    torch = pytest.importorskip("torch")
    sc = golden_scene("gen_mixed64")
    big = np.ascontiguousarray(np.concatenate([sc.primitives] * 9), PRIM_DTYPE)  # 576 > 512 surfaces
    hits_dev = torch.zeros(4, dtype=torch.int64, device="cuda:0")
    rays = np.full(big.shape[0], 4, np.int64)
    assert _noalloc(big, rays, hits_dev.data_ptr()) == 6  # RF_ERR_OVERFLOW
    bad = np.ascontiguousarray(sc.primitives, PRIM_DTYPE).copy()
    bad[3]["type"] = 7
    assert _noalloc(bad, np.full(bad.shape[0], 4, np.int64), hits_dev.data_ptr()) == 2  # RF_ERR_BAD_SCENE
    good = np.ascontiguousarray(sc.primitives, PRIM_DTYPE)
    neg = np.full(good.shape[0], 4, np.int64)
    neg[0] = -4
    assert _noalloc(good, neg, hits_dev.data_ptr()) == 1  # RF_ERR_INVALID_ARG
    # budgets beyond the stream limits are refused on the host, before any launch
    huge = np.full(good.shape[0], 4, np.int64)
    huge[5] = (1 << 46) + 4
    assert _noalloc(good, huge, hits_dev.data_ptr()) == 6
    draws = np.full(good.shape[0], 4, np.int64)
    draws[2] = (4 << 32) + 4  # more than 2^32 draws with 32-bit stream keys
    assert _noalloc(good, draws, hits_dev.data_ptr(), compat=_lib.COMPAT_STREAMS) == 6
    assert _noalloc(good, np.full(good.shape[0], 4, np.int64), hits_dev.data_ptr(), eps=float("nan")) == 1
