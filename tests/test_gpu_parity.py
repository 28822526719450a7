"""GPU parity: the CUDA library (through its C ABI) against the CPU oracle.

EXACT mode must reproduce the oracle's per-ray first-hit indices and integer
tallies bit for bit; FAST and FP64 modes are compared ray by ray with the
disagreements (grazing rays) counted and bounded.
"""
import numpy as np
import pytest

from helpers import GEN_NAMES, SAMPLE_NAMES, binom_sigma, gen_scene, golden_scene
from oracle import oracle as O
from rayfactorcl_gb300 import analytic
from rayfactorcl_gb300 import _lib
from rayfactorcl_gb300.tracer import PREC_EXACT, PREC_FAST, PREC_FP64, Tracer

pytestmark = pytest.mark.gpu

COMPATS = [0, _lib.COMPAT_ALL]


def _tracer(scene, **kw):
    t = Tracer(**kw)
    t.set_scene(scene)
    return t


def _emitters(n, k=6):
    if n <= k:
        return list(range(n))
    return sorted(set([0, 1, n // 3, n // 2, n - 2, n - 1]))


@pytest.mark.parametrize("compat", COMPATS)
@pytest.mark.parametrize("name", SAMPLE_NAMES + GEN_NAMES)
def test_exact_per_ray_hits(built_lib, oracle_lib, name, compat):
    sc = golden_scene(name)
    use_bv = bool(sc.use_bounding_volumes)
    nray = 4096 if sc.n < 100 else 1024
    p = O.params(compat=compat, use_bv=use_bv)
    with _tracer(sc, precision=PREC_EXACT, compat=compat) as t:
        for e in _emitters(sc.n):
            for first in (0, 4093):  # an unaligned start splits a Philox draw
                got = t.trace_rays(e, first, nray, use_bv=use_bv)
                exp = O.trace_rays(sc, p, e, first, first + nray)
                bad = np.nonzero(got != exp)[0]
                assert bad.size == 0, (name, e, first, bad[:8], got[bad[:8]], exp[bad[:8]])


def test_exact_per_ray_equals_reference_kernel(built_lib):
    """The CUDA kernels against the reference's own kernel source directly: every
    ray of tests/golden/ref_kernel_rays.npz (RayFactorGPU.cl's runGPU and runBVGPU
    compiled as host C++, two windows of work-items of every emitter of all 18
    fixture scenes, RF_COMPAT_ALL) has the same first hit in the EXACT kernel."""
    data = np.load(O.GOLDEN / "ref_kernel_rays.npz")
    assert len(data.files) >= 21
    for key in data.files:
        name, kernel = key.split(":")
        sc = golden_scene(name)
        use_bv = kernel == "runBVGPU"
        want = data[key]
        with _tracer(sc, precision=PREC_EXACT, compat=_lib.COMPAT_ALL) as t:
            for e in range(sc.n):
                got = np.concatenate([t.trace_rays(e, a, b - a, use_bv=use_bv) for a, b in O.window_rays()])
                assert np.array_equal(got, want[e]), (key, e, np.nonzero(got != want[e])[0][:8])


@pytest.mark.parametrize("compat", COMPATS)
@pytest.mark.parametrize("name", ["gen_enclosure3", "gen_mixed64", "input-C52-BV", "input-furnace",
                                  "gen_furnace", "input-C122", "gen_sweep0"])
def test_exact_tallies(built_lib, oracle_lib, name, compat):
    """Integer tallies equal the oracle's for uneven budgets (including 0 and non-multiples of 4)."""
    sc = golden_scene(name)
    use_bv = bool(sc.use_bounding_volumes)
    rng = np.random.default_rng(7)
    per = 20000 if sc.n < 100 else 600
    rays = rng.integers(0, per, sc.n).astype(np.int64)
    rays[0] = 0
    if sc.n > 2:
        rays[1] = 4 * 257 + 3
    p = O.params(compat=compat, use_bv=use_bv)
    exp = O.tally(sc, p, rays)
    for gpt, order in ((4, 1), (8, 1), (4, 2), (8, 2)):  # rays together / one ray at a time
        with _tracer(sc, precision=PREC_EXACT, compat=compat, rays_per_thread=gpt, test_order=order) as t:
            hits, F = t.trace(rays, use_bv=use_bv)
        assert np.array_equal(hits, exp), (name, gpt, order, np.argwhere(hits != exp)[:5])
        assert np.isnan(F[0]).all()
        nz = rays > 0
        assert np.allclose(F[nz], exp[nz] / rays[nz, None], rtol=0, atol=0)


@pytest.mark.parametrize("name", ["gen_mixed64", "input-furnace", "gen_precision_stress", "input-C122"])
def test_fast_mode_grazing_disagreements(built_lib, oracle_lib, name):
    """Hardware approximations change only rays that graze an edge."""
    sc = golden_scene(name)
    p = O.params(compat=0)
    total = bad = 0
    with _tracer(sc, precision=PREC_FAST) as t:
        for e in _emitters(sc.n):
            got = t.trace_rays(e, 0, 4096)
            exp = O.trace_rays(sc, p, e, 0, 4096)
            total += got.size
            bad += int(np.count_nonzero(got != exp))
    limit = 0.02 if name == "gen_precision_stress" else 0.002
    assert bad / total <= limit, (bad, total)


@pytest.mark.parametrize("name", ["gen_mixed64", "input-W100", "gen_precision_stress"])
def test_fp64_tracer_matches_oracle_fp64(built_lib, oracle_lib, name):
    sc = golden_scene(name)
    p = O.params(compat=0)
    total = bad = 0
    with _tracer(sc, precision=PREC_FP64) as t:
        for e in _emitters(sc.n):
            got = t.trace_rays(e, 0, 2048)
            exp = O.trace_rays(sc, p, e, 0, 2048, f64=True)
            total += got.size
            bad += int(np.count_nonzero(got != exp))
    assert bad / total <= 1e-3, (bad, total)


def test_run_gpurng_reference_budgets(built_lib, oracle_lib):
    """runCL_GPURNG budgets (main.cpp:172-173) with and without the emitter-0 quirk."""
    sc = golden_scene("input-C122")
    with _tracer(sc, compat=_lib.COMPAT_ALL) as t:
        rays, hits, F = t.run_gpurng(4000)
    exp_threads = [O.ref_nthreads(int(sc.primitives[0]["rayDensity"]), 4000)] * sc.n
    assert list(rays) == [4 * x for x in exp_threads]
    exp = O.tally(sc, O.params(), rays)
    assert np.array_equal(hits, exp)
    with _tracer(sc, compat=0) as t:
        rays0, _, _ = t.run_gpurng(4000)
    assert list(rays0) == [4 * O.ref_nthreads(int(r), 4000) for r in sc.primitives["rayDensity"]]


def test_enclosure_analytic_large(built_lib):
    """1e8 rays per surface of the 3-surface enclosure: F vs the closed form, the
    summation rule and reciprocity, FP64 normalisation on the GPU."""
    sc = gen_scene("gen_enclosure3")
    n = 100_000_000
    with _tracer(sc, precision=PREC_EXACT, key1=1) as t:
        hits, F = t.trace(np.full(3, n))
        a = np.array([np.pi * 0.25, np.pi * 0.25, np.pi])
        sum_err, recip = t.check_F(F, a)
    ref = analytic.enclosure3()
    sig = binom_sigma(ref, n)
    # EPS = 1e-3 (RayFactorGPU.cl:7) drops hits closer than 1e-3 to the origin: near
    # the rim about 1e-3 of the rays escape, a bias the tolerance allows for.
    assert np.all(np.abs(F - ref) <= 5 * sig + 1.5e-3), F - ref
    assert abs(F[0, 1] - ref[0, 1]) < 5 * sig[0, 1] + 3e-4
    assert sum_err < 2.5e-3
    assert recip < 0.01
    assert hits.sum() <= 3 * n


def test_large_budget_crosses_32bit_draws(built_lib, oracle_lib):
    """Draw indices past 2^32 use the counter's high word outside compat mode."""
    sc = golden_scene("input-C47")
    first = (1 << 34) - 2048 + 1
    p = O.params(compat=0)
    with _tracer(sc) as t:
        got = t.trace_rays(0, first, 8192)
    exp = O.trace_rays(sc, p, 0, first, first + 8192)
    assert np.array_equal(got, exp)


def test_compat_streams_limit(built_lib):
    sc = golden_scene("input-C47")
    with _tracer(sc, compat=_lib.COMPAT_STREAMS) as t:
        with pytest.raises(_lib.RfError) as ei:
            t.trace([(4 << 32) + 4, 0])
        assert ei.value.status == 6


def test_invalid_scenes_rejected(built_lib):
    sc = golden_scene("input-C47")
    with Tracer() as t:
        bad = sc.primitives.copy()
        bad[1]["type"] = 6
        with pytest.raises(_lib.RfError) as ei:
            t.set_scene(type(sc)(1e6, False, bad, sc.bounding_volumes))
        assert ei.value.status == 2
        bad = sc.primitives.copy()
        bad[0]["invm"][3] = np.nan
        with pytest.raises(_lib.RfError):
            t.set_scene(type(sc)(1e6, False, bad, sc.bounding_volumes))
        bv = golden_scene("input-C52-BV")
        bvs = bv.bounding_volumes.copy()
        bvs[0]["objEndIndex"] = 99
        with pytest.raises(_lib.RfError):
            t.set_scene(type(sc)(1e6, True, bv.primitives, bvs))
        with pytest.raises(_lib.RfError) as ei:
            t.trace([1, 1])
        assert ei.value.status == 9  # no scene
        t.set_scene(sc)
        with pytest.raises(_lib.RfError) as ei:
            t.trace([-4, 4])
        assert ei.value.status == 1
        with pytest.raises(_lib.RfError) as ei:
            t.trace([4, 4], use_bv=True)
        assert ei.value.status == 9


def test_single_primitive_and_empty_budgets(built_lib, oracle_lib):
    sc = golden_scene("input-uni")
    assert sc.n == 1
    with _tracer(sc) as t:
        hits, F = t.trace([0])
        assert hits.sum() == 0 and np.isnan(F).all()
        hits, F = t.trace([4001])
    exp = O.tally(sc, O.params(compat=0), np.array([4001]))
    assert np.array_equal(hits, exp)


@pytest.mark.parametrize("name,prec", [("gen_mixed64", PREC_EXACT), ("gen_furnace", PREC_EXACT),
                                       ("gen_sweep0", PREC_FAST)])
def test_autotune_keeps_results(built_lib, tmp_path, name, prec):
    """Every launch shape the autotuner may pick gives the same tallies; the choice is
    cached in memory and in the file."""
    sc = golden_scene(name)
    use_bv = bool(sc.use_bounding_volumes)
    rays = np.full(sc.n, 2000 if sc.n < 100 else 300, np.int64)
    with _tracer(sc, precision=prec) as t:
        ref, _ = t.trace(rays, use_bv=use_bv)
    cache = tmp_path / "tune.txt"
    with _tracer(sc, precision=prec) as t:
        cfg = t.autotune(use_bv=use_bv, cache_path=cache)
        got, _ = t.trace(rays, use_bv=use_bv)
    assert np.array_equal(got, ref)
    assert cfg["block"] in (128, 256) and cfg["rays_per_thread"] in (4, 8)
    lines = cache.read_text().splitlines()
    assert len(lines) == 1 and "|" in lines[0]
    with _tracer(sc, precision=prec) as t2:
        assert t2.autotune(use_bv=use_bv, cache_path=cache) == cfg
    assert len(cache.read_text().splitlines()) == 1  # served from the cache


@pytest.mark.parametrize("prec", [PREC_EXACT, PREC_FAST, "mixed"])
def test_split_and_resumed_runs_equal_one_run(built_lib, prec):
    """Checkpoint after a third of the rays, resume in a new context: the tallies and F
    equal one uninterrupted run (streams depend only on emitter and ray index)."""
    from rayfactorcl_gb300.tracer import PREC_MIXED
    prec = PREC_MIXED if prec == "mixed" else prec
    sc = golden_scene("gen_mixed64")
    rays = np.full(sc.n, 30001, np.int64)
    rays[5] = 0
    with _tracer(sc, precision=prec) as t:
        full, Ffull = t.trace(rays)
    part = rays // 3
    with _tracer(sc, precision=prec) as t:
        t.trace_range(np.zeros(sc.n, np.int64), part)
        ck_hits, _ = t.results()
    with _tracer(sc, precision=prec) as t2:
        t2.set_tallies(ck_hits, part)
        t2.trace_range(part, rays - part, accumulate=True)
        hits, F = t2.results()
    assert np.array_equal(hits, full)
    nz = rays > 0
    assert np.array_equal(F[nz], Ffull[nz])


def test_sharded_ranges_sum_to_one_run(built_lib):
    from rayfactorcl_gb300.shard import shard_ranges
    sc = golden_scene("gen_sweep2")
    rays = np.arange(sc.n, dtype=np.int64) * 997 + 5
    with _tracer(sc) as t:
        full, _ = t.trace(rays)
    total = np.zeros_like(full)
    for r in range(3):
        first, count = shard_ranges(rays, r, 3)
        with _tracer(sc) as t:
            t.trace_range(first, count)
            total += t.results()[0]
    assert np.array_equal(total, full)


def test_smoothing_enforces_reciprocity_and_summation(built_lib):
    """FP64 post-processing on the device: reciprocity exact, rows of a closed
    enclosure sum to one, and the result is no further from the closed form."""
    from rayfactorcl_gb300.tracer import surface_areas
    sc = gen_scene("gen_enclosure3")
    a = surface_areas(sc)
    assert np.allclose(a, [np.pi * 0.25, np.pi * 0.25, np.pi], rtol=1e-6)
    n_rays = 2_000_000
    with _tracer(sc, key1=3) as t:
        _, F = t.trace(np.full(3, n_rays))
        Fs, it, res = t.smooth_F(F, a, closed=True)
        Fo, _, _ = t.smooth_F(F, a, closed=False)
    AF = a[:, None] * Fs
    assert np.max(np.abs(AF - AF.T)) < 1e-12
    assert np.max(np.abs(Fs.sum(axis=1) - 1)) < 1e-10 and res < 1e-10 and it >= 1
    AFo = a[:, None] * Fo
    assert np.max(np.abs(AFo - AFo.T)) < 1e-12
    ref = analytic.enclosure3()
    assert np.max(np.abs(Fs - ref)) <= np.max(np.abs(F - ref)) + 2e-4
