"""GPU tests of the batched mixed-precision kernel.

Its nearest hits come from FP32 approximations (FP64 for ill-conditioned
quadrics) after bounding-sphere culling of coherent ray packets, so rays are
compared with the oracles on identical streams and disagreements (grazing
rays) are counted and bounded; F is compared with the plain kernel, the
closed forms and the FP64 tracer.

The reference's frame alignment (RayFactorGPU.cl:87-97) is discontinuous at a
surface normal of exactly -z: FP32 rounds such a normal to n.z = -1 and takes
the d = 0.5 branch (direction -o), while FP64 keeps n.z = -1 + 4e-15 and rotates
by 180 degrees about x (direction (o.x, -o.y, -o.z)).  Both are valid cosine
distributions but differ ray by ray, so a ray counts as a disagreement only if
it matches neither the FP32 nor the FP64 restatement.
"""
import numpy as np
import pytest

from helpers import binom_sigma, gen_scene, golden_scene
from oracle import oracle as O
from rayfactorcl_gb300 import analytic
from rayfactorcl_gb300.tracer import PREC_EXACT, PREC_FP64, PREC_MIXED, Tracer

pytestmark = pytest.mark.gpu


def _tracer(scene, **kw):
    t = Tracer(**kw)
    t.set_scene(scene)
    return t


def faces_minus_z(prim) -> bool:
    """Planar surface whose world normal is -z to within float rounding."""
    if int(prim["type"]) not in (3, 4, 5):
        return False
    im = prim["invm"].astype(np.float64).reshape(3, 4)
    n = im[2, :3]
    return n[2] / np.linalg.norm(n) < -0.99999


@pytest.mark.parametrize("name", ["gen_mixed64", "input-furnace", "input-W100", "gen_sweep0",
                                  "input-C122", "input-C14", "input-C47", "input-C109", "gen_enclosure3"])
def test_mixed_per_ray_vs_oracles(built_lib, oracle_lib, name):
    sc = golden_scene(name)
    p = O.params(compat=0)
    total = bad = 0
    emitters = sorted(set([0, sc.n // 2, sc.n - 1]))
    with _tracer(sc, precision=PREC_MIXED) as t:
        for e in emitters:
            got = t.trace_rays(e, 0, 8192)
            e64 = O.trace_rays(sc, p, e, 0, 8192, f64=True)
            e32 = O.trace_rays(sc, p, e, 0, 8192)
            total += got.size
            bad += int(np.count_nonzero((got != e64) & (got != e32)))
    assert bad / total <= 2e-3, (bad, total)


def test_mixed_large_scene_through_l1(built_lib, oracle_lib):
    """A 600-surface scene: too large for the shared-memory tables (512) and row
    histogram (512), so records and spheres are read through L1 and tallies go
    to global atomics.  Per-ray hits agree with the oracles and a batch with a
    small scene equals the single-scene runs."""
    from rayfactorcl_gb300 import generators
    sc = generators.mixed_scene(seed=7, total_rays=4, counts=(150, 150, 112, 94, 94)).scene
    assert sc.n == 600
    p = O.params(compat=0)
    total = bad = 0
    with _tracer(sc, precision=PREC_MIXED) as t:
        for e in (0, 299, 599):
            got = t.trace_rays(e, 0, 4096)
            e64 = O.trace_rays(sc, p, e, 0, 4096, f64=True)
            e32 = O.trace_rays(sc, p, e, 0, 4096)
            total += got.size
            bad += int(np.count_nonzero((got != e64) & (got != e32)))
    assert bad / total <= 2e-3, (bad, total)
    small = golden_scene("gen_mixed64")
    rays = [np.full(sc.n, 5000, np.int64), np.full(small.n, 7000, np.int64)]
    with Tracer(precision=PREC_MIXED) as t:
        hits, _ = t.trace_batch([sc, small], rays)
    for s_id, (scn, r) in enumerate(zip([sc, small], rays)):
        with _tracer(scn, precision=PREC_MIXED, scene_id=s_id) as t1:
            h1, _ = t1.trace(r)
        assert np.array_equal(hits[s_id], h1)


@pytest.mark.parametrize("n", [12, 13])
def test_mixed_brute_force_boundary(built_lib, oracle_lib, n):
    """Scenes of up to 12 surfaces are traced without sorting or culling, larger
    ones through packets: both agree with the oracles ray by ray."""
    from rayfactorcl_gb300 import generators
    counts = (3, 3, 2, 2, n - 10)
    sc = generators.mixed_scene(seed=11 + n, total_rays=4, counts=counts).scene
    p = O.params(compat=0)
    total = bad = 0
    with _tracer(sc, precision=PREC_MIXED) as t:
        for e in range(0, n, 3):
            got = t.trace_rays(e, 0, 8192)
            e64 = O.trace_rays(sc, p, e, 0, 8192, f64=True)
            e32 = O.trace_rays(sc, p, e, 0, 8192)
            total += got.size
            bad += int(np.count_nonzero((got != e64) & (got != e32)))
    assert bad / total <= 2e-3, (bad, total)


def test_mixed_per_ray_ragged_ranges(built_lib, oracle_lib):
    """Ray ranges that start and end inside a Philox draw (4 rays) and inside a
    32768-ray chunk: every ray keeps its stream position."""
    sc = golden_scene("gen_mixed64")
    p = O.params(compat=0)
    with _tracer(sc, precision=PREC_MIXED) as t:
        for e, first, n in ((3, 5, 3001), (40, 32766, 7), (63, 65537, 40003)):
            got = t.trace_rays(e, first, n)
            e64 = O.trace_rays(sc, p, e, first, first + n, f64=True)
            e32 = O.trace_rays(sc, p, e, first, first + n)
            bad = int(np.count_nonzero((got != e64) & (got != e32)))
            assert bad <= max(2, 2e-3 * n), (e, first, n, bad)


def test_mixed_beats_fp32_on_far_offsets(built_lib, oracle_lib):
    """Unit surfaces 1e4 from the origin, thin annuli, 89.9 degree frusta: the
    mixed kernel (re-centred, FP64 for ill-conditioned roots) agrees with the
    FP64 tracer far better than plain FP32."""
    sc = golden_scene("gen_precision_stress")
    p = O.params(compat=0)
    bad_mixed = bad_exact = total = 0
    with _tracer(sc, precision=PREC_MIXED) as tm:
        for e in range(sc.n):
            if faces_minus_z(sc.primitives[e]):
                continue
            ref = O.trace_rays(sc, p, e, 0, 4096, f64=True)
            bad_mixed += int(np.count_nonzero(tm.trace_rays(e, 0, 4096) != ref))
            bad_exact += int(np.count_nonzero(O.trace_rays(sc, p, e, 0, 4096) != ref))
            total += ref.size
    assert bad_mixed / total < 1e-3, (bad_mixed, total)
    assert bad_mixed < bad_exact, (bad_mixed, bad_exact)


def test_stress_F_error_and_refinements(built_lib):
    """Precision-stress scene (thin annuli, 89.9 degree frusta, 1e4 from the origin):
    the cancellation-free discriminants leave almost no quadric test to FP64, and F
    matches the FP64 tracer on identical streams to 1e-4 (rows of -z emitters, which
    trace different rays in FP32 and FP64, excluded) while plain FP32 is far off."""
    sc = golden_scene("gen_precision_stress")
    keep = np.array([not faces_minus_z(pr) for pr in sc.primitives])
    rays = np.full(sc.n, 400_000, np.int64)
    with _tracer(sc, precision=PREC_MIXED) as t:
        _, Fm = t.trace(rays)
        refined = t.refined_count()
    with _tracer(sc, precision=PREC_FP64) as t:
        _, F64 = t.trace(rays)
    with _tracer(sc, precision=PREC_EXACT) as t:
        _, F32 = t.trace(rays)
    err_m = float(np.abs(Fm - F64)[keep].max())
    err_e = float(np.abs(F32 - F64)[keep].max())
    assert err_m <= 1e-4, err_m
    assert err_e > 10 * err_m, (err_e, err_m)
    assert refined <= 1e-4 * rays.sum(), refined


def test_mixed_tallies_equal_fp64_statistics(built_lib, oracle_lib):
    """Same streams: tallies of the mixed kernel differ from the FP64 tracer's only by
    the few grazing rays, far inside one standard error."""
    sc = golden_scene("gen_mixed64")
    rays = np.full(sc.n, 40_000, np.int64)
    with _tracer(sc, precision=PREC_MIXED) as t:
        hm, Fm = t.trace(rays)
        nref = t.refined_count()
    with _tracer(sc, precision=PREC_FP64) as t:
        h64, F64 = t.trace(rays)
    diff = np.abs(hm - h64).sum()
    assert diff <= 2e-3 * rays.sum(), diff
    assert np.all(np.abs(Fm - F64) <= binom_sigma(F64, rays[:, None]) + 1e-4)
    assert nref >= 0


def test_enclosure_mixed_analytic(built_lib):
    sc = gen_scene("gen_enclosure3")
    n = 50_000_000
    with _tracer(sc, precision=PREC_MIXED, key1=1) as t:
        hits, F = t.trace(np.full(3, n))
    ref = analytic.enclosure3()
    sig = binom_sigma(ref, n)
    assert np.all(np.abs(F - ref) <= 5 * sig + 1.5e-3), F - ref
    assert abs(F[0, 1] - ref[0, 1]) < 5 * sig[0, 1] + 3e-4


@pytest.mark.parametrize("prec", [PREC_EXACT, PREC_MIXED])
def test_scale_relative_eps(built_lib, prec):
    """The enclosure shrunk to 1e-4: under the reference's absolute EPS = 1e-3
    (RayFactorGPU.cl:7) every hit is nearer than EPS and is dropped; with a negative
    eps (relative to the scene's extent) the view factors are the closed-form ones,
    which do not depend on size."""
    from rayfactorcl_gb300 import generators
    sc = generators.enclosure3(size=1e-4).scene
    n = 2_000_000
    rays = np.full(3, n)
    with _tracer(sc, precision=prec, key1=1) as t:
        hits_abs, _ = t.trace(rays)
    with _tracer(sc, precision=prec, key1=1, eps=-1e-4) as t:
        _, F = t.trace(rays)
    assert hits_abs.sum() == 0
    ref = analytic.enclosure3()
    sig = binom_sigma(ref, n)
    assert np.all(np.abs(F - ref) <= 5 * sig + 1e-4), F - ref


def test_batch_equals_single_scene_runs(built_lib):
    """Scene s of a batch draws the streams of scene_id = s; each scene's tallies equal a
    single-scene mixed run with that scene_id, whatever the other scenes are."""
    names = ["gen_sweep1", "gen_enclosure3", "gen_mixed64", "gen_sweep2", "input-C47"]
    scenes = [golden_scene(n) for n in names]
    rng = np.random.default_rng(3)
    rays = [rng.integers(0, 30000, sc.n).astype(np.int64) for sc in scenes]
    with Tracer(precision=PREC_MIXED) as t:
        hits, F = t.trace_batch(scenes, rays)
    for s, (sc, r) in enumerate(zip(scenes, rays)):
        with _tracer(sc, precision=PREC_MIXED, scene_id=s) as t1:
            h1, F1 = t1.trace(r)
        assert np.array_equal(hits[s], h1), names[s]
        nz = r > 0
        assert np.allclose(F[s][nz], F1[nz])
        assert np.isnan(F[s][~nz]).all()


def test_convergence_loop(built_lib):
    """The graph-driven loop stops when every row's standard error is <= tol, and its
    tallies equal one batch trace with the final budgets (streams continue)."""
    scenes = [golden_scene("gen_enclosure3"), golden_scene("input-C52"), golden_scene("gen_sweep2")]
    init = [np.full(sc.n, 4096, np.int64) for sc in scenes]
    tol = 2e-3
    with Tracer(precision=PREC_MIXED) as t:
        hits, F, rays, rounds = t.converge_batch(scenes, init, tol=tol, round_rays=20480, max_rounds=64)
    assert 1 <= rounds < 16
    for sc, h, f, r in zip(scenes, hits, F, rays):
        assert np.all(r >= 4096)
        sig = np.sqrt(f * (1 - f) / r[:, None])
        assert np.all(sig.max(axis=1) <= tol + 1e-12)
        # rows are given what their estimate still needs (at most 20480 per round), so
        # a row ends near max_j F(1-F)/tol^2 rays instead of a whole round beyond it
        need = (f * (1 - f)).max(axis=1) / tol ** 2
        assert np.all(r % 4 == 0)
        assert np.all(r <= np.maximum(4096, 1.25 * need + 4096))
    with Tracer(precision=PREC_MIXED) as t:
        h2, F2 = t.trace_batch(scenes, rays)
    for a, b in zip(hits, h2):
        assert np.array_equal(a, b)


def test_batch_rejects_bad_input(built_lib):
    from rayfactorcl_gb300 import _lib
    sc = golden_scene("input-C47")
    with Tracer(precision=PREC_MIXED) as t:
        with pytest.raises(_lib.RfError):
            t.trace_batch([sc], [np.array([-4, 4])])
        bad = sc.primitives.copy()
        bad[0]["type"] = 9
        with pytest.raises(_lib.RfError) as ei:
            t.trace_batch([type(sc)(1e6, False, bad, sc.bounding_volumes)], [np.array([4, 4])])
        assert ei.value.status == 2
        with pytest.raises(_lib.RfError):
            t.converge_batch([sc], [np.array([4, 4])], tol=0.0, round_rays=4, max_rounds=2)
        # bounding-surface semantics: at most 64 bounding surfaces in the mixed kernel
        bv = golden_scene("input-C52-BV")
        many = np.concatenate([bv.bounding_volumes] * 33)  # 66 > 64
        t.set_scene(type(bv)(1e6, True, bv.primitives, many))
        with pytest.raises(_lib.RfError) as ei:
            t.trace([4, 4], use_bv=True)
        assert ei.value.status == 8
        # nearest hits are int16 in the kernel: scenes above 32767 surfaces are refused
        big = np.repeat(sc.primitives[:1], 32768)
        with pytest.raises(_lib.RfError) as ei:
            t.trace_batch([type(sc)(1e6, False, big, sc.bounding_volumes)], [np.zeros(32768, np.int64)])
        assert _lib.STATUS[ei.value.status] == "RF_ERR_OVERFLOW"


def test_mixed_far_offset_self_hits(built_lib, oracle_lib):
    """A planar emitter never sees itself.  At 1e4 from the origin the FP32 ray origins are
    1e-3 off the plane and plain FP32 reports self-hits; the re-centred mixed kernel does not."""
    sc = golden_scene("gen_precision_stress")
    rays = np.zeros(sc.n, np.int64)
    rays[:4] = 200_000  # the thin annuli
    with _tracer(sc, precision=PREC_MIXED) as t:
        hm, _ = t.trace(rays)
    with _tracer(sc, precision=PREC_FP64) as t:
        h64, _ = t.trace(rays)
    for e in range(4):
        assert hm[e, e] == 0 and h64[e, e] == 0


@pytest.mark.parametrize("name", ["gen_mixed64", "gen_furnace", "gen_sweep0"])
def test_mixed_results_independent_of_scheduling(built_lib, name):
    """A ray's result depends on the ray alone: the same budgets traced with
    different persistent grids (so chunks meet different blocks and packets form in
    a different order), with and without the work counters, give identical tallies;
    so do two runs in a row."""
    sc = golden_scene(name)
    rng = np.random.default_rng(3)
    rays = (rng.integers(1, 40000, sc.n) * 4 + rng.integers(0, 4, sc.n)).astype(np.int64)
    runs = []
    for grid, count in ((0, False), (0, False), (7, False), (61, True), (1, False)):
        with _tracer(sc, precision=PREC_MIXED, batched_grid=grid, work_counts=count) as t:
            hits, _ = t.trace(rays)
            runs.append(hits)
            w = t.work_counts()
            if count:
                assert int(w[:6].sum()) > 0 and int(w[7]) > 0 and int(w[6]) >= int(w[:6].sum()) // 32
            else:
                assert int(w.sum()) == 0
    for h in runs[1:]:
        assert np.array_equal(h, runs[0])


@pytest.mark.parametrize("name", ["gen_enclosure3", "input-C47", "input-C122", "gen_precision_stress"])
def test_small_scene_kernel_equals_batched(built_lib, name):
    """Single scenes of at most 16 surfaces take the small-scene kernel (the plain
    kernel's launch shape); the same scene as a one-scene batch takes the batched
    kernel.  Same emission, tests and per-ray resolution: identical tallies, with
    4 and 8 rays per thread."""
    sc = golden_scene(name)
    assert sc.n <= 16
    rng = np.random.default_rng(9)
    rays = (rng.integers(1, 300000, sc.n) * 4 + rng.integers(0, 4, sc.n)).astype(np.int64)
    with Tracer(precision=PREC_MIXED) as t:
        hb, _ = t.trace_batch([sc], [rays])
    for rpt in (4, 8):
        with _tracer(sc, precision=PREC_MIXED, rays_per_thread=rpt, work_counts=True) as t:
            hs, _ = t.trace(rays)
            w = t.work_counts()
        assert np.array_equal(hs, hb[0]), (name, rpt)
        planar = np.isin(sc.primitives["type"], (3, 4, 5))
        # every ray against every surface but a planar emitter itself
        assert int(w[:6].sum()) == int(np.sum(rays * (sc.n - planar)))


def test_mixed_autotune_keeps_results(built_lib):
    """rf_autotune times the small-scene and the batched kernel for a small scene
    and keeps the faster; tallies are the same either way."""
    sc = golden_scene("gen_enclosure3")
    rays = np.full(sc.n, 400_004, np.int64)
    with _tracer(sc, precision=PREC_MIXED) as t:
        h0, _ = t.trace(rays)
        t.autotune()
        h1, _ = t.trace(rays)
    assert np.array_equal(h0, h1)


@pytest.mark.parametrize("compat", [0, "all"])
@pytest.mark.parametrize("name", ["input-C14-BV", "input-C52-BV", "gen_furnace"])
def test_mixed_bounding_surfaces_per_ray(built_lib, oracle_lib, name, compat):
    """runBVGPU semantics (RayFactorGPU.cl:580-619) in the mixed kernel: per-ray hits
    against the FP32 and FP64 restatements of the bounding-surface walk, with and
    without the reference's quirks (stale child index, sphere discriminant, shared
    streams)."""
    from rayfactorcl_gb300 import _lib
    cpt = _lib.COMPAT_ALL if compat == "all" else 0
    sc = golden_scene(name)
    p = O.params(compat=cpt, use_bv=True)
    total = bad = 0
    emitters = sorted(set([0, sc.n // 3, sc.n // 2, sc.n - 1]))
    with _tracer(sc, precision=PREC_MIXED, compat=cpt) as t:
        for e in emitters:
            got = t.trace_rays(e, 3, 8192, use_bv=True)
            e64 = O.trace_rays(sc, p, e, 3, 8195, f64=True)
            e32 = O.trace_rays(sc, p, e, 3, 8195)
            total += got.size
            bad += int(np.count_nonzero((got != e64) & (got != e32)))
            assert (got >= 0).mean() > 0.05
    assert bad / total <= 2e-3, (bad, total)


def test_mixed_bounding_surfaces_tallies(built_lib):
    """Tallies of the mixed kernel with bounding surfaces against the exact kernel's
    runBVGPU on the same streams: apart from the rows of planar emitters facing -z
    (where FP32 and FP64 frames trace different, equally valid rays; module
    docstring), rays that differ are grazing ones; every row agrees to well within
    its binomial sigma."""
    sc = golden_scene("gen_furnace")
    rays = np.full(sc.n, 20_000, np.int64)
    with _tracer(sc, precision=PREC_MIXED) as t:
        hm, Fm = t.trace(rays, use_bv=True)
    with _tracer(sc, precision=PREC_EXACT) as t:
        he, Fe = t.trace(rays, use_bv=True)
    keep = np.array([not faces_minus_z(sc.primitives[e]) for e in range(sc.n)])
    assert keep.sum() > sc.n // 2
    diff = np.abs(hm.astype(np.int64) - he.astype(np.int64))[keep]
    assert int(diff.sum()) <= 2e-3 * 2 * rays[keep].sum()
    # sigma of the difference of two estimates of the same F (independent rays on
    # the -z rows), with a floor of one hit for cells neither run saw often
    Fbar = 0.5 * (Fm + Fe)
    sig = np.sqrt(2 * np.maximum(Fbar * (1 - Fbar), 1.0 / rays[:, None]) / rays[:, None])
    assert float(np.max(np.abs(Fm - Fe) / sig)) < 5


@pytest.mark.parametrize("name,use_bv", [("gen_furnace", True), ("gen_furnace", False), ("input-furnace", False),
                                         ("input-W100", False)])
def test_segment_stacks_per_ray(built_lib, oracle_lib, name, use_bv):
    """A segment stack (consecutive cylinders tiling one longer cylinder) is one
    cylinder test whose root names the ring: per ray it gives the ring that testing
    the rings one by one gives (split_stacks), but for roots within rounding of the
    rim between two rings, and it agrees with the oracles as the per-ring tests do.
    Emitters on the stack, at its ends and off it."""
    from rayfactorcl_gb300.tracer import segment_stacks
    sc = golden_scene(name)
    st = segment_stacks(sc, use_bv)
    assert st
    a, m = st[0]
    emitters = sorted(set([a, a + m // 2, a + m - 1, (a + m) % sc.n, sc.n - 1]))
    p = O.params(compat=0, use_bv=use_bv)
    total = diff = bad = on = 0
    with _tracer(sc, precision=PREC_MIXED) as t, _tracer(sc, precision=PREC_MIXED, split_stacks=True) as ts:
        for e in emitters:
            got = t.trace_rays(e, 0, 16384, use_bv=use_bv)
            ref = ts.trace_rays(e, 0, 16384, use_bv=use_bv)
            e64 = O.trace_rays(sc, p, e, 0, 16384, f64=True)
            e32 = O.trace_rays(sc, p, e, 0, 16384)
            total += got.size
            diff += int(np.count_nonzero(got != ref))
            bad += int(np.count_nonzero((got != e64) & (got != e32)))
            on += int(np.count_nonzero((got >= a) & (got < a + m)))
    assert on > total // 20
    assert diff <= max(3, 2e-4 * total), (diff, total)
    assert bad / total <= 2e-3, (bad, total)


def test_segment_stacks_cut_the_tests(built_lib):
    """On the furnace the 180 wall rings are one test instead of one per ring, and
    so are the 20 annuli of each end plate: far fewer cylinder and annulus tests,
    the same tallies to within the few rays on a rim between two wall rings."""
    sc = golden_scene("gen_furnace")
    rays = np.full(sc.n, 40_000, np.int64)
    res = {}
    for split in (False, True):
        with _tracer(sc, precision=PREC_MIXED, work_counts=True, split_stacks=split) as t:
            hits, _ = t.trace(rays, True)
            res[split] = (hits, t.work_counts())
    (h0, w0), (h1, w1) = res[False], res[True]
    assert int(w0[0]) * 4 < int(w1[0]) and int(w0[3]) * 2 < int(w1[3]), (w0, w1)
    assert int(np.abs(h0 - h1).sum()) <= max(10, 2e-4 * int(rays.sum()))


def _furnace_plus(k: int):
    """The furnace's surfaces (ring stacks and plates) followed by k surfaces of a
    random mixed scene: past 512 surfaces the kernel reads the tables through L1."""
    from rayfactorcl_gb300 import generators
    from rayfactorcl_gb300.scene import Scene
    fur = golden_scene("gen_furnace")
    extra = generators.mixed_scene(seed=21, total_rays=4, counts=(k // 4, k // 4, k // 6, k // 6, k - 2 * (k // 4) - 2 * (k // 6))).scene
    return Scene(primitives=np.concatenate([fur.primitives, extra.primitives]))


def test_segment_stacks_beyond_the_shared_memory_tables(built_lib, oracle_lib):
    """Ring stacks and plates in a 602-surface scene (tables read through L1, plate
    radii through __ldg): per ray against ring-by-ring and the oracles."""
    from rayfactorcl_gb300.tracer import segment_stacks
    sc = _furnace_plus(350)
    assert sc.n == 602 and segment_stacks(sc)[:3] == [(0, 180), (180, 20), (200, 20)]
    p = O.params(compat=0)
    total = diff = bad = 0
    with _tracer(sc, precision=PREC_MIXED) as t, _tracer(sc, precision=PREC_MIXED, split_stacks=True) as ts:
        for e in (0, 90, 185, 215, 240, 400, 601):
            got = t.trace_rays(e, 0, 8192)
            ref = ts.trace_rays(e, 0, 8192)
            e64 = O.trace_rays(sc, p, e, 0, 8192, f64=True)
            e32 = O.trace_rays(sc, p, e, 0, 8192)
            total += got.size
            diff += int(np.count_nonzero(got != ref))
            bad += int(np.count_nonzero((got != e64) & (got != e32)))
    assert diff <= max(3, 2e-4 * total), (diff, total)
    assert bad / total <= 2e-3, (bad, total)


def test_segment_stacks_in_batches_and_the_convergence_loop(built_lib):
    """Scenes with stacks in a batch (any position) equal their single-scene runs, and
    the graph-driven loop's tallies equal a batch trace with its final budgets."""
    scenes = [golden_scene("gen_mixed64"), golden_scene("input-W100"), golden_scene("gen_furnace")]
    rng = np.random.default_rng(5)
    rays = [rng.integers(0, 20000, sc.n).astype(np.int64) * 4 for sc in scenes]
    with Tracer(precision=PREC_MIXED) as t:
        hits, _ = t.trace_batch(scenes, rays)
    for s, (sc, r) in enumerate(zip(scenes, rays)):
        with _tracer(sc, precision=PREC_MIXED, scene_id=s) as t1:
            h1, _ = t1.trace(r)
        assert np.array_equal(hits[s], h1), s
    init = [np.full(sc.n, 4096, np.int64) for sc in scenes[1:]]
    with Tracer(precision=PREC_MIXED) as t:
        hc, F, final, rounds = t.converge_batch(scenes[1:], init, tol=4e-3, round_rays=8192, max_rounds=32)
    with Tracer(precision=PREC_MIXED) as t:
        h2, _ = t.trace_batch(scenes[1:], final)
    for a, b in zip(hc, h2):
        assert np.array_equal(a, b)


def _many_bounding_spheres(nbv: int):
    """nbv copies of the 3-surface enclosure on a grid, 3 apart, each under a sphere
    bounding surface (every other one checked immediately, settings = 1)."""
    from rayfactorcl_gb300.scene import BV_DTYPE, Scene
    enc = golden_scene("gen_enclosure3")
    prims, bvs = [], np.zeros(nbv, BV_DTYPE)
    for b in range(nbv):
        shift = 3.0 * np.array([b % 4, (b // 4) % 4, b // 16], np.float64)
        for pr in enc.primitives:
            q = pr.copy()
            m = q["m"].astype(np.float64).reshape(3, 4)
            im = q["invm"].astype(np.float64).reshape(3, 4)
            m[:, 3] += shift
            im[:, 3] -= im[:, :3] @ shift
            q["m"] = m.reshape(-1).astype(np.float32)
            q["invm"] = im.reshape(-1).astype(np.float32)
            prims.append(q)
        c = shift + np.array([0.0, 0.0, 0.5])
        r = 0.75
        inv = np.zeros((3, 4))
        inv[:, :3] = np.eye(3) / r
        inv[:, 3] = -c / r
        bvs[b]["invm"] = inv.reshape(-1).astype(np.float32)
        bvs[b]["type"] = 2  # sphere
        bvs[b]["settings"] = b % 2
        bvs[b]["objStartIndex"], bvs[b]["objEndIndex"] = 3 * b, 3 * b + 3
    return Scene(1e6, True, np.array(prims), bvs)


@pytest.mark.parametrize("nbv", [24, 64])
def test_mixed_many_bounding_surfaces_per_ray(built_lib, oracle_lib, nbv):
    """Up to 64 bounding surfaces (72 and 192 surfaces): the walk skips, warp by
    warp, the surfaces no ray of the packet can reach, and per ray it agrees with the
    FP32 and FP64 restatements of runBVGPU as with a few."""
    sc = _many_bounding_spheres(nbv)
    p = O.params(compat=0, use_bv=True)
    total = bad = hit = 0
    with _tracer(sc, precision=PREC_MIXED) as t:
        for e in (0, 3 * nbv // 3 + 1, 3 * nbv // 2 + 2, 3 * nbv - 1):
            got = t.trace_rays(e, 0, 8192, use_bv=True)
            e64 = O.trace_rays(sc, p, e, 0, 8192, f64=True)
            e32 = O.trace_rays(sc, p, e, 0, 8192)
            total += got.size
            hit += int(np.count_nonzero(got >= 0))
            bad += int(np.count_nonzero((got != e64) & (got != e32)))
    assert hit > total // 2  # closed enclosures: rays stay in their own
    assert bad / total <= 2e-3, (bad, total)
