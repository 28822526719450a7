"""The CPU oracle pinned against the reference's own code and exact rules."""
import json
import math

import numpy as np
import pytest

from helpers import GOLDEN, golden_scene, gen_scene
from oracle import oracle as O


def test_philox_matches_reference_header(oracle_lib):
    """Random123/philox.h (compiled from the reference) vs the oracle's Philox4x32-10."""
    kat = json.loads((GOLDEN / "philox_kat.json").read_text())
    assert len(kat) >= 100
    for row in kat:
        assert list(O.philox(row["ctr"], row["key"])) == row["out"], row


def test_reference_stream_value(oracle_lib):
    """ctr {1,f00dcafe,deadbeef,beeff00d}, key {0,decafbad} (RayFactorGPU.cl:486-497)."""
    out = O.philox([1, 0xF00DCAFE, 0xDEADBEEF, 0xBEEFF00D], [0, 0xDECAFBAD])
    assert [hex(int(v)) for v in out] == ["0xa9e1fa3", "0xbb160856", "0x266df5ba", "0x11ba516a"]
    u = O.uniforms(O.params(), 0, 0)
    expect = np.array([(int(v) >> 8) * 2.0 ** -24 for v in out], np.float32)
    assert np.array_equal(u, expect)


def test_default_streams_depend_on_emitter(oracle_lib):
    p = O.params(compat=0)
    a, b = O.uniforms(p, 0, 5), O.uniforms(p, 1, 5)
    assert not np.array_equal(a, b)
    pc = O.params(compat=O.COMPAT_STREAMS)
    assert np.array_equal(O.uniforms(pc, 0, 5), O.uniforms(pc, 1, 5))
    # the high word of the draw index reaches the counter outside compat mode
    assert not np.array_equal(O.uniforms(p, 3, 7), O.uniforms(p, 3, 7 + (1 << 32)))


def test_sincos_error_bound(oracle_lib):
    """Project-owned sin/cos on every argument the tracer can form: u * 2pi_f, u on the 24-bit grid."""
    u = (np.arange(1 << 24, dtype=np.float64) * 2.0 ** -24).astype(np.float32)
    x = (u * np.float32(2 * np.float32(np.pi))).astype(np.float32)
    s, c = O.sincos(x)
    xs = x.astype(np.float64)
    es = np.abs(s.astype(np.float64) - np.sin(xs))
    ec = np.abs(c.astype(np.float64) - np.cos(xs))
    # within two float ulps of |value|, and 1.2e-7 absolute near zero
    lim_s = np.maximum(2 * np.spacing(np.abs(np.sin(xs)).astype(np.float32)).astype(np.float64), 1.2e-7)
    lim_c = np.maximum(2 * np.spacing(np.abs(np.cos(xs)).astype(np.float32)).astype(np.float64), 1.2e-7)
    assert np.all(es <= lim_s), float(es.max())
    assert np.all(ec <= lim_c), float(ec.max())
    assert float(np.max(es)) < 1.2e-7 and float(np.max(ec)) < 1.2e-7


def _object_space(prim, p):
    im = prim["invm"].astype(np.float64).reshape(3, 4)
    return im[:, :3] @ p + im[:, 3]


@pytest.mark.parametrize("name", ["gen_mixed64", "input-C122", "input-C14", "input-C47", "input-C109"])
def test_emission_lies_on_surface(oracle_lib, name):
    sc = golden_scene(name)
    p = O.params(compat=0)
    for e in range(sc.n):
        pr = sc.primitives[e]
        t = int(pr["type"])
        cos_sum = 0.0
        K = 400
        for ray in range(K):
            s, c = O.emit_ray(sc.primitives, e, p, ray)
            q = _object_space(pr, s.astype(np.float64))
            scale = np.abs(sc.primitives[e]["m"].astype(np.float64)).max()
            tol = 2e-5 * max(1.0, scale)
            if t == 0:    # cylinder
                assert abs(math.hypot(q[0], q[1]) - 1) < 1e-4 and -1e-5 <= q[2] <= 1 + 1e-5
            elif t == 1:  # frustum
                rho = 1 + (pr["util1"] - 1) * q[2]
                assert abs(math.hypot(q[0], q[1]) - rho) < 1e-4 and -1e-5 <= q[2] <= 1 + 1e-5
            elif t == 2:
                assert abs(np.linalg.norm(q) - 1) < 1e-4
            elif t == 3:
                r2 = q[0] ** 2 + q[1] ** 2
                assert abs(q[2]) < tol and pr["util1"] - 1e-4 <= r2 <= pr["util2"] + 1e-4
            elif t == 4:
                assert abs(q[2]) < tol and abs(q[0]) <= 1 + 1e-5 and abs(q[1]) <= 1 + 1e-5
            elif t == 5:
                assert abs(q[2]) < tol and q[0] ** 2 + q[1] ** 2 <= 1 + 1e-4
            # RayFactorGPU.cl:87-97 divides by 1 + n.z: the rotated direction loses
            # accuracy for normals close to -z, as in the reference
            assert abs(np.linalg.norm(c) - 1) < 2e-3
            cos_sum += 1.0
        assert cos_sum == K


def test_cosine_weighting(oracle_lib):
    """Directions from a +z disc follow cos(theta): E[cos] = 2/3, E[cos^2] = 1/2."""
    sc = golden_scene("input-C47")
    p = O.params(compat=0)
    cs = np.array([O.emit_ray(sc.primitives, 0, p, r)[1][2] for r in range(20000)])
    assert np.all(cs >= 0)
    assert abs(cs.mean() - 2 / 3) < 0.01
    assert abs((cs ** 2).mean() - 0.5) < 0.01


def _ref_nthreads(rd, ns, wg=128):
    """main.cpp:172-173 in Python integers (int32 overflow -> None)."""
    prod = rd * ns
    if not (-(2 ** 31) <= prod < 2 ** 31):
        return None
    nt = int(prod / 4) if prod >= 0 else -int(-prod / 4)
    if nt < 0:
        return None
    rem = nt % wg
    return nt + wg - rem if rem > wg // 2 else nt - rem


@pytest.mark.parametrize("rd,ns", [(3, 1000000), (1, 256), (1, 257), (1, 255), (1, 64 * 4), (1, 65 * 4),
                                   (2, 1000), (7, 12345), (2147, 1000000), (0, 100)])
def test_ref_launch_size_rule(oracle_lib, rd, ns):
    got = O.ref_nthreads(rd, ns)
    exp = _ref_nthreads(rd, ns)
    assert got == (-1 if exp is None else exp)
    if exp is not None:
        assert got % 128 == 0


def test_ref_launch_size_ties_round_down(oracle_lib):
    assert O.ref_nthreads(1, 4 * (128 + 64)) == 128        # remainder 64 = wg/2 rounds down
    assert O.ref_nthreads(1, 4 * (128 + 65)) == 256
    assert O.ref_nthreads(3000, 1000000) == -1              # int32 overflow in main.cpp:172


def test_generated_scene_matches_reference_loader():
    for name in ["gen_enclosure3", "gen_mixed64", "gen_furnace", "gen_precision_stress"]:
        assert gen_scene(name).to_bytes() == golden_scene(name).to_bytes()


# --- per-ray pin to the reference's own kernel source ------------------------
# tests/golden/ref_kernel_rays.npz holds the first hit of every ray that the
# reference's RayFactorGPU.cl (runGPU :481-527, runBVGPU :530-626), compiled as
# host C++ by oracle/build.py, traced for two windows of work-items of every
# emitter of all 18 fixture scenes.  Streams, sphere discriminant and stale
# bounding-surface index are the reference's (RF_COMPAT_ALL).

def _ref_rays():
    data = np.load(GOLDEN / "ref_kernel_rays.npz")
    return {k: data[k] for k in data.files}


def _oracle_rows(sc, use_bv, lib_=None):
    rows = []
    for e in range(sc.n):
        rows.append(np.concatenate([O.trace_rays(sc, O.params(use_bv=use_bv), e, a, b, lib_=lib_)
                                    for a, b in O.window_rays()]))
    return np.stack(rows)


def test_reference_kernel_fixture_covers_every_scene():
    from helpers import SAMPLE_NAMES, GEN_NAMES
    ref = _ref_rays()
    for name in SAMPLE_NAMES + GEN_NAMES:
        assert f"{name}:runGPU" in ref
        if golden_scene(name).bounding_volumes.shape[0]:
            assert f"{name}:runBVGPU" in ref
    hit = np.concatenate([v.ravel() for v in ref.values()])
    assert hit.size > 100000 and 0.3 < float(np.mean(hit >= 0)) < 0.95


def test_oracle_equals_reference_kernel_per_ray(oracle_lib):
    """Every ray of the fixture: the oracle's first hit equals the reference kernel's."""
    for key, want in _ref_rays().items():
        name, kernel = key.split(":")
        got = _oracle_rows(golden_scene(name), kernel == "runBVGPU")
        assert np.array_equal(got, want), (key, int((got != want).sum()))


def test_planted_oracle_mistake_is_caught(oracle_lib, tmp_path):
    """A convention slip that keeps the statistics -- discRay's point with sin and
    cos swapped (RayFactorGPU.cl:304-309) -- fails the per-ray pin."""
    from oracle import build as B
    bad = O.load_variant(B.build_oracle_variant(tmp_path / "librf_oracle_planted.so",
                                                ["RFO_PLANTED_DISC_SWAP"]))
    ref = _ref_rays()
    sc = golden_scene("gen_enclosure3")  # two disc emitters
    got = _oracle_rows(sc, False, lib_=bad)
    want = ref["gen_enclosure3:runGPU"]
    disc_rows = [e for e in range(sc.n) if int(sc.primitives[e]["type"]) == 5]
    assert disc_rows and not np.array_equal(got[disc_rows], want[disc_rows])
    other = [e for e in range(sc.n) if e not in disc_rows]
    assert np.array_equal(got[other], want[other])


def test_oracle_equals_compiled_reference_kernel_more_rays(oracle_lib):
    """Wider windows straight against the reference kernel compiled here (needs the
    reference checkout; the committed fixture above covers the rest)."""
    from oracle import build as B
    if not B.reference_present():
        pytest.skip("reference checkout not present")
    B.build_ref()
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", GOLDEN / "make_golden.py")
    MG = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(MG)
    from helpers import SAMPLE_NAMES, GEN_NAMES
    lib = MG.load_ref_kernel()
    rng = np.random.default_rng(5)
    for name in SAMPLE_NAMES + GEN_NAMES:
        sc = golden_scene(name)
        g0 = int(rng.integers(8, 1 << 30))
        windows = ((g0, g0 + 24),)
        for use_bv in ([0, 1] if sc.bounding_volumes.shape[0] else [0]):
            want = MG.ref_kernel_rays(lib, sc, use_bv, windows)
            got = np.stack([O.trace_rays(sc, O.params(use_bv=use_bv), e, 4 * g0, 4 * (g0 + 24))
                            for e in range(sc.n)])
            assert np.array_equal(got, want), (name, use_bv, int((got != want).sum()))
