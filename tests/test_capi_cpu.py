"""The C ABI on the CPU: the library loads and exports everything the header
declares, the header compiles as C and C++ with the reference's struct sizes, the
integration shim compiles against the reference's own Scene.h, and the host-side
rules (budgets, output format, validation) behave as the reference does."""
import ctypes
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

from helpers import GEN_NAMES, SAMPLE_NAMES, golden_scene
from oracle import oracle as O
from rayfactorcl_gb300 import _lib
from rayfactorcl_gb300.scene import BV_DTYPE, PRIM_DTYPE, parse_scene_xml

ROOT = Path(__file__).resolve().parent.parent
HEADER = ROOT / "include" / "rayfactor_gb300.h"
from oracle.build import REFERENCE  # noqa: E402  (RF_REFERENCE_DIR, else ../reference)


def _declared():
    text = HEADER.read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(rf_[A-Za-z0-9_]+)\s*\(", text)))


def test_header_declares_exported_symbols(built_lib):
    declared = _declared()
    assert len(declared) >= 20
    L = ctypes.CDLL(str(built_lib))
    for name in declared:
        assert hasattr(L, name), name
    assert sorted(_lib.EXPORTS) == declared


def test_library_loads_without_gpu(built_lib):
    L = _lib.load()
    assert L.rf_abi_version() == 1
    assert L.rf_status_string(6) == b"size overflow"


def _compile(src: str, lang: str, tmp_path: Path, extra=()):
    f = tmp_path / ("t.c" if lang == "c" else "t.cpp")
    f.write_text(src)
    exe = tmp_path / "t"
    cc = "gcc" if lang == "c" else "g++"
    r = subprocess.run([cc, "-std=c11" if lang == "c" else "-std=c++17", "-Wall", "-Werror",
                        "-I", str(HEADER.parent), *extra, str(f), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout


@pytest.mark.parametrize("lang", ["c", "cpp"])
def test_header_compiles_with_reference_layouts(tmp_path, lang):
    src = """#include "rayfactor_gb300.h"
#include <stdio.h>
int main(void) { printf("%d %d %d", (int)sizeof(rf_primitive), (int)sizeof(rf_bounding_volume),
                        (int)sizeof(rf_config)); return 0; }
"""
    out = _compile(src, lang, tmp_path)
    assert out.split() == ["112", "72", str(ctypes.sizeof(_lib.RfConfig))]
    assert PRIM_DTYPE.itemsize == 112 and BV_DTYPE.itemsize == 72


SHIM_DIR = ROOT / "tests" / "shim"


def build_shim_program(out: Path, stub: bool, lib: Path) -> Path:
    """tests/shim/shim_main.cpp + include/rayfactor_gb300_shim.hpp linked with the
    library: with the reference's own Scene/TinyXML-2/affine sources (stub=False)
    or with the test stand-in tests/shim/scene_stub.h (stub=True)."""
    cmd = ["g++", "-std=c++17", "-O1", "-w", "-I", str(HEADER.parent), "-I", str(SHIM_DIR)]
    srcs = [str(SHIM_DIR / "shim_main.cpp")]
    if stub:
        cmd.append("-DRF_SHIM_SCENE_STUB")
    else:
        rfc = REFERENCE / "RayFactorCL"
        aff, txml = rfc / "Affine Transformation", rfc / "TinyXML-2"
        cmd += ["-I", str(rfc), "-I", str(aff), "-I", str(txml)]
        srcs += [str(rfc / "Scene.cpp"), str(txml / "tinyxml2.cpp"), str(aff / "AffineTransformation.cpp"),
                 str(aff / "Matrices.cpp")]
    cmd += ["-o", str(out), *srcs, "-L", str(lib.parent), "-lrayfactor_gb300",
            "-Wl,-rpath," + str(lib.parent)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return out


def _run_shim(exe: Path, scene_arg: Path, cwd: Path):
    return subprocess.run([str(exe), str(scene_arg)], capture_output=True, text=True, cwd=cwd, timeout=600)


def _gpu_present() -> bool:
    L = _lib.load()
    h = ctypes.c_void_p()
    st = L.rf_create(ctypes.byref(h), None)
    if st == 0:
        L.rf_destroy(h)
    return st == 0


def test_shim_links_with_reference_scene_loader(built_lib, tmp_path):
    """The drop-in for runCL_GPURNG (include/rayfactor_gb300_shim.hpp) compiled and
    linked with the reference's own Scene.cpp, TinyXML-2 and affine code and the
    library, then run as the reference's main() on a sample scene: it reads the XML
    with the reference loader and calls the C ABI.  Without a GPU the call must come
    back with the library's no-device error, not an exit or a crash."""
    rfc = REFERENCE / "RayFactorCL"
    if not (rfc / "Scene.cpp").exists():
        pytest.skip("reference checkout not present")
    exe = build_shim_program(tmp_path / "shim_ref", False, built_lib)
    r = _run_shim(exe, REFERENCE / "sample-geometries" / "input-C47.xml", tmp_path)
    if _gpu_present():
        assert r.returncode == 0 and (tmp_path / "output.txt").exists(), r.stderr
    else:
        assert r.returncode == 1 and "rayfactor_gb300: no CUDA device" in r.stderr, (r.returncode, r.stderr)
        assert not (tmp_path / "output.txt").exists()


def test_shim_builds_with_scene_stand_in(built_lib, tmp_path):
    """The same program with the test stand-in Scene (used by the GPU test where the
    reference checkout is absent) builds and reaches the C ABI."""
    exe = build_shim_program(tmp_path / "shim_stub", True, built_lib)
    r = _run_shim(exe, ROOT / "tests" / "golden" / "scenes" / "input-C47.bin", tmp_path)
    if _gpu_present():
        assert r.returncode == 0, r.stderr
    else:
        assert r.returncode == 1 and "no CUDA device" in r.stderr, r.stderr


def _budgets(sc, n_samples, compat):
    prims = np.ascontiguousarray(sc.primitives, PRIM_DTYPE)
    out = np.zeros(sc.n, np.int64)
    st = _lib.load().rf_ray_budgets(_lib.ptr(prims), sc.n, n_samples, compat, _lib.ptr(out))
    return st, out


@pytest.mark.parametrize("name", SAMPLE_NAMES + GEN_NAMES)
def test_ray_budgets_follow_reference_rule(built_lib, oracle_lib, name):
    """main.cpp:172-173 (+178): rays = round_to_128(rayDensity*n/4) * 4; with the
    compat flag every emitter uses emitter 0's rayDensity."""
    sc = golden_scene(name)
    for n_samples in (1000, 12345):
        st, got = _budgets(sc, n_samples, 0)
        exp = [O.ref_nthreads(int(r), n_samples) for r in sc.primitives["rayDensity"]]
        if min(exp) < 0:
            assert st == 6
            continue
        assert st == 0 and list(got) == [4 * e for e in exp]
        st, got = _budgets(sc, n_samples, _lib.COMPAT_BUDGET)
        e0 = O.ref_nthreads(int(sc.primitives["rayDensity"][0]), n_samples)
        assert st == 0 and np.all(got == 4 * e0)


def test_ray_budget_overflow_is_an_error(built_lib):
    sc = golden_scene("input-furnace")  # rayDensity up to 201: 2e7 samples overflow int32 (main.cpp:172)
    st, _ = _budgets(sc, 20_000_000, 0)
    assert st == 6


def test_output_txt_format(built_lib, tmp_path):
    """main.cpp:236-249 stores F as float and streams it with precision 8, a comma after
    every value: compare with the same values through a C++ ostream."""
    vals = [0.0, 0.171252, 1.0 / 3.0, 1e-9, 0.5, float("nan"), 123456789.0, 2.5e-5, 1.0]
    F = np.array(vals).reshape(3, 3)
    path = tmp_path / "output.txt"
    assert _lib.load().rf_write_output_txt(str(path).encode(), _lib.ptr(F), 3) == 0
    lits = ", ".join("NAN" if v != v else repr(v) for v in vals)
    src = """#include <cmath>
#include <iostream>
int main() { std::cout.precision(8); const double v[] = {%s};
  for (int i = 0; i < 3; ++i) { for (int j = 0; j < 3; ++j) std::cout << (float)v[3 * i + j] << ",";
                                std::cout << std::endl; } return 0; }
""" % lits
    expect = _compile(src, "cpp", tmp_path)
    assert path.read_text() == expect
    assert expect.splitlines()[0] == "0,0.171252,0.33333334,"


def test_create_without_gpu_or_with_bad_config(built_lib):
    L = _lib.load()
    cfg = _lib.RfConfig()
    L.rf_config_default(ctypes.byref(cfg))
    assert cfg.key1 == 0xDECAFBAD and abs(cfg.eps - 1e-3) < 1e-9 and cfg.compat == 0
    h = ctypes.c_void_p()
    bad = _lib.RfConfig.from_buffer_copy(cfg)
    bad.struct_size = 7
    assert L.rf_create(ctypes.byref(h), ctypes.byref(bad)) == 1
    bad = _lib.RfConfig.from_buffer_copy(cfg)
    bad.precision = 9
    assert L.rf_create(ctypes.byref(h), ctypes.byref(bad)) == 1
    bad = _lib.RfConfig.from_buffer_copy(cfg)
    bad.eps = float("nan")
    assert L.rf_create(ctypes.byref(h), ctypes.byref(bad)) == 1
    st = L.rf_create(ctypes.byref(h), ctypes.byref(cfg))
    if st == 0:
        L.rf_destroy(h)  # a GPU is present
    else:
        assert st == 7  # RF_ERR_NO_DEVICE: no CPU fallback


def test_scene_loader_edge_cases():
    # a comment as the first child of <settings>: the reference loop does not run
    xml = """<project><settings><!-- c --><globalRayDensity value="5" /></settings>
             <geometry><primitive type="disc"><scale x="1" y="1" z="1" /></primitive></geometry></project>"""
    sc = parse_scene_xml(xml)
    assert sc.global_ray_density == 0.0 and sc.n == 1
    with pytest.raises(ValueError):
        parse_scene_xml("<notaproject/>")
    with pytest.raises(ValueError):
        parse_scene_xml("""<project><settings><globalRayDensity value="5" /></settings>
            <geometry><primitive type="annulus"><smallRadius value="1" /></primitive></geometry></project>""")
    # unknown types are skipped, "true" and integers parse as booleans (tinyxml2.cpp:959-973)
    sc = parse_scene_xml("""<project><settings><useBoundingVolumes value="1" /></settings>
        <geometry><bv type="teapot"/></geometry></project>""")
    assert sc.use_bounding_volumes and sc.bounding_volumes.shape[0] == 0


def test_scene_bytes_roundtrip():
    for name in GEN_NAMES:
        sc = golden_scene(name)
        assert type(sc).from_bytes(sc.to_bytes()).to_bytes() == sc.to_bytes()


@pytest.mark.parametrize("name", SAMPLE_NAMES)
def test_loader_matches_reference_on_samples(name):
    xml = REFERENCE / "sample-geometries" / f"{name}.xml"
    if not xml.exists():
        pytest.skip("reference checkout not present")
    from rayfactorcl_gb300.scene import read_scene
    assert read_scene(xml).to_bytes() == golden_scene(name).to_bytes()


def test_cli_reports_missing_file(built_lib, tmp_path, capsys):
    from rayfactorcl_gb300.__main__ import main
    assert main([str(tmp_path / "missing.xml")]) == 1


def test_surface_areas_and_area_budgets(built_lib):
    import math
    from rayfactorcl_gb300 import generators
    from rayfactorcl_gb300.tracer import budgets_by_area, surface_areas
    for w in (generators.enclosure3(), generators.mixed_scene(seed=2), generators.furnace_scene()):
        a = surface_areas(w.scene)
        assert np.allclose(a, w.areas, rtol=5e-6)
        b = budgets_by_area(w.scene, 10**9)
        assert np.all(b % 4 == 0) and abs(int(b.sum()) - 10**9) < 4 * w.scene.n
        assert np.allclose(b / b.sum(), a / a.sum(), atol=1e-8)
    # the file's <rayDensity> weights the area budgets exactly (the reference
    # truncates it into its integer area proxy, Scene.cpp:362-387)
    xml = """<project><settings><globalRayDensity value="1" /></settings><geometry>
        <primitive type="disc"><rayDensity value="2.5" /><scale x="1" y="1" z="1" /></primitive>
        <primitive type="disc"><scale x="1" y="1" z="1" /><translation x="0" y="0" z="1" /></primitive>
        <primitive type="disc"><rayDensity value="0.5" /><scale x="2" y="2" z="1" /></primitive>
        </geometry></project>"""
    sc = parse_scene_xml(xml)
    assert np.array_equal(sc.density, [2.5, 1.0, 0.5])
    assert list(sc.primitives["rayDensity"]) == [6, 3, 0]  # (int)2.5*pi, pi, (int)0.5*4pi
    b = budgets_by_area(sc, 10**8)
    w = np.array([2.5 * math.pi, math.pi, 0.5 * 4 * math.pi])
    assert np.allclose(b / b.sum(), w / w.sum(), atol=1e-7)
    assert np.allclose(budgets_by_area(sc, 10**8, use_density=False) / 10**8,
                       np.array([1, 1, 4]) / 6, atol=1e-7)
    # an ellipsoid: Knud Thomsen's formula (Scene.cpp:373-374) is within 1.061 %
    xml = """<project><settings><globalRayDensity value="1" /></settings><geometry>
        <primitive type="sphere"><scale x="1" y="2" z="3" /></primitive></geometry></project>"""
    sc = parse_scene_xml(xml)
    p = 1.6075
    thomsen = 4 * math.pi * ((2 ** p + 3 ** p + 6 ** p) / 3) ** (1 / p)
    assert abs(surface_areas(sc)[0] / thomsen - 1) < 0.0107


def test_segment_stacks(built_lib):
    """Runs of consecutive cylinders that tile one longer cylinder (a furnace wall
    of rings) and of concentric annuli in one plane whose radii meet (an end plate
    of rings) are found from the tables alone; a ring moved, resized or turned, a
    gap between two annuli, or a bounding surface's child range ends a run."""
    from rayfactorcl_gb300.tracer import segment_stacks
    assert segment_stacks(golden_scene("input-W100")) == [(0, 55)]
    fur = segment_stacks(golden_scene("input-furnace"))  # the reference's own furnace model
    assert fur[:2] == [(0, 180), (180, 128)] and fur[-2:] == [(360, 26), (386, 26)] and len(fur) == 11
    assert all(c >= 2 for _, c in fur)
    for name in ("gen_mixed64", "gen_enclosure3", "gen_precision_stress", "input-C47", "gen_sweep0"):
        assert segment_stacks(golden_scene(name)) == []
    sc = golden_scene("gen_furnace")
    plates = [(180, 20), (200, 20)]
    assert segment_stacks(sc) == [(0, 180)] + plates

    def edited(k, edit):
        s2 = sc.__class__.from_bytes(sc.to_bytes())
        if edit == "gap":
            s2.primitives["util1"][k] *= np.float32(1.0 + 2.0 ** -20)
            return s2
        m = s2.primitives["m"][k].astype(np.float64).reshape(3, 4)
        if edit == "shift":
            m[2, 3] += 1e-3 * m[2, 2]
        elif edit == "radius":
            m[:, 0] *= 1.001
        else:
            m[:, :2] = m[:, [1, 0]]  # x and y axes swapped: same cylinder, another frame
        s2.primitives["m"][k] = m.reshape(-1).astype(np.float32)
        return s2

    assert segment_stacks(edited(100, "shift")) == [(0, 100), (101, 79)] + plates
    for k, edit in ((50, "radius"), (140, "turn")):
        assert segment_stacks(edited(k, edit)) == [(0, k), (k + 1, 179 - k)] + plates, edit
    assert segment_stacks(edited(190, "gap")) == [(0, 180), (180, 10), (190, 10), (200, 20)]
    # bounding-surface child ranges cut runs
    bvs = np.array(sc.bounding_volumes, BV_DTYPE)
    cut = np.concatenate([bvs[:1], bvs])
    cut[0]["objEndIndex"] = 90
    cut[1]["objStartIndex"] = 90
    s3 = sc.__class__.from_bytes(sc.to_bytes())
    s3.bounding_volumes = cut
    assert segment_stacks(s3) == [(0, 90), (90, 90)] + plates
    assert segment_stacks(s3, use_bv=False) == [(0, 180)] + plates
    L = _lib.load()
    k = ctypes.c_int32()
    assert L.rf_segment_stacks(None, 0, None, 0, None, None, 0, ctypes.byref(k)) == 1
