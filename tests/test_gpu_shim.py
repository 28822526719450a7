"""GPU test of the drop-in for runCL_GPURNG (include/rayfactor_gb300_shim.hpp).

A host program built from tests/shim/shim_main.cpp -- the reference's main()
(RayFactorCL/main.cpp:275-284) with runCL_GPURNG replaced by runCUDA_GPURNG --
links librayfactor_gb300.so and writes output.txt.  The Scene it hands to the
shim holds the tables the reference's own loader produced for the sample
geometry (tests/golden/scenes/*.bin, read by the stand-in tests/shim/scene_stub.h;
the CPU suite links the same program with the reference's Scene.cpp itself).
Its output.txt must equal, byte for byte, the file written by rf_run_gpurng +
rf_write_output_txt on the same tables with the reference's budgets, streams and
quirks (RF_COMPAT_ALL)."""
import numpy as np
import pytest

from helpers import GOLDEN, golden_scene
from rayfactorcl_gb300 import _lib
from rayfactorcl_gb300.tracer import Tracer, write_output_txt
from test_capi_cpu import _run_shim, build_shim_program

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["input-C47", "input-C52-BV"])
def test_shim_output_equals_library_run(built_lib, tmp_path, name):
    exe = build_shim_program(tmp_path / "shim", True, built_lib)
    r = _run_shim(exe, GOLDEN / "scenes" / f"{name}.bin", tmp_path)
    assert r.returncode == 0, r.stderr
    got = (tmp_path / "output.txt").read_bytes()
    sc = golden_scene(name)
    with Tracer(compat=_lib.COMPAT_ALL) as t:
        t.set_scene(sc)
        rays, hits, F = t.run_gpurng(int(sc.global_ray_density), use_bv=bool(sc.use_bounding_volumes))
    assert rays.min() > 0 and hits.sum() > 0
    write_output_txt(tmp_path / "expected.txt", F)
    assert got == (tmp_path / "expected.txt").read_bytes()
    rows = [ln for ln in got.decode().splitlines() if ln]
    assert len(rows) == sc.n and all(ln.endswith(",") for ln in rows)
    assert np.isfinite(F).all()
