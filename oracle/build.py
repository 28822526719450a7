"""Build recipe for the test oracle (test infrastructure, not the product).

* ``oracle/_build/librf_oracle.so`` -- the C restatement in ``rf_oracle.c``,
  compiled with ``-O2 -ffp-contract=off`` (every rounding as written) and
  OpenMP for the multi-core CPU baseline.
* ``oracle/_ref/ref_philox_kat`` and ``oracle/_ref/ref_scene_dump`` -- the
  reference's own Random123 Philox header and Scene/TinyXML-2/affine sources,
  compiled from where they lie in the reference checkout (``RF_REFERENCE_DIR``,
  default ``/root/reference``) together with the two small drivers in
  ``ref_tools/``.  Built only when the checkout is present; nothing is copied
  out of it.  Their outputs are committed as fixtures under ``tests/golden/``.
"""
from __future__ import annotations

import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
REFERENCE = Path(os.environ.get("RF_REFERENCE_DIR", "/root/reference"))

ORACLE_SO = BUILD / "librf_oracle.so"
REF_KAT = REF_OUT / "ref_philox_kat"
REF_SCENE = REF_OUT / "ref_scene_dump"


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_oracle(force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    src = [HERE / "rf_oracle.c"]
    if force or _stale(ORACLE_SO, src + [HERE / "rf_oracle.h"]):
        tmp = ORACLE_SO.with_suffix(".so.tmp%d" % os.getpid())
        _run(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fopenmp",
              "-fPIC", "-shared", "-Wall", "-o", str(tmp), *map(str, src), "-lm"])
        os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


def reference_present() -> bool:
    return (REFERENCE / "RayFactorCL" / "Scene.cpp").exists()


def build_ref(force: bool = False) -> bool:
    """Compile the reference-side tools; False when the checkout is absent."""
    if not reference_present():
        return False
    REF_OUT.mkdir(exist_ok=True)
    rfc = REFERENCE / "RayFactorCL"
    aff = rfc / "Affine Transformation"
    txml = rfc / "TinyXML-2"
    common = ["g++", "-std=c++11", "-O2", "-ffp-contract=off", "-w"]
    kat_src = HERE / "ref_tools" / "ref_philox_kat.cpp"
    if force or _stale(REF_KAT, [kat_src]):
        _run(common + ["-I", str(rfc), "-o", str(REF_KAT), str(kat_src)])
    dump_src = HERE / "ref_tools" / "ref_scene_dump.cpp"
    if force or _stale(REF_SCENE, [dump_src]):
        _run(common + ["-I", str(rfc), "-I", str(aff), "-I", str(txml), "-o", str(REF_SCENE),
                       str(dump_src), str(rfc / "Scene.cpp"), str(txml / "tinyxml2.cpp"),
                       str(aff / "AffineTransformation.cpp"), str(aff / "Matrices.cpp")])
    return True


def main() -> int:
    force = "--force" in sys.argv
    print(build_oracle(force))
    print("reference tools:", "built" if build_ref(force) else "skipped (no checkout)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
