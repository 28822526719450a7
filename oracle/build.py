"""Build recipe for the test oracle (test infrastructure, not the product).

* ``oracle/_build/librf_oracle.so`` -- the C restatement in ``rf_oracle.c``,
  compiled with ``-O2 -ffp-contract=off`` (every rounding as written) and
  OpenMP for the multi-core CPU baseline.
* ``oracle/_ref/ref_philox_kat`` and ``oracle/_ref/ref_scene_dump`` -- the
  reference's own Random123 Philox header and Scene/TinyXML-2/affine sources,
  compiled from where they lie in the reference checkout together with the two
  small drivers in ``ref_tools/``.
* ``oracle/_ref/librf_refkernel.so`` -- the reference's OpenCL C kernel source
  (RayFactorCL/RayFactorGPU.cl) compiled as host C++: ``ref_tools/cl_compat.h``
  supplies the OpenCL types and builtins with the oracle's fixed op mapping,
  ``rewrite_cl`` makes the few token rewrites OpenCL C needs (vector literals,
  one swizzle, address-space keywords), and ``ref_tools/ref_kernel_host.cpp``
  runs runGPU / runBVGPU work-item by work-item.  The rewritten text goes to
  g++ on its standard input and is never written to disk.

The reference checkout is ``RF_REFERENCE_DIR`` when set, else a directory named
``reference`` beside the repository.  The reference tools are built only when
the checkout is present; nothing is copied out of it.  Their outputs are
committed as fixtures under ``tests/golden/``.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
BUILD = HERE / "_build"
REF_OUT = HERE / "_ref"
REFERENCE = Path(os.environ.get("RF_REFERENCE_DIR", str(HERE.parent.parent / "reference")))

ORACLE_SO = BUILD / "librf_oracle.so"
REF_KAT = REF_OUT / "ref_philox_kat"
REF_SCENE = REF_OUT / "ref_scene_dump"
REF_KERNEL = REF_OUT / "librf_refkernel.so"


def _run(cmd: list[str], stdin: str | None = None) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True, input=stdin)
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


def build_oracle_variant(out: Path, defines: list[str]) -> Path:
    """The oracle compiled with extra -D switches into `out` (tests only)."""
    _run(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-w",
          *["-D" + d for d in defines], "-o", str(out), str(HERE / "rf_oracle.c"), "-lm"])
    return out


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
    kern_deps = [HERE / "ref_tools" / "cl_compat.h", HERE / "ref_tools" / "ref_kernel_host.cpp",
                 HERE / "rf_oracle.c", HERE / "rf_oracle.h", Path(__file__)]
    if force or _stale(REF_KERNEL, kern_deps):
        build_ref_kernel()
    return True


def rewrite_cl(text: str) -> str:
    """Token rewrites that make RayFactorGPU.cl valid C++ (no logic changes):
    OpenCL vector literals become constructor calls, the .yzwx swizzle a member
    call, and the address-space qualifiers disappear (__constant: static const)."""
    text = re.sub(r"\(float4\)\s*\(", "make_float4(", text)
    text = re.sub(r"\.yzwx\b", ".yzwx()", text)
    for kw in ("__kernel", "__global", "__local"):
        text = re.sub(r"\b%s\b" % kw, "", text)
    text = re.sub(r"\bglobal\b", "", text)
    text = re.sub(r"\b__constant\b", "static const", text)
    return text


def build_ref_kernel() -> Path:
    """Compile the reference kernel source with cl_compat.h and the driver."""
    rfc = REFERENCE / "RayFactorCL"
    cl = (rfc / "RayFactorGPU.cl").read_text()
    tools = HERE / "ref_tools"
    unit = ('#include "cl_compat.h"\n#line 1 "RayFactorGPU.cl"\n' + rewrite_cl(cl) +
            '\n#line 1 "ref_kernel_host.cpp"\n#include "ref_kernel_host.cpp"\n')
    obj = REF_OUT / "rf_oracle_sincos.o"
    _run(["gcc", "-std=c11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-c", "-w",
          "-o", str(obj), str(HERE / "rf_oracle.c")])
    tmp = REF_KERNEL.with_suffix(".so.tmp%d" % os.getpid())
    _run(["g++", "-std=c++11", "-O2", "-ffp-contract=off", "-fno-fast-math", "-Wno-narrowing", "-w",
          "-fPIC", "-shared", "-I", str(tools), "-I", str(HERE), "-I", str(rfc), "-o", str(tmp),
          "-x", "c++", "-", "-x", "none", str(obj), "-lm"], stdin=unit)
    os.replace(tmp, REF_KERNEL)
    return REF_KERNEL


def main() -> int:
    force = "--force" in sys.argv
    print(build_oracle(force))
    print("reference tools:", "built" if build_ref(force) else "skipped (no checkout)")
    return 0


if __name__ == "__main__":
    sys.exit(main())
