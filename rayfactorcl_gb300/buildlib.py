"""Build ``librayfactor_gb300.so`` (the C ABI of include/rayfactor_gb300.h) in tree.

Each CUDA translation unit is compiled for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, then linked with
the static CUDA runtime so the library needs nothing but the driver.
``rf_kern_exact.cu`` is compiled with ``-fmad=false`` so that products and sums
written separately in the source keep separate roundings (bit-exact mode).
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
INCLUDE = ROOT / "include"
OBJ = PKG / "_build"
LIB = PKG / "librayfactor_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "-I", str(INCLUDE), "-I", str(CSRC)]
UNITS = {
    "rf_kern_exact.cu": ["-fmad=false"],
    "rf_kern_fast.cu": [],
    "rf_kern_batched.cu": [],
    "rf_kern_post.cu": [],
    "rf_capi.cu": [],
    "rf_noalloc.cu": [],
}
HEADERS = ["rf_internal.h", "rf_device.cuh", "rf_trace_kernels.cuh", "rf_batched.cuh", "rf_mixed_small.cuh"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build the library")


def _deps() -> list[Path]:
    hs = [CSRC / h for h in HEADERS if (CSRC / h).exists()]
    return hs + [INCLUDE / "rayfactor_gb300.h"]


def _stale(out: Path, deps: list[Path]) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def _compile(unit: str, extra: list[str], force: bool) -> Path:
    src = CSRC / unit
    obj = OBJ / (Path(unit).stem + ".o")
    if force or _stale(obj, [src, *_deps()]):
        tmp = obj.with_suffix(".o.tmp%d" % os.getpid())
        cmd = [nvcc(), *ARCH, *COMMON, *extra, "-c", str(src), "-o", str(tmp)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed for %s:\n%s%s" % (unit, r.stdout, r.stderr))
        os.replace(tmp, obj)
    return obj


def build(force: bool = False, verbose: bool = False) -> Path:
    OBJ.mkdir(exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], force), UNITS.items()))
    if force or _stale(LIB, objs):
        tmp = LIB.with_suffix(".so.tmp%d" % os.getpid())
        cmd = [nvcc(), *ARCH, "-shared", "-o", str(tmp), *map(str, objs)]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
        os.replace(tmp, LIB)
    if verbose:
        print(LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
