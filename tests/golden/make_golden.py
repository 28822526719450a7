"""Regenerate the golden fixtures in this folder from the reference's own code.

Run from the repository root:  python tests/golden/make_golden.py

* ``philox_kat.json`` -- Philox4x32-10 outputs of the reference's
  RayFactorCL/Random123/philox.h (built by oracle/build.py into
  oracle/_ref/ref_philox_kat) on the counters and keys the tracer uses.
* ``scenes/<name>.bin`` -- Primitive/BoundingVolume tables produced by the
  reference's Scene.cpp + TinyXML-2 + affine code (oracle/_ref/ref_scene_dump)
  for every sample geometry of the reference and for the seeded workload
  scenes whose XML is committed beside them as ``scenes/gen_<name>.xml``.
* ``ref_kernel_rays.npz`` -- per-ray first-hit surfaces (-1 = none) written by
  the reference's own kernel source, RayFactorCL/RayFactorGPU.cl compiled on the
  host (oracle/_ref/librf_refkernel.so): runGPU on every scene above and
  runBVGPU on those with bounding surfaces, for work-items REF_WINDOWS of every
  emitter.  Key ``<scene>:<kernel>``, value int16 [n_emitters, 4 x work-items].

Needs the reference checkout (RF_REFERENCE_DIR, else ``reference`` beside the
repository).
"""
from __future__ import annotations

import json
import subprocess
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import build as obuild  # noqa: E402
from rayfactorcl_gb300 import generators  # noqa: E402

HERE = Path(__file__).resolve().parent
SCENES = HERE / "scenes"


def kat_inputs():
    rng = np.random.Generator(np.random.PCG64(123))
    rows = []
    ref_ctr = [1, 0xF00DCAFE, 0xDEADBEEF, 0xBEEFF00D]
    for gid in list(range(16)) + [127, 128, 1000, 65535, 2**31 - 1, 2**31, 2**32 - 1]:
        rows.append((ref_ctr, [gid, 0xDECAFBAD]))
        rows.append((ref_ctr, [gid, 12345]))
    for emitter in (0, 1, 5, 63, 411):
        for gid in (0, 1, 7, 2**32 + 3):
            rows.append(([1, emitter, gid >> 32, 0xBEEFF00D], [gid & 0xFFFFFFFF, 0xDECAFBAD]))
    for _ in range(32):
        c = [int(v) for v in rng.integers(0, 2**32, 4, dtype=np.uint64)]
        k = [int(v) for v in rng.integers(0, 2**32, 2, dtype=np.uint64)]
        rows.append((c, k))
    rows.append(([0, 0, 0, 0], [0, 0]))
    rows.append(([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2))
    return rows


def make_kat():
    rows = kat_inputs()
    text = "".join("%x %x %x %x %x %x\n" % (*c, *k) for c, k in rows)
    r = subprocess.run([str(obuild.REF_KAT)], input=text, capture_output=True, text=True, check=True)
    outs = [[int(w, 16) for w in line.split()] for line in r.stdout.strip().splitlines()]
    assert len(outs) == len(rows)
    data = [{"ctr": c, "key": k, "out": o} for (c, k), o in zip(rows, outs)]
    (HERE / "philox_kat.json").write_text(json.dumps(data, indent=0))
    return len(data)


def dump(xml_path: Path, out: Path):
    subprocess.run([str(obuild.REF_SCENE), str(xml_path), str(out)], check=True,
                   capture_output=True)


def generated_workloads():
    ws = [generators.enclosure3(), generators.mixed_scene(), generators.furnace_scene(),
          generators.precision_stress()]
    ws += generators.batched_sweep(n_scenes=3, seed=4)
    return ws


def make_scenes():
    SCENES.mkdir(exist_ok=True)
    names = []
    for xml in sorted((obuild.REFERENCE / "sample-geometries").glob("*.xml")):
        dump(xml, SCENES / (xml.stem + ".bin"))
        names.append(xml.stem)
    for w in generated_workloads():
        xp = SCENES / f"gen_{w.name}.xml"
        xp.write_text(w.xml)
        dump(xp, SCENES / f"gen_{w.name}.bin")
        names.append("gen_" + w.name)
    return names


# work-item (global id) windows of the per-ray fixture: the first ids, and a
# window across 2^20 at an odd offset
from oracle.oracle import REF_WINDOWS  # noqa: E402


def ref_kernel_rays(lib, scene, use_bv: int, windows=REF_WINDOWS) -> np.ndarray:
    """Per-ray hits of the compiled reference kernel for every emitter."""
    import ctypes
    prims = np.ascontiguousarray(scene.primitives)
    bvs = np.ascontiguousarray(scene.bounding_volumes)
    rows = []
    for e in range(scene.n):
        parts = []
        for g0, g1 in windows:
            out = np.full(4 * (g1 - g0), -7, np.int32)
            rc = lib.rfr_trace_rays(prims.ctypes.data, prims.shape[0],
                                    bvs.ctypes.data if bvs.shape[0] else None, bvs.shape[0],
                                    use_bv, e, g0, g1, out.ctypes.data)
            if rc != 0:
                raise RuntimeError(f"reference kernel failed ({rc})")
            parts.append(out)
        rows.append(np.concatenate(parts))
    return np.stack(rows)


def load_ref_kernel():
    import ctypes
    lib = ctypes.CDLL(str(obuild.REF_KERNEL))
    P = ctypes.c_void_p
    lib.rfr_trace_rays.argtypes = [P, ctypes.c_int32, P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                   ctypes.c_int64, ctypes.c_int64, P]
    lib.rfr_trace_rays.restype = ctypes.c_int
    return lib


def make_ref_rays(names):
    from rayfactorcl_gb300.scene import Scene
    lib = load_ref_kernel()
    data = {}
    for name in names:
        sc = Scene.from_bytes((SCENES / f"{name}.bin").read_bytes())
        kernels = ["runGPU"] + (["runBVGPU"] if sc.bounding_volumes.shape[0] else [])
        for k in kernels:
            data[f"{name}:{k}"] = ref_kernel_rays(lib, sc, int(k == "runBVGPU")).astype(np.int16)
    np.savez_compressed(HERE / "ref_kernel_rays.npz", **data)
    return sum(v.size for v in data.values())


def main():
    if not obuild.build_ref():
        print("reference checkout not found; nothing regenerated")
        return 1
    print("philox vectors:", make_kat())
    names = make_scenes()
    print("scenes:", ", ".join(names))
    print("reference-kernel rays:", make_ref_rays(names))
    return 0


if __name__ == "__main__":
    sys.exit(main())
