"""Regenerate the golden fixtures in this folder from the reference's own code.

Run from the repository root:  python tests/golden/make_golden.py

* ``philox_kat.json`` -- Philox4x32-10 outputs of the reference's
  RayFactorCL/Random123/philox.h (built by oracle/build.py into
  oracle/_ref/ref_philox_kat) on the counters and keys the tracer uses.
* ``scenes/<name>.bin`` -- Primitive/BoundingVolume tables produced by the
  reference's Scene.cpp + TinyXML-2 + affine code (oracle/_ref/ref_scene_dump)
  for every sample geometry of the reference and for the seeded workload
  scenes whose XML is committed beside them as ``scenes/gen_<name>.xml``.

Needs the reference checkout (RF_REFERENCE_DIR, default /root/reference).
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


def main():
    if not obuild.build_ref():
        print("reference checkout not found; nothing regenerated")
        return 1
    print("philox vectors:", make_kat())
    print("scenes:", ", ".join(make_scenes()))
    return 0


if __name__ == "__main__":
    sys.exit(main())
