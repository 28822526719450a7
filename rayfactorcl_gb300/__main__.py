"""Command line: the reference program's main() (RayFactorCL/main.cpp:275-284) on the GPU.

    python -m rayfactorcl_gb300 [input.xml] [-o output.txt] [--compat] [--precision exact]
                                [--record run.json] [--split-stacks]

Reads the scene (Scene::readScene, Scene.cpp:24-52), runs runCL_GPURNG with
n_samples = globalRayDensity (main.cpp:281) and writes the view-factor matrix in
the reference's output.txt format (main.cpp:236-249).  ``--record`` also writes a
JSON run record: rays, times, rays/s, the largest binomial standard error of F,
the summation-rule residual and, in mixed precision, the FP64 re-evaluations.
"""
from __future__ import annotations

import argparse
import json
import sys
import time

import numpy as np

from . import _lib
from .scene import read_scene
from .tracer import PREC_EXACT, PREC_FAST, PREC_FP64, PREC_MIXED, run_cl_gpurng


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m rayfactorcl_gb300",
                                 description="Monte Carlo view factors of a RayFactorCL scene on the GPU")
    ap.add_argument("input", nargs="?", default="input.xml")
    ap.add_argument("-o", "--output", default="output.txt")
    ap.add_argument("--compat", action="store_true",
                    help="reproduce the reference run for run, including its known quirks")
    ap.add_argument("--precision", default="exact", choices=["exact", "fast", "mixed", "fp64"])
    ap.add_argument("--device", type=int, default=0)
    ap.add_argument("--record", default=None, help="write a JSON run record to this path")
    ap.add_argument("--split-stacks", action="store_true",
                    help="mixed precision: test every ring of a segmented wall or end plate on its own")
    args = ap.parse_args(argv)
    prec = {"exact": PREC_EXACT, "fast": PREC_FAST, "mixed": PREC_MIXED, "fp64": PREC_FP64}[args.precision]
    try:
        scene = read_scene(args.input)
    except (OSError, ValueError) as e:
        print(f"Failed to load file \"{args.input}\": {e}", file=sys.stderr)
        return 1
    print("=========== RayFactor GB300 =============")
    print(f"Number of objects : {scene.n}")
    t0 = time.perf_counter()
    stats: dict = {}
    try:
        rays, hits, F = run_cl_gpurng(int(scene.global_ray_density), scene, output=args.output,
                                      stats=stats, precision=prec, device=args.device,
                                      compat=_lib.COMPAT_ALL if args.compat else 0,
                                      split_stacks=args.split_stacks)
    except _lib.RfError as e:
        print(f"rayfactor_gb300: {e}", file=sys.stderr)
        return 1
    dt = time.perf_counter() - t0
    total = int(rays.sum())
    print(f"Rays traced : {total} in {dt:.3f} s -> {args.output}")
    if args.record:
        shot = rays > 0
        Fs = np.where(shot[:, None], F, 0.0)
        sig = np.sqrt(np.clip(Fs * (1.0 - Fs), 0.0, None) / np.maximum(rays, 1)[:, None])
        rec = {"input": str(args.input), "output": str(args.output), "surfaces": int(scene.n),
               "precision": args.precision, "compat": bool(args.compat), "rays": total,
               "wall_s": dt, "kernel_ms": stats.get("kernel_ms"), "launches": stats.get("launches"),
               "rays_per_s_kernel": total / (stats["kernel_ms"] * 1e-3) if stats.get("kernel_ms") else None,
               "max_binomial_sigma": float(sig[shot].max()) if shot.any() else None,
               "max_row_sum_error": float(np.abs(Fs[shot].sum(axis=1) - 1.0).max()) if shot.any() else None,
               "fp64_refined_tests": stats.get("fp64_refined_tests", 0)}
        with open(args.record, "w") as f:
            json.dump(rec, f, indent=1)
    return 0


if __name__ == "__main__":
    sys.exit(main())
