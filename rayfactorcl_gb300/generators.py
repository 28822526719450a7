"""Seeded synthetic scenes for the five benchmark workloads, written as scene
XML in the reference's format (RayFactorCL/Scene.cpp:191-282 grammar) so that
the reference loader and :func:`rayfactorcl_gb300.scene.parse_scene_xml` read
the same file.  Random draws use numpy's PCG64, which gives the same numbers on
every platform.

* :func:`enclosure3` -- disc / disc / inward cylinder closed enclosure (r=0.5, h=1).
* :func:`mixed_scene` -- 16 cylinders, 16 frusta, 12 discs, 10 annuli, 10 spheres,
  radii U[0.05,1], lengths U[0.1,2], random axes, centres U[-3,3]^3.
* :func:`furnace_scene` -- 180-segment inward wall (r=0.1 m, L=1.8 m), 2x20 end
  annuli, a fibre cylinder (r=62.5e-6 m), a 30-frustum neck-down, bounding surfaces.
* :func:`batched_sweep` -- 256 mixed scenes with log-uniform primitive counts.
* :func:`precision_stress` -- thin annuli (r_in/r_out=0.999), 89.9 degree frusta,
  unit-size primitives offset 1e4 from the origin.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .scene import Scene, parse_scene_xml


def _f(v: float) -> str:
    return repr(float(v))


class _Xml:
    def __init__(self, description: str, global_ray_density: float = 1000000.0,
                 use_bv: bool = False):
        self.lines = ['<?xml version="1.0" ?>', "<project>", "\t<settings>",
                      f'\t\t<globalRayDensity value="{_f(global_ray_density)}" />',
                      f"\t\t<description>{description}</description>"]
        if use_bv:
            self.lines.append('\t\t<useBoundingVolumes value="true" />')
        self.lines += ["\t</settings>", "\t<geometry>"]

    def prim(self, ptype: str, *, scale=None, rotate=None, translate=None, small=None,
             large=None, bounding=None, indent: int = 2, tag: str = "primitive", extra: str = ""):
        pad = "\t" * indent
        attrs = f'type="{ptype}"'
        if bounding is not None:
            attrs += f' isBounding="{"true" if bounding else "false"}"'
        attrs += extra
        self.lines.append(f"{pad}<{tag} {attrs}>")
        if small is not None:
            self.lines.append(f'{pad}\t<smallRadius value="{_f(small)}" />')
        if large is not None:
            self.lines.append(f'{pad}\t<largeRadius value="{_f(large)}" />')
        if scale is not None:
            self.lines.append(f'{pad}\t<scale x="{_f(scale[0])}" y="{_f(scale[1])}" z="{_f(scale[2])}" />')
        if rotate is not None:
            deg, ax = rotate
            self.lines.append(f'{pad}\t<rotate degrees="{_f(deg)}" x="{_f(ax[0])}" y="{_f(ax[1])}" z="{_f(ax[2])}" />')
        if translate is not None:
            t = translate
            self.lines.append(f'{pad}\t<translation x="{_f(t[0])}" y="{_f(t[1])}" z="{_f(t[2])}" />')

    def close(self, indent: int = 2, tag: str = "primitive"):
        self.lines.append("\t" * indent + f"</{tag}>")

    def raw(self, line: str):
        self.lines.append(line)

    def text(self) -> str:
        return "\n".join(self.lines + ["\t</geometry>", "</project>", ""])


def _axis_rotation(a: np.ndarray):
    """(degrees, unit axis) of the rotation taking +z onto the unit vector a."""
    a = a / np.linalg.norm(a)
    cz = float(np.clip(a[2], -1.0, 1.0))
    axis = np.array([-a[1], a[0], 0.0])
    n = np.linalg.norm(axis)
    if n < 1e-12:
        return (0.0, (1.0, 0.0, 0.0)) if cz > 0 else (180.0, (1.0, 0.0, 0.0))
    axis /= n
    # the reference rotates "clockwise" (AffineTransformation.cpp:23): the
    # matrix it builds for +theta about u is the usual rotation by -theta.
    return -math.degrees(math.acos(cz)), tuple(axis)


@dataclass
class Workload:
    """A scene plus its per-emitter ray budgets and stream key."""
    name: str
    xml: str
    scene: Scene
    rays: np.ndarray            # int64 per emitter
    areas: np.ndarray           # float64 exact surface areas per primitive
    key1: int = 0xDECAFBAD


def _budget_by_area(areas: np.ndarray, total: int) -> np.ndarray:
    w = areas / areas.sum()
    rays = np.floor(w * total / 4.0).astype(np.int64) * 4
    return np.maximum(rays, 4)


def enclosure3(rays_per_surface: int = 10_000_000, seed: int = 1, size: float = 1.0) -> Workload:
    """Coaxial discs of radius size/2, size apart, closed by an inward cylinder
    (the view factors do not depend on size)."""
    h, r = size, 0.5 * size
    x = _Xml(f"3-surface closed enclosure: coaxial discs r={r:g}, h={h:g}, inward cylinder")
    x.prim("disc", scale=(r, r, 1.0))
    x.close()
    x.prim("disc", scale=(r, r, 1.0), rotate=(180.0, (1.0, 0.0, 0.0)), translate=(0.0, 0.0, h))
    x.close()
    x.prim("cylinderSurface", bounding=True, small=1.0, scale=(r, r, h))
    x.close()
    text = x.text()
    sc = parse_scene_xml(text)
    areas = np.array([math.pi * r * r, math.pi * r * r, 2 * math.pi * r * h])
    rays = np.full(3, rays_per_surface, np.int64)
    return Workload("enclosure3", text, sc, rays, areas, key1=seed & 0xFFFFFFFF)


def mixed_scene(seed: int = 2, total_rays: int = 100_000_000,
                counts=(16, 16, 12, 10, 10), name: str = "mixed64") -> Workload:
    rng = np.random.Generator(np.random.PCG64(seed))
    x = _Xml(f"mixed-primitive scene, seed {seed}")
    areas = []
    kinds = (["cyl"] * counts[0] + ["fru"] * counts[1] + ["disc"] * counts[2]
             + ["ann"] * counts[3] + ["sph"] * counts[4])
    for kind in kinds:
        r = float(rng.uniform(0.05, 1.0))
        length = float(rng.uniform(0.1, 2.0))
        v = rng.normal(size=3)
        axis = v / np.linalg.norm(v)
        rot = _axis_rotation(axis)
        c = rng.uniform(-3.0, 3.0, size=3)
        if kind == "cyl":
            x.prim("cylinderSurface", small=1.0, scale=(r, r, length), rotate=rot, translate=c)
            areas.append(2 * math.pi * r * length)
        elif kind == "fru":
            top = float(rng.uniform(0.0, 1.0))
            x.prim("frustum", small=top, scale=(r, r, length), rotate=rot, translate=c)
            slant = math.hypot(length, r * (1 - top))
            areas.append(math.pi * r * (1 + top) * slant)
        elif kind == "disc":
            x.prim("disc", scale=(r, r, 1.0), rotate=rot, translate=c)
            areas.append(math.pi * r * r)
        elif kind == "ann":
            rin = r * float(rng.uniform(0.1, 0.9))
            x.prim("annulus", small=rin, large=r, rotate=rot, translate=c)
            areas.append(math.pi * (r * r - rin * rin))
        else:
            x.prim("sphere", scale=(r, r, r), translate=c)
            areas.append(4 * math.pi * r * r)
        x.close()
    text = x.text()
    sc = parse_scene_xml(text)
    areas = np.array(areas)
    return Workload(name, text, sc, _budget_by_area(areas, total_rays), areas,
                    key1=seed & 0xFFFFFFFF)


def furnace_scene(total_rays: int = 1_000_000_000, seed: int = 3) -> Workload:
    """Fibre-drawing furnace: inward wall of 180 segments inside one bounding
    cylinder, 20 annuli at each end, a thin fibre on the axis below a 30-frustum
    neck-down.  Every primitive sits under a bounding surface."""
    R, L, nseg = 0.1, 1.8, 180
    seg = L / nseg
    r_fibre = 62.5e-6
    r_pre = 0.02
    neck_z0, neck_z1 = 0.6, 1.2
    x = _Xml("furnace-like enclosure with bounding surfaces", use_bv=True)
    areas = []
    # BV 0: the wall
    x.prim("cylinderSurface", small=1.0, scale=(R, R, L), tag="bv", indent=2)
    x.raw("\t\t\t<children>")
    for i in range(nseg):
        x.prim("cylinderSurface", bounding=True, small=1.0, scale=(R, R, seg),
               translate=(0.0, 0.0, i * seg), indent=4)
        x.close(indent=4)
        areas.append(2 * math.pi * R * seg)
    x.raw("\t\t\t</children>")
    x.close(tag="bv")
    # BV 1/2: bottom and top end plates, 20 rings each from r_pre to R
    edges = np.linspace(r_pre, R, 21)
    for end, (z, rot) in enumerate([(0.0, None), (L, (180.0, (1.0, 0.0, 0.0)))]):
        x.prim("annulus", small=r_pre, large=R, rotate=rot, translate=(0.0, 0.0, z),
               tag="bv", indent=2)
        x.raw("\t\t\t<children>")
        for k in range(20):
            x.prim("annulus", small=edges[k], large=edges[k + 1], rotate=rot,
                   translate=(0.0, 0.0, z), indent=4)
            x.close(indent=4)
            areas.append(math.pi * (edges[k + 1] ** 2 - edges[k] ** 2))
        x.raw("\t\t\t</children>")
        x.close(tag="bv")
    # BV 3: the preform / neck-down / fibre column, checked immediately
    x.prim("cylinderSurface", small=1.0, scale=(r_pre, r_pre, L), tag="bv", indent=2,
           extra=' intermediateCheck="true"')
    x.raw("\t\t\t<children>")
    x.prim("cylinderSurface", small=1.0, scale=(r_fibre, r_fibre, neck_z0), indent=4)
    x.close(indent=4)
    areas.append(2 * math.pi * r_fibre * neck_z0)
    radii = np.geomspace(r_fibre, r_pre, 31)
    dz = (neck_z1 - neck_z0) / 30
    for k in range(30):
        r0, r1 = radii[k], radii[k + 1]
        x.prim("frustum", small=r1 / r0, scale=(r0, r0, dz),
               translate=(0.0, 0.0, neck_z0 + k * dz), indent=4)
        x.close(indent=4)
        areas.append(math.pi * (r0 + r1) * math.hypot(dz, r1 - r0))
    x.prim("cylinderSurface", small=1.0, scale=(r_pre, r_pre, L - neck_z1),
           translate=(0.0, 0.0, neck_z1), indent=4)
    x.close(indent=4)
    areas.append(2 * math.pi * r_pre * (L - neck_z1))
    x.raw("\t\t\t</children>")
    x.close(tag="bv")
    text = x.text()
    sc = parse_scene_xml(text)
    areas = np.array(areas)
    return Workload("furnace", text, sc, _budget_by_area(areas, total_rays), areas,
                    key1=seed & 0xFFFFFFFF)


def batched_sweep(n_scenes: int = 256, seed: int = 4, min_prims: int = 10,
                  max_prims: int = 400, min_budget: float = 1e5, max_budget: float = 1e7):
    """Independent mixed scenes with log-uniform primitive counts and
    log-uniform per-emitter budgets."""
    rng = np.random.Generator(np.random.PCG64(seed))
    out = []
    for s in range(n_scenes):
        n = int(round(math.exp(rng.uniform(math.log(min_prims), math.log(max_prims)))))
        frac = np.array([16, 16, 12, 10, 10], float) / 64.0
        counts = np.floor(frac * n).astype(int)
        counts[0] += n - counts.sum()
        w = mixed_scene(seed=seed * 100003 + s, total_rays=4, counts=tuple(int(c) for c in counts),
                        name=f"sweep{s}")
        b = np.exp(rng.uniform(math.log(min_budget), math.log(max_budget), size=w.scene.n))
        w.rays = (np.floor(b / 4.0).astype(np.int64) * 4)
        out.append(w)
    return out


def precision_stress(total_rays: int = 100_000_000, seed: int = 5) -> Workload:
    """Thin annuli, 89.9 degree frusta and unit primitives 1e4 from the origin."""
    rng = np.random.Generator(np.random.PCG64(seed))
    x = _Xml("precision stress: thin annuli, 89.9 degree frusta, far offsets")
    areas = []
    off = np.array([1e4, 0.0, 0.0])
    # a closed unit box of sorts around the offset point: coaxial thin annuli
    for k in range(4):
        rout = 1.0 + 0.25 * k
        rin = 0.999 * rout
        rot = (180.0, (1.0, 0.0, 0.0)) if k % 2 else None
        x.prim("annulus", small=rin, large=rout, rotate=rot,
               translate=off + np.array([0.0, 0.0, float(k % 2)]))
        x.close()
        areas.append(math.pi * (rout ** 2 - rin ** 2))
    tan_half = math.tan(math.radians(89.9))
    for k in range(4):
        top = 0.5
        h = (1.0 - top) / tan_half
        x.prim("frustum", small=top, scale=(1.0, 1.0, h),
               translate=off + np.array([0.0, 0.0, 0.2 + 0.2 * k]))
        x.close()
        areas.append(math.pi * (1 + top) * math.hypot(h, 1 - top))
    for k in range(8):
        v = rng.normal(size=3)
        rot = _axis_rotation(v / np.linalg.norm(v))
        c = off + rng.uniform(-1.0, 1.0, size=3) * 2.0
        if k % 2:
            x.prim("cylinderSurface", small=1.0, scale=(0.5, 0.5, 1.0), rotate=rot, translate=c)
            areas.append(2 * math.pi * 0.5)
        else:
            x.prim("sphere", scale=(0.5, 0.5, 0.5), translate=c)
            areas.append(4 * math.pi * 0.25)
        x.close()
    text = x.text()
    sc = parse_scene_xml(text)
    areas = np.array(areas)
    return Workload("precision_stress", text, sc, _budget_by_area(areas, total_rays), areas,
                    key1=seed & 0xFFFFFFFF)
