"""Scene tables and the XML scene reader.

The tables handed to the tracer are byte-identical to the reference's
``Primitive`` (112 bytes) and ``BoundingVolume`` (72 bytes) structs
(RayFactorCL/RayfactorConstants.h:38-56).  :func:`read_scene` restates the
reference's XML loader (RayFactorCL/Scene.cpp:24-452) and its affine helpers
(RayFactorCL/Affine Transformation/AffineTransformation.cpp:14-111,
Matrices.cpp:22-58) with the same single-precision roundings, so that a scene
file yields the same bits here as in the reference host program.  Fields the
reference leaves uninitialised read as 0 (``useBoundingVolumes`` when the
setting is absent, ``settings`` of a bounding surface without
``intermediateCheck``, ``util1``/``util2`` of discs and rectangles).
"""
from __future__ import annotations

import ctypes
import math
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

# RayfactorConstants.h:25-33
CYLINDER, FRUSTUM, SPHERE, ANNULUS, RECTANGLE, DISC, NONE = range(7)
TYPE_NAMES = {CYLINDER: "cylinder", FRUSTUM: "frustum", SPHERE: "sphere", ANNULUS: "annulus",
              RECTANGLE: "rectangle", DISC: "disc", NONE: "none"}

PRIM_DTYPE = np.dtype([("m", "<f4", (12,)), ("invm", "<f4", (12,)), ("type", "<i4"),
                       ("rayDensity", "<i4"), ("util1", "<f4"), ("util2", "<f4")])
BV_DTYPE = np.dtype([("invm", "<f4", (12,)), ("type", "<i4"), ("settings", "<i4"),
                     ("objStartIndex", "<i4"), ("objEndIndex", "<i4"), ("util1", "<f4"),
                     ("util2", "<f4")])
assert PRIM_DTYPE.itemsize == 112 and BV_DTYPE.itemsize == 72

F32 = np.float32
_PI_F = F32(3.141592)              # RayfactorConstants.h:12 (PI)
_AFF_PI = F32(3.141592653589793)   # AffineTransformation.h:189
_AFF_SEPS = F32(0.00001)           # AffineTransformation.h:188


@dataclass
class Scene:
    """Mirror of the reference ``Scene`` (RayFactorCL/Scene.h:22-36)."""
    global_ray_density: float = 0.0
    use_bounding_volumes: bool = False
    primitives: np.ndarray = field(default_factory=lambda: np.zeros(0, PRIM_DTYPE))
    bounding_volumes: np.ndarray = field(default_factory=lambda: np.zeros(0, BV_DTYPE))
    description: str = ""
    # each primitive's <rayDensity value> from the file (Scene.cpp:307-321; 1 when
    # absent), kept unrounded for area budgets; not part of the table bytes
    density: np.ndarray | None = None

    @property
    def n(self) -> int:
        return int(self.primitives.shape[0])

    def to_bytes(self) -> bytes:
        head = np.array([self.n, int(self.bounding_volumes.shape[0])], "<i4").tobytes()
        head += np.array([self.global_ray_density], "<f4").tobytes()
        head += np.array([1 if self.use_bounding_volumes else 0], "<i4").tobytes()
        return b"RFSC" + head + self.primitives.tobytes() + self.bounding_volumes.tobytes()

    @classmethod
    def from_bytes(cls, blob: bytes) -> "Scene":
        if blob[:4] != b"RFSC":
            raise ValueError("not a scene table blob")
        n, nb = np.frombuffer(blob, "<i4", 2, 4)
        grd = float(np.frombuffer(blob, "<f4", 1, 12)[0])
        ubv = bool(np.frombuffer(blob, "<i4", 1, 16)[0])
        off = 20
        prims = np.frombuffer(blob, PRIM_DTYPE, int(n), off).copy()
        off += int(n) * PRIM_DTYPE.itemsize
        bvs = np.frombuffer(blob, BV_DTYPE, int(nb), off).copy()
        return cls(grd, ubv, prims, bvs)


# --------------------------------------------------------------------------
# attribute parsing with the C library's sscanf, as TinyXML-2 does
# (tinyxml2.cpp:943-989)
# --------------------------------------------------------------------------
_libc = ctypes.CDLL(None)
_sscanf = _libc.sscanf


def _scan_float(s: str | None):
    if s is None:
        return None
    v = ctypes.c_float()
    if _sscanf(s.encode(), b"%f", ctypes.byref(v)) == 1:
        return F32(v.value)
    return None


def _scan_int(s: str | None):
    if s is None:
        return None
    v = ctypes.c_int()
    if _sscanf(s.encode(), b"%d", ctypes.byref(v)) == 1:
        return int(v.value)
    return None


def _float_attr(el, name, default=F32(0.0)):
    """XMLElement::FloatAttribute / QueryFloatAttribute (tinyxml2.h:884,907)."""
    v = _scan_float(el.get(name))
    return default if v is None else v


def _bool_attr(el, name) -> bool:
    """XMLElement::BoolAttribute (tinyxml2.h:880, tinyxml2.cpp:959-973)."""
    s = el.get(name)
    if s is None:
        return False
    ival = _scan_int(s)
    ival = -1 if ival is None else ival
    if ival > 0 or s == "true":
        return True
    return False


def _is_comment(node) -> bool:
    return node.tag is ET.Comment


def _first_child_is_element(el) -> bool:
    """``el->FirstChild()->ToElement() != NULL``: no leading text, first node an element."""
    if el.text is not None and el.text.strip():
        return False
    kids = list(el)
    return bool(kids) and not _is_comment(kids[0])


def _has_child_node(el) -> bool:
    return (el.text is not None and el.text.strip() != "") or len(el) > 0


def _elements(el):
    """Iteration from ``FirstChild()->ToElement()`` over ``NextSiblingElement()``."""
    if not _first_child_is_element(el):
        return []
    return [k for k in el if not _is_comment(k)]


# --------------------------------------------------------------------------
# 4x4 matrices in float (Matrix4.h:13-23, Matrices.cpp:22-58).  Storage index
# 4*c+r; every product and partial sum is rounded to float.
# --------------------------------------------------------------------------
def _identity():
    m = np.zeros(16, np.float32)
    m[[0, 5, 10, 15]] = 1.0
    return m


def _pre_multiply(x, a):
    """Matrices.cpp:22-38: x[4c+r] = sum_k a[4k+r] * x[4c+k]."""
    tmp = x.copy()
    out = np.zeros(16, np.float32)
    for c in range(4):
        for r in range(4):
            s = F32(0.0)
            for k in range(4):
                s = F32(s + F32(a[4 * k + r] * tmp[4 * c + k]))
            out[4 * c + r] = s
    x[:] = out


def _post_multiply(x, a):
    """Matrices.cpp:41-57: x[4c+r] = sum_k x[4k+r] * a[4c+k]."""
    tmp = x.copy()
    out = np.zeros(16, np.float32)
    for c in range(4):
        for r in range(4):
            s = F32(0.0)
            for k in range(4):
                s = F32(s + F32(tmp[4 * k + r] * a[4 * c + k]))
            out[4 * c + r] = s
    x[:] = out


def _rot_parts(angle, x, y, z):
    ang = F32(F32(F32(angle) * _AFF_PI) / F32(180.0))
    c = F32(math.cos(float(ang)))      # cos(float) resolves to the double overload
    s = F32(math.sin(float(ang)))
    return c, s, F32(F32(1.0) - c)


def _rotate(m, angle, x, y, z):
    """AffineTransformation.cpp:14-35."""
    c, s, mc = _rot_parts(angle, x, y, z)
    rm = _identity()
    rm[0] = c + mc * x * x
    rm[1] = mc * x * y + s * z
    rm[2] = mc * x * z - s * y
    rm[4] = mc * y * x - s * z
    rm[5] = c + mc * y * y
    rm[6] = mc * y * z + s * x
    rm[8] = mc * z * x + s * y
    rm[9] = mc * z * y - s * x
    rm[10] = c + mc * z * z
    _post_multiply(m, rm)


def _inv_rotate(m, angle, x, y, z):
    """AffineTransformation.cpp:38-58."""
    c, s, mc = _rot_parts(angle, x, y, z)
    rm = _identity()
    rm[0] = c + mc * x * x
    rm[1] = mc * x * y - s * z
    rm[2] = mc * x * z + s * y
    rm[4] = mc * y * x + s * z
    rm[5] = c + mc * y * y
    rm[6] = mc * y * z - s * x
    rm[8] = mc * z * x - s * y
    rm[9] = mc * z * y + s * x
    rm[10] = c + mc * z * z
    _pre_multiply(m, rm)


def _scale(m, sx, sy, sz):
    s = _identity()
    s[0], s[5], s[10] = sx, sy, sz
    _post_multiply(m, s)


def _inv_scale(m, sx, sy, sz):
    s = _identity()
    s[0], s[5], s[10] = F32(1.0) / sx, F32(1.0) / sy, F32(1.0) / sz
    _pre_multiply(m, s)


def _translate(m, x, y, z):
    t = _identity()
    t[3], t[7], t[11] = x, y, z
    _post_multiply(m, t)


def _inv_translate(m, x, y, z):
    t = _identity()
    t[3], t[7], t[11] = -x, -y, -z
    _pre_multiply(m, t)


def _trunc_int(v: float) -> int:
    """C conversion to int (toward zero); out-of-range values are reported."""
    if not math.isfinite(v) or abs(v) >= 2 ** 31:
        raise ValueError(f"rayDensity {v!r} does not fit an int")
    return int(v)


def _ray_density(ptype, rd, xs, ys, zs, util1, util2) -> int:
    """Scene.cpp:361-387 -- per-type area proxy, with the reference's mixed
    float/double arithmetic and truncating (int) casts."""
    ird = int(rd)  # (int)rayDensity
    if ptype == CYLINDER:
        v = ird * 2.0 * float(_PI_F) * float(zs) * math.pow(
            0.5 * (math.pow(float(xs), 2) + math.pow(float(ys), 2)), 0.5)
        return _trunc_int(v)
    if ptype == FRUSTUM:
        sm = F32(util1 + F32(1e-5))
        inner = F32(F32(F32(xs * xs) + F32(ys * ys)) * sm) * sm
        v = ird * (math.sqrt(float(inner)) * float(F32(1.0) + sm) * float(zs) * float(_PI_F)) \
            / (math.sqrt(2.0) * float(sm))
        return _trunc_int(v)
    if ptype == SPHERE:
        p = F32(1.6075)
        pp = float(p)
        a = math.pow(float(xs), pp) * math.pow(float(ys), pp)
        b = math.pow(float(xs), pp) * math.pow(float(zs), pp)
        c = math.pow(float(ys), pp) * math.pow(float(zs), pp)
        v = ird * (float(F32(4.0) * _PI_F) * math.pow((a + b + c) / 3.0, float(F32(1.0) / p)))
        return _trunc_int(v)
    if ptype == ANNULUS:
        v = F32(F32(F32(F32(rd) * _PI_F) * F32(util2 - util1)) + F32(0.5))
        return _trunc_int(float(v))
    if ptype == RECTANGLE:
        v = F32(F32(F32(F32(F32(ird) * F32(2.0)) * xs) * F32(2.0)) * ys)
        return _trunc_int(float(v))
    if ptype == DISC:
        v = F32(F32(F32(F32(ird) * _PI_F) * xs) * ys)
        return _trunc_int(float(v))
    return 1


def _init_transform(el, rec, with_forward: bool):
    """Scene.cpp:296-359 / 392-449: apply scale/rotate/translate in document
    order; returns (xScale, yScale, zScale, rayDensity, children_element)."""
    trm, inv = _identity(), _identity()
    xs = ys = zs = F32(1.0)
    rd = F32(1.0)
    children = []
    for child in _elements(el):
        name = child.tag
        if name == "rayDensity" and with_forward:
            rd = _float_attr(child, "value")
        elif name == "translation":
            x, y, z = (_float_attr(child, k) for k in "xyz")
            if with_forward:
                _translate(trm, x, y, z)
            _inv_translate(inv, x, y, z)
        elif name == "scale":
            xs, ys, zs = (_float_attr(child, k) for k in "xyz")
            if with_forward:
                _scale(trm, xs, ys, zs)
            _inv_scale(inv, xs, ys, zs)
        elif name == "rotate":
            deg = _float_attr(child, "degrees")
            x, y, z = (_float_attr(child, k) for k in "xyz")
            if with_forward:
                _rotate(trm, deg, x, y, z)
            _inv_rotate(inv, deg, x, y, z)
        elif name == "children" and not with_forward:
            children.append(child)
    if with_forward:
        rec["m"] = trm[:12]
    rec["invm"] = inv[:12]
    return xs, ys, zs, rd, children


class _Loader:
    def __init__(self):
        self.prims: list[np.void] = []
        self.bvs: list[np.void] = []
        self.density: list[float] = []

    def load_geometry(self, geometry):
        """Scene.cpp:191-282."""
        for el in _elements(geometry):
            rec = np.zeros((), PRIM_DTYPE)
            ptype = el.get("type")
            bound_mod = F32(1.0)
            if el.get("isBounding") is not None:
                bound_mod = F32(-1.0) if el.get("isBounding") == "true" else F32(1.0)
            if ptype in ("cylinderSurface", "taperedCylinderSurface", "frustum"):
                small = F32(1.0)
                node = el.find("smallRadius")
                if node is not None:
                    v = _scan_float(node.get("value"))
                    small = small if v is None else v
                if small == F32(1.0):
                    rec["type"] = CYLINDER
                else:
                    rec["type"] = FRUSTUM
                    rec["util1"] = small
                rec["util2"] = bound_mod
            elif ptype == "annulus":
                rec["type"] = ANNULUS
                sr_node, lr_node = el.find("smallRadius"), el.find("largeRadius")
                if sr_node is None or lr_node is None:
                    raise ValueError("annulus needs smallRadius and largeRadius (Scene.cpp:250-251)")
                sr = _scan_float(sr_node.get("value"))
                lr = _scan_float(lr_node.get("value"))
                sr = F32(0.0) if sr is None else sr
                lr = F32(0.0) if lr is None else lr
                rec["util1"] = F32(sr * sr)
                rec["util2"] = F32(lr * lr)
            elif ptype == "rectangle":
                rec["type"] = RECTANGLE
            elif ptype == "disc":
                rec["type"] = DISC
            elif ptype == "sphere":
                rec["type"] = SPHERE
                rec["util2"] = bound_mod
            else:
                continue  # type none is not stored (Scene.cpp:275)
            self.density.append(self.init_primitive(el, rec))
            self.prims.append(rec)

    def init_primitive(self, el, rec):
        """Scene.cpp:296-390."""
        if not _has_child_node(el):
            return 1.0  # the reference returns before touching the matrices
        xs, ys, zs, rd, _ = _init_transform(el, rec, True)
        rec["rayDensity"] = _ray_density(int(rec["type"]), rd, xs, ys, zs,
                                         F32(rec["util1"]), F32(rec["util2"]))
        return float(rd)

    def load_bounding_volumes(self, geometry):
        """Scene.cpp:97-175."""
        for el in _elements(geometry):
            rec = np.zeros((), BV_DTYPE)
            if el.get("intermediateCheck") is not None:
                rec["settings"] = 1
            ptype = el.get("type")
            if ptype in ("cylinderSurface", "taperedCylinderSurface", "frustum"):
                small = F32(1.0)
                node = el.find("smallRadius")
                if node is not None:
                    v = _scan_float(node.get("value"))
                    small = small if v is None else v
                if small == F32(1.0):
                    rec["type"] = CYLINDER
                else:
                    rec["type"] = FRUSTUM
                    rec["util1"] = small
            elif ptype == "annulus":
                rec["type"] = ANNULUS
                sr = _scan_float(el.find("smallRadius").get("value"))
                lr = _scan_float(el.find("largeRadius").get("value"))
                rec["util1"] = F32(sr * sr)
                rec["util2"] = F32(lr * lr)
            elif ptype == "rectangle":
                rec["type"] = RECTANGLE
            elif ptype == "disc":
                rec["type"] = DISC
            elif ptype == "sphere":
                rec["type"] = SPHERE
            else:
                continue
            self.init_bv(el, rec)
            self.bvs.append(rec)

    def init_bv(self, el, rec):
        """Scene.cpp:392-452 (children are loaded in document order)."""
        if not _has_child_node(el):
            return
        inv = _identity()
        for child in _elements(el):
            name = child.tag
            if name == "translation":
                _inv_translate(inv, *(_float_attr(child, k) for k in "xyz"))
            elif name == "scale":
                _inv_scale(inv, *(_float_attr(child, k) for k in "xyz"))
            elif name == "rotate":
                deg = _float_attr(child, "degrees")
                _inv_rotate(inv, deg, *(_float_attr(child, k) for k in "xyz"))
            elif name == "children":
                rec["objStartIndex"] = len(self.prims)
                self.load_geometry(child)
                rec["objEndIndex"] = len(self.prims)
        rec["invm"] = inv[:12]


def parse_scene_xml(text: str) -> Scene:
    """Scene::readScene (Scene.cpp:24-52) on an XML string."""
    parser = ET.XMLParser(target=ET.TreeBuilder(insert_comments=True))
    root = ET.fromstring(text, parser=parser)
    if root.tag != "project":
        raise ValueError("scene XML needs a <project> root")
    settings, geometry = root.find("settings"), root.find("geometry")
    if settings is None or geometry is None:
        raise ValueError("scene XML needs <settings> and <geometry>")
    sc = Scene()
    for child in _elements(settings):          # Scene.cpp:64-84
        if child.tag == "globalRayDensity":
            sc.global_ray_density = float(_float_attr(child, "value"))
        elif child.tag == "useBoundingVolumes":
            sc.use_bounding_volumes = _bool_attr(child, "value")
        elif child.tag == "description":
            sc.description = (child.text or "").strip()
    ld = _Loader()
    if sc.use_bounding_volumes:
        ld.load_bounding_volumes(geometry)
    else:
        ld.load_geometry(geometry)
    sc.primitives = np.array(ld.prims, PRIM_DTYPE) if ld.prims else np.zeros(0, PRIM_DTYPE)
    sc.density = np.array(ld.density, np.float64)
    sc.bounding_volumes = np.array(ld.bvs, BV_DTYPE) if ld.bvs else np.zeros(0, BV_DTYPE)
    return sc


def read_scene(path: str | Path) -> Scene:
    """Scene::readScene (Scene.cpp:24-52) on a file."""
    text = Path(path).read_text()
    return parse_scene_xml(text)
