"""Traced view factors against closed forms and FP64 quadrature (GPU).

1e8 rays from the emitter of each case, on the exact kernel (the reference's
method, bit-exact with the CPU restatement) and the mixed-precision kernel, with
a scale-relative self-hit threshold (eps = -1e-6: 1e-6 of the scene's bounding
diagonal) so that the reference's absolute EPS = 1e-3 (RayFactorGPU.cl:7), which
drops hits nearer than 1e-3 where surfaces meet, does not bias the estimate.
Requirement: |F - F_ref| <= 1e-4 + 3 sigma, sigma the binomial standard error.
"""
import math

import numpy as np
import pytest

from helpers import golden_scene
from rayfactorcl_gb300 import analytic
from rayfactorcl_gb300.generators import _Xml
from rayfactorcl_gb300.scene import parse_scene_xml
from rayfactorcl_gb300.tracer import PREC_EXACT, PREC_MIXED, Tracer

pytestmark = pytest.mark.gpu

RAYS = 100_000_000


def _coaxial_discs():
    x = _Xml("coaxial discs r=0.5, 1 apart")
    x.prim("disc", scale=(0.5, 0.5, 1.0))
    x.close()
    x.prim("disc", scale=(0.5, 0.5, 1.0), rotate=(180.0, (1.0, 0.0, 0.0)), translate=(0.0, 0.0, 1.0))
    x.close()
    return parse_scene_xml(x.text()), 0, 1, analytic.coaxial_discs(0.5, 0.5, 1.0)


def _concentric_cylinders():
    x = _Xml("concentric cylinders r=0.5 and 1, length 1")
    x.prim("cylinderSurface", small=1.0, scale=(0.5, 0.5, 1.0))
    x.close()
    x.prim("cylinderSurface", bounding=True, small=1.0, scale=(1.0, 1.0, 1.0))
    x.close()
    return parse_scene_xml(x.text()), 1, 0, analytic.concentric_cylinders(0.5, 1.0, 1.0)


def _sphere_disc():
    x = _Xml("sphere r=0.5 to a coaxial disc r=1 at 2 from its centre")
    x.prim("sphere", scale=(0.5, 0.5, 0.5))
    x.close()
    x.prim("disc", scale=(1.0, 1.0, 1.0), rotate=(180.0, (1.0, 0.0, 0.0)), translate=(0.0, 0.0, 2.0))
    x.close()
    return parse_scene_xml(x.text()), 0, 1, analytic.sphere_to_coaxial_disc(1.0, 2.0)


def _c77():
    sc = golden_scene("input-C77")  # cylinder r=2, length 1; annulus 2..3 around its base
    return sc, 0, 1, analytic.cylinder_to_base_annulus_quadrature(2.0, 1.0, 3.0)


def _c77_reverse():
    sc, _, _, f = _c77()
    return sc, 1, 0, f * (2 * math.pi * 2.0 * 1.0) / (math.pi * (9.0 - 4.0))  # reciprocity


CASES = {"coaxial_discs": _coaxial_discs, "concentric_cylinders": _concentric_cylinders,
         "sphere_to_disc": _sphere_disc, "C77_cylinder_to_annulus": _c77, "C77_annulus_to_cylinder": _c77_reverse}


@pytest.mark.parametrize("prec", [PREC_EXACT, PREC_MIXED])
@pytest.mark.parametrize("case", list(CASES))
def test_traced_view_factor(built_lib, case, prec):
    sc, i, j, ref = CASES[case]()
    rays = np.zeros(sc.n, np.int64)
    rays[i] = RAYS
    with Tracer(precision=prec, eps=-1e-6, key1=7) as t:
        t.set_scene(sc)
        hits, F = t.trace(rays)
    sigma = math.sqrt(ref * (1 - ref) / RAYS)
    assert abs(F[i, j] - ref) <= 1e-4 + 3 * sigma, (case, prec, F[i, j], ref, sigma)
    assert int(hits[i].sum()) <= RAYS
