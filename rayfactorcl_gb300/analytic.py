"""Closed-form diffuse view factors used to state the error of traced F.

Each formula follows from the double-area integral
F_12 = 1/A_1 * int int cos(t1) cos(t2) / (pi s^2) dA_2 dA_1 by the standard
contour/disc-algebra reductions; the test suite checks each one against FP64
Gauss-Legendre quadrature of that integral.
"""
from __future__ import annotations

import math

import numpy as np


def coaxial_discs(r1: float, r2: float, h: float) -> float:
    """Disc of radius r1 to a parallel coaxial disc of radius r2 at distance h."""
    R1, R2 = r1 / h, r2 / h
    X = 1.0 + (1.0 + R2 * R2) / (R1 * R1)
    return 0.5 * (X - math.sqrt(X * X - 4.0 * (R2 / R1) ** 2))


def disc_to_ring(r: float, a: float, b: float, h: float) -> float:
    """Disc of radius r to a parallel coaxial ring a <= rho <= b at distance h."""
    return coaxial_discs(r, b, h) - coaxial_discs(r, a, h)


def ring_to_ring(a1: float, b1: float, a2: float, b2: float, h: float) -> float:
    """Ring [a1,b1] to a parallel coaxial ring [a2,b2] at distance h (disc algebra)."""
    def AF(r, s):  # A(disc r) * F(disc r -> disc s)
        return math.pi * r * r * coaxial_discs(r, s, h) if r > 0 else 0.0
    num = (AF(b1, b2) - AF(b1, a2)) - (AF(a1, b2) - AF(a1, a2))
    return num / (math.pi * (b1 * b1 - a1 * a1))


def perpendicular_rectangles(w: float, h: float, l: float) -> float:
    """Rectangle w x l to a perpendicular rectangle h x l sharing the edge of length l."""
    W, H = w / l, h / l
    W2, H2 = W * W, H * H
    s = math.sqrt(W2 + H2)
    t = W * math.atan(1 / W) + H * math.atan(1 / H) - s * math.atan(1 / s)
    a = (1 + W2) * (1 + H2) / (1 + W2 + H2)
    b = (W2 * (1 + W2 + H2) / ((1 + W2) * (W2 + H2))) ** W2
    c = (H2 * (1 + H2 + W2) / ((1 + H2) * (H2 + W2))) ** H2
    return (t + 0.25 * math.log(a * b * c)) / (math.pi * W)


def sphere_to_rectangle_corner(a: float, b: float, h: float) -> float:
    """Sphere whose centre is at height h above one corner of an a x b rectangle."""
    A, B = a / h, b / h
    return math.atan(A * B / math.sqrt(1 + A * A + B * B)) / (4 * math.pi)


def sphere_to_coaxial_disc(a: float, h: float) -> float:
    """Sphere to a disc of radius a whose centre is h from the sphere's centre."""
    return 0.5 * (1.0 - 1.0 / math.sqrt(1.0 + (a / h) ** 2))


def enclosure3(r: float = 0.5, h: float = 1.0) -> np.ndarray:
    """Two coaxial discs of radius r at distance h closed by the cylinder between
    them (order: disc, disc, cylinder)."""
    f12 = coaxial_discs(r, r, h)
    a_d, a_c = math.pi * r * r, 2 * math.pi * r * h
    f13 = 1.0 - f12
    f31 = a_d * f13 / a_c
    return np.array([[0.0, f12, f13], [f12, 0.0, f13], [f31, f31, 1.0 - 2 * f31]])


def areas_of(ws_areas) -> np.ndarray:
    return np.asarray(ws_areas, np.float64)


def concentric_cylinders(r1: float, r2: float, l: float) -> float:
    """Inner surface of a cylinder of radius r2 to the outer surface of a coaxial
    cylinder of radius r1 < r2, both of length l with common ends (F_21)."""
    R, L = r2 / r1, l / r1
    A = L * L + R * R - 1.0
    B = L * L - R * R + 1.0
    inner = (math.sqrt((A + 2.0) ** 2 - (2.0 * R) ** 2) * math.acos(B / (R * A))
             + B * math.asin(1.0 / R) - 0.5 * math.pi * A)
    return 1.0 / R - (math.acos(B / A) - inner / (2.0 * L)) / (math.pi * R)


def concentric_cylinders_quadrature(r1: float, r2: float, l: float) -> float:
    """The same view factor by FP64 quadrature of the double-area integral.  With
    the outer point at angle 0 and the inner one at angle phi, both axial integrals
    have closed forms (int int dz1 dz2 / (q + (z1-z2)^2)^2 over [0,l]^2), leaving one
    integral over |phi| < acos(r1/r2), where the inner surface faces the outer point."""
    from scipy.integrate import quad

    def axial(q):
        rq = math.sqrt(q)
        j1 = l / (2 * q * (q + l * l)) + math.atan(l / rq) / (2 * q * rq)
        j2 = 1 / (2 * q) - 1 / (2 * (q + l * l))
        return 2 * (l * j1 - j2)

    def f(phi):
        c = math.cos(phi)
        q = r1 * r1 + r2 * r2 - 2 * r1 * r2 * c
        return (r2 - r1 * c) * (r2 * c - r1) * axial(q)

    p0 = math.acos(r1 / r2)
    val, _ = quad(f, -p0, p0, epsabs=1e-14, epsrel=1e-12, limit=200)
    return r1 * val / (math.pi * l)


def cylinder_to_base_annulus_quadrature(r1: float, l: float, r2: float) -> float:
    """Outer surface of a cylinder (radius r1, length l) to the annulus r1 <= rho <= r2
    around its base, in the base plane and facing the cylinder's side (the
    sample geometry input-C77.xml).  The double-area integral with the cylinder
    point at angle 0: the axial integral int_0^l z dz / (q + z^2)^2 and the
    angular one over |phi| < acos(r1/rho) (where the annulus point lies in front
    of the cylinder surface; int dphi / (a - b cos phi) by the half-angle
    tangent) are closed forms, leaving one FP64 quadrature over rho.  The
    cylinder is convex and the annulus flat, so nothing blocks the lines."""
    from scipy.integrate import quad

    def g(rho, dm, a):  # int_{-p0}^{p0} (rho cos phi - r1) / (a - b cos phi) dphi, b = 2 rho r1, dm = a - b
        b = 2 * rho * r1
        p0 = math.acos(min(1.0, r1 / rho))
        root = math.sqrt(dm * (a + b))
        return -(rho / b) * 2 * p0 + (rho * a / b - r1) * 4 / root * math.atan(
            math.sqrt((a + b) / dm) * math.tan(0.5 * p0))

    def f(t):  # rho = r1 + t^2 spreads the edge's square-root behaviour
        rho = r1 + t * t
        if t == 0.0:
            return 0.0
        e2 = (rho - r1) ** 2  # a - b without cancellation
        a0 = rho * rho + r1 * r1
        return 2 * t * rho * 0.5 * (g(rho, e2, a0) - g(rho, e2 + l * l, a0 + l * l))

    val, _ = quad(f, 0.0, math.sqrt(r2 - r1), epsabs=1e-14, epsrel=1e-12, limit=400)
    return val / (math.pi * l)
