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
