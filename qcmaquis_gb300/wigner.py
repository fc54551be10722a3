"""Wigner 6j / 9j symbols and the SU(2) coupling factors built on them.

The reference takes its recoupling coefficients from GSL
(``gsl_sf_coupling_6j/9j``, declared in
``dmrg/framework/dmrg/block_matrix/symmetry/gsl_coupling.h:18-23``); GSL is not
vendored there and not installed here, so the symbols are computed from the
Racah closed form: the 6j symbol as the Racah single sum, and the 9j symbol
as the standard sum over products of three 6j symbols.  All arguments are
doubled spins, as in the GSL API.  The sums are evaluated in exact rational
arithmetic and only the final square root is taken in floating point, so each
value is correctly rounded to within one or two ulps.

The coupling helpers restate ``mod_coupling`` / ``set_coupling``
(``gsl_coupling.h:163-204``) and ``conjugate_correction``
(``mp_tensors/contractions/non-abelian/gemm.hpp:17-46``).
"""
from __future__ import annotations

import math
from fractions import Fraction
from functools import lru_cache

from .symmetry import triangle


def _fact(n: int) -> int:
    return math.factorial(n)


def _delta_sq(a2: int, b2: int, c2: int) -> Fraction:
    """Triangle coefficient squared, doubled-spin arguments."""
    return Fraction(_fact((a2 + b2 - c2) // 2) * _fact((a2 - b2 + c2) // 2) * _fact((-a2 + b2 + c2) // 2),
                    _fact((a2 + b2 + c2) // 2 + 1))


@lru_cache(maxsize=None)
def _sixj_parts(j1, j2, j3, j4, j5, j6):
    """Return (sum, prefactor^2) of the Racah formula, both exact rationals."""
    if not (triangle(j1, j2, j3) and triangle(j1, j5, j6) and triangle(j4, j2, j6) and triangle(j4, j5, j3)):
        return Fraction(0), Fraction(0)
    a1 = (j1 + j2 + j3) // 2
    a2 = (j1 + j5 + j6) // 2
    a3 = (j4 + j2 + j6) // 2
    a4 = (j4 + j5 + j3) // 2
    b1 = (j1 + j2 + j4 + j5) // 2
    b2 = (j2 + j3 + j5 + j6) // 2
    b3 = (j3 + j1 + j6 + j4) // 2
    tmin = max(a1, a2, a3, a4)
    tmax = min(b1, b2, b3)
    s = Fraction(0)
    for t in range(tmin, tmax + 1):
        num = _fact(t + 1)
        den = (_fact(t - a1) * _fact(t - a2) * _fact(t - a3) * _fact(t - a4)
               * _fact(b1 - t) * _fact(b2 - t) * _fact(b3 - t))
        term = Fraction(num, den)
        s += -term if (t % 2) else term
    pref = _delta_sq(j1, j2, j3) * _delta_sq(j1, j5, j6) * _delta_sq(j4, j2, j6) * _delta_sq(j4, j5, j3)
    return s, pref


@lru_cache(maxsize=None)
def wigner6j(j1: int, j2: int, j3: int, j4: int, j5: int, j6: int) -> float:
    """{j1 j2 j3; j4 j5 j6} with doubled-spin arguments."""
    s, pref = _sixj_parts(j1, j2, j3, j4, j5, j6)
    if s == 0 or pref == 0:
        return 0.0
    return float(s) * math.sqrt(float(pref))


@lru_cache(maxsize=None)
def wigner9j(a: int, b: int, c: int, d: int, e: int, f: int, g: int, h: int, i: int) -> float:
    """{a b c; d e f; g h i} with doubled-spin arguments.

    9j = sum_x (-1)^{2x} (2x+1) {a d g; h i x} {b e h; d x f} {c f i; x a b}
    """
    if not (triangle(a, b, c) and triangle(d, e, f) and triangle(g, h, i)
            and triangle(a, d, g) and triangle(b, e, h) and triangle(c, f, i)):
        return 0.0
    xmin = max(abs(a - i), abs(h - d), abs(b - f))
    xmax = min(a + i, h + d, b + f)
    # exact accumulation: each 6j = S * sqrt(P); the product of three is
    # S1 S2 S3 sqrt(P1 P2 P3).  Terms share no common radicand in general, so
    # accumulate in floating point with compensated summation.
    total = 0.0
    comp = 0.0
    for x in range(xmin, xmax + 1, 2):
        s1, p1 = _sixj_parts(a, d, g, h, i, x)
        if s1 == 0:
            continue
        s2, p2 = _sixj_parts(b, e, h, d, x, f)
        if s2 == 0:
            continue
        s3, p3 = _sixj_parts(c, f, i, x, a, b)
        if s3 == 0:
            continue
        sign = -1.0 if (x % 2) else 1.0  # (-1)^{2x} with x doubled: odd doubled x -> half-integer
        term = sign * (x + 1) * float(s1 * s2 * s3) * math.sqrt(float(p1 * p2 * p3))
        y = term - comp
        t = total + y
        comp = (t - total) - y
        total = t
    return total


def mod_coupling(a, b, c, d, e, f, g, h, i) -> float:
    """sqrt((g+1)(h+1)(c+1)(f+1)) * 9j  (``gsl_coupling.h:163-172``)."""
    return math.sqrt((g + 1.0) * (h + 1.0) * (c + 1.0) * (f + 1.0)) * wigner9j(a, b, c, d, e, f, g, h, i)


def set_coupling(a, b, c, d, e, f, g, h, i, init: float):
    """The four coupling cases of one MPO entry (``gsl_coupling.h:175-204``).

    Case index: 0 = neither sparse-entry spin is 2, 1 = row spin 2,
    2 = column spin 2, 3 = both.
    """
    prefactor = math.sqrt((i + 1.0) * (a + 1.0) / ((g + 1.0) * (c + 1.0))) * init
    out = [0.0, 0.0, 0.0, 0.0]
    if triangle(a, b, c):
        out[0] = prefactor * mod_coupling(a, b, c, d, e, f, g, h, i)
        out[2] = prefactor * mod_coupling(a, b, c, d, e, f, g, 2, i)
    if triangle(a, 2, c):
        out[1] = prefactor * mod_coupling(a, 2, c, d, e, f, g, h, i)
        out[3] = prefactor * mod_coupling(a, 2, c, d, e, f, g, 2, i)
    return out


def conjugate_correction(lc_spin: int, rc_spin: int, tensor_spin: int) -> float:
    """Phase factor of a Hermitian-conjugate boundary block (``gemm.hpp:17-46``)."""
    S = min(rc_spin, lc_spin)
    diff = rc_spin - lc_spin
    if tensor_spin == 0:
        return 1.0
    if tensor_spin == 1:
        if diff > 0:
            return -math.sqrt((S + 1.0) / (S + 2.0))
        if diff < 0:
            return math.sqrt((S + 2.0) / (S + 1.0))
        return 0.0
    if tensor_spin == 2:
        if diff > 0:
            return -math.sqrt((S + 1.0) / (S + 3.0))
        if diff < 0:
            return -math.sqrt((S + 3.0) / (S + 1.0))
        return 1.0
    raise ValueError("hermitian conjugate for reduced tensor operators only implemented up to rank 1")


__all__ = ["wigner6j", "wigner9j", "mod_coupling", "set_coupling", "conjugate_correction"]
