"""The oracle's SU(2) recoupling coefficients (test infrastructure).

The reference takes 6j and 9j symbols from GSL (``gsl_sf_coupling_6j/9j``,
declared in ``bm/symmetry/gsl_coupling.h:18-23``; GSL is not vendored and has
no pinned version).  Here they follow the published closed forms, evaluated
in exact integer arithmetic with a single final square root:

* 6j: Racah's single-sum formula, {a b c; d e f} = T(abc) T(aef) T(dbf) T(dec)
  sum_t (-1)^t (t+1)! / prod (t - triad sums)! prod (quad sums - t)!, where
  T(xyz)^2 = (x+y-z)! (x-y+z)! (-x+y+z)! / (x+y+z+1)!;
* 9j: the sum over x of (-1)^{2x} (2x+1) {a b c; f i x} {d e f; b x h}
  {g h i; x a d} (Varshalovich 10.2.1, arguments of {a b c; d e f; g h i}).

Arguments are doubled spins, as in the GSL API.  The values are checked
against the reference's 9j table (``dmrg/tests/test_wigner.cpp:18-56``) and
against an independent exact evaluation (sympy) in the tests.

The coupling helpers restate ``SU2::mod_coupling`` and ``SU2::set_coupling``
(``gsl_coupling.h:155-204``) and ``conjugate_correction``
(``ct/non-abelian/gemm.hpp:17-46``).
"""
from __future__ import annotations

import math
from fractions import Fraction
from functools import lru_cache

from .qn import triangle


def _f(n: int) -> int:
    return math.factorial(n)


def _tri2(x: int, y: int, z: int) -> Fraction:
    """T(xyz)^2 for doubled spins x, y, z forming a triad."""
    return Fraction(_f((x + y - z) // 2) * _f((x - y + z) // 2) * _f((y + z - x) // 2), _f((x + y + z) // 2 + 1))


@lru_cache(maxsize=None)
def _racah6j(a: int, b: int, c: int, d: int, e: int, f: int):
    """(S, P) with {a b c; d e f} = S * sqrt(P), S and P exact rationals."""
    triads = ((a, b, c), (a, e, f), (d, b, f), (d, e, c))
    if not all(triangle(*t) for t in triads):
        return Fraction(0), Fraction(0)
    lo = max(sum(t) // 2 for t in triads)
    quads = ((a + b + d + e) // 2, (b + c + e + f) // 2, (a + c + d + f) // 2)
    hi = min(quads)
    S = Fraction(0)
    for t in range(lo, hi + 1):
        den = 1
        for tr in triads:
            den *= _f(t - sum(tr) // 2)
        for q in quads:
            den *= _f(q - t)
        term = Fraction(_f(t + 1), den)
        S += -term if t & 1 else term
    P = _tri2(a, b, c) * _tri2(a, e, f) * _tri2(d, b, f) * _tri2(d, e, c)
    return S, P


@lru_cache(maxsize=None)
def sixj(a: int, b: int, c: int, d: int, e: int, f: int) -> float:
    S, P = _racah6j(a, b, c, d, e, f)
    if S == 0 or P == 0:
        return 0.0
    return float(S) * math.sqrt(float(P))


@lru_cache(maxsize=None)
def ninej(a: int, b: int, c: int, d: int, e: int, f: int, g: int, h: int, i: int) -> float:
    """{a b c; d e f; g h i}, doubled spins."""
    rows_cols = ((a, b, c), (d, e, f), (g, h, i), (a, d, g), (b, e, h), (c, f, i))
    if not all(triangle(*t) for t in rows_cols):
        return 0.0
    x_lo = max(abs(a - i), abs(b - f), abs(d - h))
    x_hi = min(a + i, b + f, d + h)
    terms = []
    for x in range(x_lo, x_hi + 1, 2):
        s1, p1 = _racah6j(a, b, c, f, i, x)
        s2, p2 = _racah6j(d, e, f, b, x, h)
        s3, p3 = _racah6j(g, h, i, x, a, d)
        if s1 == 0 or s2 == 0 or s3 == 0:
            continue
        sgn = -1 if x & 1 else 1
        terms.append(sgn * (x + 1) * float(s1 * s2 * s3) * math.sqrt(float(p1 * p2 * p3)))
    return math.fsum(terms)


def mod_coupling(a, b, c, d, e, f, g, h, i) -> float:
    """``SU2::mod_coupling``: sqrt((g+1)(h+1)(c+1)(f+1)) times the 9j symbol."""
    return math.sqrt((g + 1.0) * (h + 1.0) * (c + 1.0) * (f + 1.0)) * ninej(a, b, c, d, e, f, g, h, i)


def set_coupling(a, b, c, d, e, f, g, h, i, init: float):
    """``SU2::set_coupling``: the four couplings of one sparse operator entry, indexed by
    (row spin == 2) + 2 * (column spin == 2); zero where the triangle fails."""
    pre = math.sqrt((i + 1.0) * (a + 1.0) / ((g + 1.0) * (c + 1.0))) * init
    out = [0.0, 0.0, 0.0, 0.0]
    if triangle(a, b, c):
        out[0] = pre * mod_coupling(a, b, c, d, e, f, g, h, i)
        out[2] = pre * mod_coupling(a, b, c, d, e, f, g, 2, i)
    if triangle(a, 2, c):
        out[1] = pre * mod_coupling(a, 2, c, d, e, f, g, h, i)
        out[3] = pre * mod_coupling(a, 2, c, d, e, f, g, 2, i)
    return out


def conjugate_correction(lc_spin: int, rc_spin: int, tensor_spin: int) -> float:
    """Factor of a Hermitian-partner boundary block (``ct/non-abelian/gemm.hpp:17-46``)."""
    S = min(lc_spin, rc_spin)
    diff = rc_spin - lc_spin
    if tensor_spin == 0:
        return 1.0
    if tensor_spin == 1:
        if diff == 0:
            return 0.0
        return -math.sqrt((S + 1.0) / (S + 2.0)) if diff > 0 else math.sqrt((S + 2.0) / (S + 1.0))
    if tensor_spin == 2:
        if diff == 0:
            return 1.0
        return -math.sqrt((S + 1.0) / (S + 3.0)) if diff > 0 else -math.sqrt((S + 3.0) / (S + 1.0))
    raise ValueError("Hermitian conjugate only defined for operators of rank <= 1")


# names used by the oracle's restatements
wigner6j = sixj
wigner9j = ninej

__all__ = ["sixj", "ninej", "wigner6j", "wigner9j", "mod_coupling", "set_coupling", "conjugate_correction"]
