"""Exact diagonalisation of the same Hamiltonian (tests only).

Builds H = sum t_pq a+_p,s a_q,s + 1/2 sum (pq|rs) a+_p,s a+_r,t a_s,t a_q,s + E_core
in the determinant basis at fixed (N, Sz) from the 8-fold-symmetric integral
map used by the reference (``tests/Fixtures/LiHFixture.h:29-94`` format:
1-based (i,j,k,l) for V, (i,j,0,0) for t, (0,0,0,0) for the core energy) and
returns the lowest eigenvalue of the requested total spin.  This pins the
integral conventions and the SU2 MPO independently of any DMRG code.
"""
from __future__ import annotations

import itertools

import numpy as np


def expand_integrals(L, ints):
    t = np.zeros((L, L))
    V = np.zeros((L, L, L, L))
    core = 0.0
    for (i, j, k, l), v in ints.items():
        if i == 0 and j == 0 and k == 0 and l == 0:
            core += v
        elif k == 0 and l == 0:
            t[i - 1, j - 1] = v
            t[j - 1, i - 1] = v
        else:
            i, j, k, l = i - 1, j - 1, k - 1, l - 1
            for a, b, c, d in [(i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k),
                               (k, l, i, j), (l, k, i, j), (k, l, j, i), (l, k, j, i)]:
                V[a, b, c, d] = v
    return t, V, core


def _apply_ann(det, p):
    if not (det >> p) & 1:
        return None, 0
    sign = -1 if bin(det & ((1 << p) - 1)).count("1") % 2 else 1
    return det ^ (1 << p), sign


def _apply_cre(det, p):
    if (det >> p) & 1:
        return None, 0
    sign = -1 if bin(det & ((1 << p) - 1)).count("1") % 2 else 1
    return det | (1 << p), sign


def fci_energies(L, ints, nelec, twoS=0, nroots=1):
    """Lowest eigenvalues with total spin S = twoS/2 (Sz = S sector filtered by S^2)."""
    return [e for e, _ in fci_states(L, ints, nelec, twoS, nroots)[0]]


def fci_rdms(L, dets, vec):
    """Spin-summed RDMs of a CI vector: gamma_pq = sum_s <a+_ps a_qs> and the
    chemist-ordered Gamma_pqrs = sum_st <a+_ps a+_rt a_st a_qs>, so that
    E = core + sum t_pq gamma_pq + 1/2 sum (pq|rs) Gamma_pqrs."""
    index = {d: i for i, d in enumerate(dets)}
    g1 = np.zeros((L, L))
    g2 = np.zeros((L, L, L, L))
    for col, d in enumerate(dets):
        c = vec[col]
        if c == 0.0:
            continue
        for p in range(L):
            for q in range(L):
                for s in (0, 1):
                    d1, s1 = _apply_ann(d, 2 * q + s)
                    if d1 is None:
                        continue
                    d2, s2 = _apply_cre(d1, 2 * p + s)
                    if d2 is None or d2 not in index:
                        continue
                    g1[p, q] += vec[index[d2]] * c * s1 * s2
        for p, q, r, s_ in itertools.product(range(L), repeat=4):
            for sa in (0, 1):
                for sb in (0, 1):
                    d1, h1 = _apply_ann(d, 2 * q + sa)
                    if d1 is None:
                        continue
                    d2, h2 = _apply_ann(d1, 2 * s_ + sb)
                    if d2 is None:
                        continue
                    d3, h3 = _apply_cre(d2, 2 * r + sb)
                    if d3 is None:
                        continue
                    d4, h4 = _apply_cre(d3, 2 * p + sa)
                    if d4 is None or d4 not in index:
                        continue
                    g2[p, q, r, s_] += vec[index[d4]] * c * h1 * h2 * h3 * h4
    return g1, g2


def fci_states(L, ints, nelec, twoS=0, nroots=1):
    """([(energy, CI vector)], determinants) of the lowest states with total spin twoS/2."""
    t, V, core = expand_integrals(L, ints)
    nalpha = (nelec + twoS) // 2
    nbeta = nelec - nalpha
    # spin orbital p -> bit 2*orb + spin
    dets = []
    for ao in itertools.combinations(range(L), nalpha):
        for bo in itertools.combinations(range(L), nbeta):
            d = 0
            for o in ao:
                d |= 1 << (2 * o)
            for o in bo:
                d |= 1 << (2 * o + 1)
            dets.append(d)
    index = {d: i for i, d in enumerate(dets)}
    n = len(dets)
    H = np.zeros((n, n))
    for col, d in enumerate(dets):
        H[col, col] += core
        for p in range(L):
            for q in range(L):
                if t[p, q] == 0.0:
                    continue
                for s in (0, 1):
                    d1, s1 = _apply_ann(d, 2 * q + s)
                    if d1 is None:
                        continue
                    d2, s2 = _apply_cre(d1, 2 * p + s)
                    if d2 is None:
                        continue
                    H[index[d2], col] += t[p, q] * s1 * s2
        for p, q, r, s_ in itertools.product(range(L), repeat=4):
            v = V[p, q, r, s_]
            if v == 0.0:
                continue
            for sa in (0, 1):
                for sb in (0, 1):
                    # a+_{p sa} a+_{r sb} a_{s sb} a_{q sa}
                    d1, g1 = _apply_ann(d, 2 * q + sa)
                    if d1 is None:
                        continue
                    d2, g2 = _apply_ann(d1, 2 * s_ + sb)
                    if d2 is None:
                        continue
                    d3, g3 = _apply_cre(d2, 2 * r + sb)
                    if d3 is None:
                        continue
                    d4, g4 = _apply_cre(d3, 2 * p + sa)
                    if d4 is None:
                        continue
                    H[index[d4], col] += 0.5 * v * g1 * g2 * g3 * g4
    # S^2 = S- S+ + Sz(Sz+1)
    S2 = np.zeros((n, n))
    sz = 0.5 * (nalpha - nbeta)
    for col, d in enumerate(dets):
        S2[col, col] += sz * (sz + 1)
        for p in range(L):
            for q in range(L):
                # S- S+ = sum_pq a+_{p b} a_{p a} a+_{q a} a_{q b}
                d1, g1 = _apply_ann(d, 2 * q + 1)
                if d1 is None:
                    continue
                d2, g2 = _apply_cre(d1, 2 * q)
                if d2 is None:
                    continue
                d3, g3 = _apply_ann(d2, 2 * p)
                if d3 is None:
                    continue
                d4, g4 = _apply_cre(d3, 2 * p + 1)
                if d4 is None:
                    continue
                S2[index[d4], col] += g1 * g2 * g3 * g4
    w, U = np.linalg.eigh(H)
    target = 0.25 * twoS * (twoS + 2)
    out = []
    for k in range(n):
        s2 = float(U[:, k] @ S2 @ U[:, k])
        if abs(s2 - target) < 1e-6:
            out.append((float(w[k]), U[:, k].copy()))
            if len(out) == nroots:
                break
    return out, dets
