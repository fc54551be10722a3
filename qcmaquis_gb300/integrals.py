"""Synthetic molecular integrals and the integral-map format.

Integral maps use the layout of the reference's fixtures
(``dmrg/tests/Fixtures/LiHFixture.h:29-94``): 1-based keys ``(i,j,k,l)`` for the
two-electron integrals (ij|kl), ``(i,j,0,0)`` for the one-electron t_ij and
``(0,0,0,0)`` for the core energy; only the 8-fold-unique representatives are
stored, in the canonical order produced by ``align``
(``dmrg/framework/dmrg/utils/align.h:19-27``).

The generator makes the seeded synthetic Hamiltonians the benchmark workloads
are defined on: t symmetric with an evenly spaced diagonal in ``diag_range``
and N(0, 0.05) off-diagonals; V_pqrs = sum_{k<16} L^k_pq L^k_rs with L^k
symmetric N(0, 0.1), which is positive semidefinite with 8-fold symmetry.
"""
from __future__ import annotations

from typing import Dict, Tuple

import numpy as np

from .model import align


def synthetic_integrals(L: int, seed: int = 0, diag_range=(-2.0, -0.5), rank: int = 16,
                        offdiag_sigma: float = 0.05, chol_sigma: float = 0.1, core: float = 0.0):
    rng = np.random.default_rng(seed)
    t = np.diag(np.linspace(diag_range[0], diag_range[1], L))
    off = rng.normal(0.0, offdiag_sigma, size=(L, L))
    off = np.triu(off, 1)
    t = t + off + off.T
    V = np.zeros((L, L, L, L))
    for _ in range(rank):
        Lk = rng.normal(0.0, chol_sigma, size=(L, L))
        Lk = np.triu(Lk) + np.triu(Lk, 1).T
        V += np.einsum("pq,rs->pqrs", Lk, Lk)
    return t, V, core


def to_integral_map(t: np.ndarray, V: np.ndarray, core: float = 0.0, cutoff: float = 0.0) -> Dict[Tuple[int, int, int, int], float]:
    L = t.shape[0]
    out: Dict[Tuple[int, int, int, int], float] = {}
    for i in range(L):
        for j in range(i + 1):
            for k in range(L):
                for l in range(k + 1):
                    key = align(i, j, k, l)
                    if key != (i, j, k, l):
                        continue
                    v = float(V[i, j, k, l])
                    if abs(v) > cutoff:
                        out[(i + 1, j + 1, k + 1, l + 1)] = v
    for i in range(L):
        for j in range(i + 1):
            v = float(t[i, j])
            if abs(v) > cutoff:
                out[(i + 1, j + 1, 0, 0)] = v
    out[(0, 0, 0, 0)] = float(core)
    return out


def synthetic_integral_map(L: int, seed: int = 0, diag_range=(-2.0, -0.5)):
    t, V, core = synthetic_integrals(L, seed, diag_range)
    return to_integral_map(t, V, core)


def write_fcidump(path: str, L: int, nelec: int, twoS: int, ints) -> None:
    """Plain FCIDUMP (header + ``value i j k l`` lines), as read by
    ``models/chem/parse_integrals.h:43-214``."""
    with open(path, "w") as f:
        f.write(f" &FCI NORB={L},NELEC={nelec},MS2={twoS},\n  ORBSYM=" + "1," * L + "\n  ISYM=1,\n &END\n")
        for (i, j, k, l), v in ints.items():
            f.write(f"{v: .16e} {i} {j} {k} {l}\n")


def read_fcidump(path: str):
    ints = {}
    with open(path) as f:
        lines = f.readlines()
    body = lines[4:]
    for line in body:
        parts = line.split()
        if len(parts) != 5:
            continue
        v = float(parts[0])
        key = tuple(int(x) for x in parts[1:])
        ints[key] = v
    return ints


__all__ = ["synthetic_integrals", "to_integral_map", "synthetic_integral_map", "write_fcidump", "read_fcidump"]
