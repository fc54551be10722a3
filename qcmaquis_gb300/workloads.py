"""Benchmark and test workloads.

``sigma_workload`` builds the sigma-vector microbenchmark: one H_eff.psi on the
middle two sites of an L-orbital, N-electron, S=0 SU2U1 Hamiltonian with
seeded synthetic integrals (diagonal in ``diag_range``), a random normalised
MPS at bond dimension ``m`` over valid quantum-number sectors (left-canonical
left of the pair, right-canonical right of it) and boundaries built on the
GPU from that MPS.  Everything is seeded; nothing is read from disk.
"""
from __future__ import annotations

import time
from dataclasses import dataclass, field
from typing import Dict, List

import numpy as np

from .block_matrix import BlockMatrix
from .integrals import synthetic_integral_map
from .model import QCModel
from .mpo import make_mpo, make_twosite_mpo
from .mps import bond_indices, left_canonical_chain, right_canonical_chain, two_site_random
from .symmetry import Index, index_product


@dataclass
class SigmaWorkload:
    L: int
    nelec: int
    m: int
    site: int
    model: object
    mpo: object
    ts_mpo: object
    psi_host: object
    left_sites: List
    right_sites: List
    timings: Dict[str, float] = field(default_factory=dict)
    psi: object = None
    left: object = None
    right: object = None

    def describe(self) -> Dict:
        return {"L": self.L, "N": self.nelec, "S": 0, "m": self.m, "sites": [self.site, self.site + 1],
                "mpo_bond_dims": [self.ts_mpo.row_dim, self.ts_mpo.col_dim],
                "bond_left": self.psi_host.left_i.sum_of_sizes(), "bond_right": self.psi_host.right_i.sum_of_sizes(),
                "psi_elements": int(self.psi_host.data.num_elements())}


def build_sigma_host(L=24, nelec=24, m=1024, seed=1, diag_range=(-3.0, -0.3), site=None) -> SigmaWorkload:
    t0 = time.time()
    ints = synthetic_integral_map(L, seed=seed, diag_range=diag_range)
    model = QCModel(L, ints, nelec)
    mpo = make_mpo(model)
    t1 = time.time()
    site = (L // 2 - 1) if site is None else site
    phys = model.phys
    bonds = bond_indices(L, phys, (nelec, 0), m)
    rng = np.random.default_rng(seed + 1000)
    lefts, lb = left_canonical_chain(phys, bonds, site, rng)
    rights, rb = right_canonical_chain(phys, bonds, L, site + 2, rng)
    phys2 = index_product(phys, phys)
    psi = two_site_random(phys2, lb, rb, rng)
    t2 = time.time()
    ts = make_twosite_mpo(mpo[site], mpo[site + 1], phys, phys)
    t3 = time.time()
    w = SigmaWorkload(L, nelec, m, site, model, mpo, ts, psi, lefts, rights)
    w.timings = {"mpo_s": t1 - t0, "mps_s": t2 - t1, "ts_mpo_s": t3 - t2}
    return w


def upload_sigma_workload(w: SigmaWorkload, engine) -> SigmaWorkload:
    """Build L[site] and R[site+2] on the GPU with the boundary-step plans."""
    from .engine import DeviceBoundary, DeviceMPSTensor
    t0 = time.time()
    phys = w.model.phys
    one = lambda c: BlockMatrix.from_indices(Index([(c, 1)]), Index([(c, 1)]), fill=1.0)
    left = DeviceBoundary.from_host([one((0, 0))], device=engine.device)
    for i, t in enumerate(w.left_sites):
        left = engine.overlap_mpo_left_step(DeviceMPSTensor.from_host(t, device=engine.device), left, w.mpo[i])
    right = DeviceBoundary.from_host([one((w.nelec, 0))], device=engine.device)
    for k in range(len(w.right_sites) - 1, -1, -1):
        i = w.site + 2 + k
        right = engine.overlap_mpo_right_step(DeviceMPSTensor.from_host(w.right_sites[k], device=engine.device),
                                              right, w.mpo[i])
    w.psi = DeviceMPSTensor.from_host(w.psi_host, device=engine.device)
    w.left, w.right = left, right
    import torch
    torch.cuda.synchronize()
    w.timings["boundaries_s"] = time.time() - t0
    return w


__all__ = ["SigmaWorkload", "build_sigma_host", "upload_sigma_workload"]
