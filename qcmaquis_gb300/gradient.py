"""Gradient of the DMRG energy with respect to the Hamiltonian's integrals, on
the GPU (the adjoint of the local energy).

For an MPS Psi (any gauge) and the SU2U1 MPO H, E = <Psi|H|Psi>/<Psi|Psi> +
E_core is linear in every MPO term scale.  At site j, with the full
environments L[j] (sites < j) and R[j+1] (sites > j), the local energy
<psi_j| H_eff psi_j> is <Psi|H|Psi>; its gradient with respect to the site-j
term scales comes from one native energy-gradient plan (K1, the adjoint of K3
and per-term dots of the K2 tables, ``qcm_plan_energy_gradient``).  The MPO is
built with every model term as its own labelled scale
(``TaggedMPOMaker(merge_site_terms=False)``) and every model term records its
coefficient as a linear combination of integrals (``Term.src``), so
dE/d(integral) is the chain rule over those two maps.

The right environments are kept for all sites and the left one is carried along
the chain, so at most L + 1 boundaries are resident.  At a converged ground
state the integral gradient is the spin-summed RDM data: dE/dt_pq =
gamma_pq + gamma_qp (p != q), dE/d(pq|rs) = 1/2 sum of the chemist-ordered
Gamma over the 8-fold copies of the integral (the reference obtains RDMs by
separate expectation values instead,
``models/measurements/tagged_nrankrdm_su2u1.h``).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, List, Optional

import numpy as np
import torch

from . import native as N
from .engine import DeviceBoundary, DeviceMPSTensor, Engine
from .mpo import TaggedMPOMaker


@dataclass
class EnergyGradient:
    energy: float                      # <H>/<Psi|Psi> + core
    norm: float                        # <Psi|Psi>
    d_integrals: Dict[tuple, float]    # dE/d(value) per key of the integral map
    d_terms: np.ndarray                # dE/d(coefficient) per model term (normalised energy)
    site_seconds: float = 0.0


def chain_to_integrals(model, mpo, site_grads: List[np.ndarray], fmpos: List[N.FMpo], norm: float):
    """dE/d(model term coefficient) and dE/d(integral) of the normalised energy from the
    per-site gradients dE_raw/d(term scale) (flattened term order of each FMpo)."""
    d_coeff = np.zeros(len(model.terms))
    for g, f in zip(site_grads, fmpos):
        for tt, lab in enumerate(f.term_label):
            if lab is not None:
                d_coeff[lab] += g[tt]
    d_coeff /= norm
    for lab in mpo.core_labels:
        d_coeff[lab] = 1.0
    d_int: Dict[tuple, float] = {}
    for lab, term in enumerate(model.terms):
        for u, fct in term.src.items():
            d_int[u] = d_int.get(u, 0.0) + fct * d_coeff[lab]
    return d_coeff, d_int


def term_gradients(mpo, mps: List[DeviceMPSTensor], nelec: int, twoS: int = 0, engine: Optional[Engine] = None,
                   device="cuda"):
    """d<Psi|H|Psi>/d(term scale) of every term of every site tensor of ``mpo`` (one
    energy-gradient plan per site with the full environments L[j], R[j+1]).
    Returns (per-site gradients, per-site FMpo, <Psi|H|Psi> per site, seconds of the
    site plans)."""
    import time
    from .sweep import _ones_boundary
    engine = engine or Engine(device)
    L = len(mpo)
    right_end = (nelec, twoS)
    right: List[Optional[DeviceBoundary]] = [None] * (L + 1)
    right[L] = _ones_boundary(right_end, engine.device)
    for j in range(L - 1, 0, -1):
        right[j] = engine.overlap_mpo_right_step(mps[j], right[j + 1], mpo[j])
    left = _ones_boundary((0, 0), engine.device)
    e_sites, grads, fmpos = [], [], []
    t0 = time.time()
    for j in range(L):
        f = N.FMpo(mpo[j])
        t = mps[j]
        p = N.plan_energy_gradient(t.phys_i, t.left_i, t.right_i, t.layout, left.layout, right[j + 1].layout, f,
                                   engine.hermitian)
        p.upload()
        out = torch.empty(max(p.out_elems, 1), dtype=torch.float64, device=engine.device)
        engine.run(p, ket=t.data, left=left, right=right[j + 1], out=out, precision=N.PREC_FP64)
        g = out[:f.n_terms].cpu().numpy()
        e_sites.append(float(np.dot(f.term_scale[:f.n_terms], g)))
        grads.append(g)
        fmpos.append(f)
        if j + 1 < L:
            left = engine.overlap_mpo_left_step(t, left, mpo[j])
        right[j + 1] = None
    torch.cuda.synchronize()
    return grads, fmpos, e_sites, time.time() - t0


def energy_gradient(model, mps: List[DeviceMPSTensor], nelec: int, twoS: int = 0,
                    engine: Optional[Engine] = None, device="cuda") -> EnergyGradient:
    """dE/d(integral) for every integral of ``model`` at the MPS ``mps`` (left-paired
    device tensors)."""
    from .sweep import overlap
    engine = engine or Engine(device)
    mpo = TaggedMPOMaker(model, merge_site_terms=False).create_mpo()
    grads, fmpos, e_sites, site_s = term_gradients(mpo, mps, nelec, twoS, engine)
    nrm = overlap(mps)
    e_raw = float(np.mean(e_sites))
    d_coeff, d_int = chain_to_integrals(model, mpo, grads, fmpos, nrm)
    return EnergyGradient(energy=e_raw / nrm + mpo.core_energy, norm=nrm, d_integrals=d_int, d_terms=d_coeff,
                          site_seconds=site_s)


def rdm_sums_from_gamma(L: int, keys, g1: np.ndarray, g2: np.ndarray) -> Dict[tuple, float]:
    """dE/d(integral) implied by spin-summed RDMs (gamma_pq, chemist Gamma_pqrs) for the
    1-based keys of an integral map: t (i,j,0,0) -> gamma_ij + gamma_ji (i != j) or
    gamma_ii; (ij|kl) -> 1/2 sum of Gamma over the distinct 8-fold copies; core -> 1."""
    out = {}
    for key in keys:
        i, j, k, l = key
        if i == 0 and j == 0 and k == 0 and l == 0:
            out[key] = 1.0
        elif k == 0 and l == 0:
            a, b = i - 1, j - 1
            out[key] = g1[a, b] + (g1[b, a] if a != b else 0.0)
        else:
            a, b, c, d = i - 1, j - 1, k - 1, l - 1
            copies = {(a, b, c, d), (b, a, c, d), (a, b, d, c), (b, a, d, c),
                      (c, d, a, b), (d, c, a, b), (c, d, b, a), (d, c, b, a)}
            out[key] = 0.5 * sum(g2[x] for x in copies)
    return out


__all__ = ["EnergyGradient", "energy_gradient", "term_gradients", "chain_to_integrals", "rdm_sums_from_gamma"]
