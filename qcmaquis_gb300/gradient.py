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

The right environments are kept for all sites (or, with ``store_every`` = k,
every k-th one, the others recomputed per segment) and the left one is carried
along the chain.  At a converged ground
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


class CheckpointedRight:
    """Right environments R[1..L] of a left-to-right pass, with every k-th kept.

    ``step(j, R[j+1])`` gives R[j]; R[L] is ``last``.  The constructor runs the
    right-to-left pass once and keeps R[L] and every R[j] with j % k == 0; reading an
    R[i] that was not kept recomputes the segment from the next kept one above it down
    to i (held until the pass moves on).  Reads go upward in i and ``release(i)`` drops
    R[i] once site i-1 is done, so at most about L/k + k environments are resident
    instead of L + 1, for at most one more step per site.  Every R[i] is the value the
    keep-all pass gives (the same steps on the same inputs)."""

    def __init__(self, step, last, L: int, k: int = 1, nbytes=None):
        self.step = step
        self.k = max(1, int(k))
        self.nbytes = nbytes
        self.stored = {L: last}
        self.segment = {}
        self.env_bytes = {}
        self.peak_bytes = 0
        cur = last
        for j in range(L - 1, 0, -1):
            cur = step(j, cur)
            if nbytes is not None:
                self.env_bytes[j] = nbytes(cur)
            if self.k == 1 or j % self.k == 0:
                self.stored[j] = cur
            self._track()

    def __getitem__(self, i: int):
        if i in self.stored:
            return self.stored[i]
        if i not in self.segment:
            self.segment.clear()
            top = min(x for x in self.stored if x > i)
            b = self.stored[top]
            for jj in range(top - 1, i - 1, -1):
                b = self.step(jj, b)
                self.segment[jj] = b
                self._track()
        return self.segment[i]

    def _track(self):
        """The most bytes the resident environments have held (with ``nbytes``)."""
        if self.nbytes is not None:
            held = sum(self.nbytes(b) for b in list(self.stored.values()) + list(self.segment.values()))
            self.peak_bytes = max(self.peak_bytes, held)

    def release(self, i: int):
        self.stored.pop(i, None)
        self.segment.pop(i, None)

    def resident(self) -> int:
        return len(self.stored) + len(self.segment)


def term_gradients(mpo, mps: List[DeviceMPSTensor], nelec: int, twoS: int = 0, engine: Optional[Engine] = None,
                   device="cuda", store_every: int = 1, stats: Optional[dict] = None):
    """d<Psi|H|Psi>/d(term scale) of every term of every site tensor of ``mpo`` (one
    energy-gradient plan per site with the full environments L[j], R[j+1]).

    ``store_every`` = k > 1 keeps only every k-th right environment (and R[L]) from the
    first right-to-left pass and recomputes the others segment by segment when the
    left-to-right pass reaches them: about L/k + k environments are resident instead
    of L + 1, for one more boundary step per site.  The results are bitwise those of
    k = 1 (the same boundary steps on the same inputs).
    Returns (per-site gradients, per-site FMpo, <Psi|H|Psi> per site, seconds of the
    site plans); ``stats``, when given, receives the byte size of every right
    environment, the most environments resident at once and the per-site energies."""
    import time
    from .sweep import _ones_boundary
    engine = engine or Engine(device)
    L = len(mpo)
    rights = CheckpointedRight(lambda j, b: engine.overlap_mpo_right_step(mps[j], b, mpo[j]),
                               _ones_boundary((nelec, twoS), engine.device), L, store_every,
                               nbytes=lambda b: b.data.numel() * b.data.element_size())
    peak = rights.resident()
    left = _ones_boundary((0, 0), engine.device)
    e_sites, grads, fmpos = [], [], []
    t0 = time.time()
    for j in range(L):
        f = N.FMpo(mpo[j])
        t = mps[j]
        R = rights[j + 1]
        peak = max(peak, rights.resident())
        p = N.plan_energy_gradient(t.phys_i, t.left_i, t.right_i, t.layout, left.layout, R.layout, f,
                                   engine.hermitian)
        p.upload()
        out = torch.empty(max(p.out_elems, 1), dtype=torch.float64, device=engine.device)
        engine.run(p, ket=t.data, left=left, right=R, out=out, precision=N.PREC_FP64)
        g = out[:f.n_terms].cpu().numpy()
        e_sites.append(float(np.dot(f.term_scale[:f.n_terms], g)))
        grads.append(g)
        fmpos.append(f)
        if j + 1 < L:
            left = engine.overlap_mpo_left_step(t, left, mpo[j])
        rights.release(j + 1)
        del R
    torch.cuda.synchronize()
    if stats is not None:
        stats.update(env_bytes=rights.env_bytes, peak_resident_environments=peak, site_energies=e_sites,
                     peak_environment_bytes=rights.peak_bytes)
    return grads, fmpos, e_sites, time.time() - t0


def energy_gradient(model, mps: List[DeviceMPSTensor], nelec: int, twoS: int = 0,
                    engine: Optional[Engine] = None, device="cuda", store_every: int = 1,
                    stats: Optional[dict] = None) -> EnergyGradient:
    """dE/d(integral) for every integral of ``model`` at the MPS ``mps`` (left-paired
    device tensors).  ``store_every`` > 1 recomputes right environments instead of
    storing them all (``term_gradients``)."""
    from .sweep import overlap
    engine = engine or Engine(device)
    mpo = TaggedMPOMaker(model, merge_site_terms=False).create_mpo()
    grads, fmpos, e_sites, site_s = term_gradients(mpo, mps, nelec, twoS, engine, store_every=store_every,
                                                   stats=stats)
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
