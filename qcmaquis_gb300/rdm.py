"""Spin-free 1- and 2-RDMs of an SU2U1 MPS through the adjoint.

The reference measures every RDM element as a separate expectation value:
for each index tuple it builds an MPO from that element's spin-summed operator
terms and contracts it with the state (``models/measurements/
tagged_nrankrdm_su2u1.h:83-193``): the 1-RDM element (p1, p2) from one
positional two-term (p1 != p2, scale sqrt(2)) or the number operator (p1 = p2),
the 2-RDM element (p1, p2, p3, p4) from ``SpinSumSU2::V_term(1, p1, p2, p3,
p4)``, over the tuples of ``iterate_nrdm<2>`` (``measurements_details.h:308-327``).

Here all elements' terms go into ONE MPO, every term its own labelled scale, and
one pass of energy-gradient plans along the chain gives d<Psi|O|Psi>/d(scale)
for every term at once; an element is the sum of its terms' coefficients times
those derivatives (the expectation value is linear in each scale), divided by
<Psi|Psi>.  The measurement MPO is not Hermitian, so its boundaries and plans
contract every MPO bond (no Hermitian-partner shortcut).
"""
from __future__ import annotations

import math
import types
from typing import Dict, List, Optional, Tuple

import numpy as np

from .engine import Engine
from .model import SpinSum, Term, tm_positional_two_term
from .mpo import TaggedMPOMaker


def iterate_nrdm2(L: int) -> List[Tuple[int, int, int, int]]:
    """The 2-RDM index tuples for bra = ket (``measurements_details.h:308-327``)."""
    out = []
    for p1 in range(L):
        for p2 in range(L):
            for p3 in range(min(p1, p2), L):
                for p4 in range(p3, L):
                    out.append((p1, p2, p3, p4))
    return out


def rdm_terms(model, rank: int):
    """(element index tuples, terms, owning element of each term) of the 1-RDM (rank 1)
    or 2-RDM (rank 2) measurement."""
    c = model.col
    L = model.L
    elems, terms, owner = [], [], []
    if rank == 1:
        for p1 in range(L):
            for p2 in range(p1, L):
                if p1 != p2:
                    ts = [tm_positional_two_term(True, math.sqrt(2.0), p1, p2, c.create.couple_down,
                                                 c.create.fill_couple_up, c.destroy.couple_down,
                                                 c.destroy.fill_couple_up)]
                else:
                    t = Term(1.0)
                    t.push(p1, c.count.no_couple)
                    ts = [t]
                elems.append((p1, p2))
                for t in ts:
                    terms.append(t)
                    owner.append(len(elems) - 1)
    elif rank == 2:
        ss = SpinSum(c)
        for pos in iterate_nrdm2(L):
            elems.append(pos)
            for t in ss.V_term(1.0, *pos):
                terms.append(t)
                owner.append(len(elems) - 1)
    else:
        raise ValueError("rank must be 1 or 2")
    return elems, terms, owner


def measurement_mpo(model, terms):
    """One MPO holding every term as its own labelled scale (label = term index)."""
    src = types.SimpleNamespace(L=model.L, tag_handler=model.tag_handler, ops=model.ops, terms=terms)
    return TaggedMPOMaker(src, merge_site_terms=False).create_mpo()


def elements_from_term_gradients(mpo, terms, owner, n_elems, site_grads, fmpos, norm) -> np.ndarray:
    """sum over an element's terms of coeff * d<O>/d(scale), divided by <Psi|Psi>."""
    d = np.zeros(len(terms))
    for g, f in zip(site_grads, fmpos):
        for tt, lab in enumerate(f.term_label):
            if lab is not None:
                d[lab] += g[tt]
    vals = np.zeros(n_elems)
    for k, t in enumerate(terms):
        vals[owner[k]] += t.coeff * d[k]
    return vals / norm


def measure_rdm(model, mps, nelec: int, rank: int = 2, twoS: int = 0, engine: Optional[Engine] = None
                ) -> Dict[tuple, float]:
    """{index tuple: value} of the spin-free ``rank``-RDM of the device MPS ``mps``, the
    elements and their order as the reference's measurement produces them."""
    from .gradient import term_gradients
    from .sweep import overlap
    elems, terms, owner = rdm_terms(model, rank)
    mpo = measurement_mpo(model, terms)
    # a measurement MPO is not Hermitian (an element's terms come without their
    # conjugates), so every MPO bond is contracted: no Hermitian-partner shortcut
    if engine is None or engine.hermitian:
        engine = Engine(mps[0].data.device, hermitian=False)
    grads, fmpos, _, _ = term_gradients(mpo, mps, nelec, twoS, engine)
    vals = elements_from_term_gradients(mpo, terms, owner, len(elems), grads, fmpos, overlap(mps))
    return dict(zip(elems, vals.tolist()))


__all__ = ["iterate_nrdm2", "rdm_terms", "measurement_mpo", "elements_from_term_gradients", "measure_rdm"]
