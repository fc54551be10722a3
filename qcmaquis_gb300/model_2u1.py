"""Quantum-chemistry Hamiltonian in TwoU1 symmetry (conserved N_up and N_down).

The abelian counterpart of ``model.QCModel``, for the reference's ``2u1``
chemistry model (``dmrg/framework/dmrg/models/chem/2u1/model.hpp:11-140``):

* charges (N_up, N_down); one orbital has the four states
  |0> = (0,0), |up> = (1,0), |dn> = (0,1), |updn> = (1,1), one state each, with
  |updn> = c+_up c+_dn |0> (so c+_dn carries the local sign of the up
  electron, as the reference's ``create_down = fill * create_down``);
* fermion signs by the Jordan-Wigner string: the orbitals are ordered site by
  site (up before down), c_{i s} = F_0 ... F_{i-1} (x) c~_{i s} with
  F = (-1)^(n_up + n_dn) and c~ acting on site i only;
* H = sum_pq t_pq sum_s c+_ps c_qs + 1/2 sum_pqrs (pq|rs) sum_st
  c+_ps c+_rt c_ts c_qs + E_core, from the same 8-fold-symmetric integral map as
  the SU2U1 model (``tests/Fixtures/LiHFixture.h`` key format).

The terms are generated here from that operator form, not by the reference's
``TermMaker``/``ChemHelper`` case analysis: every spin-orbital product is
brought to one local operator per site (the product, in operator order, of the
site's own ladder operators and of F for every operator acting further right),
equal operator strings are merged, and the tagged MPO builder
(``mpo.TaggedMPOMaker``) adds the fill strings between the sites.  The
Hamiltonian is the same operator as the reference's, so energies agree; the
MPO's bond labelling is this builder's own.

Operator blocks are stored as (phys_in, phys_out) with entry (in, out) =
<out|O|in>, the orientation the contraction kernels read (as in ``model.py``).
"""
from __future__ import annotations

from typing import Dict, List, Tuple

import numpy as np

from .block_matrix import BlockMatrix
from .model import BOSONIC, FERMIONIC, Operators, TagHandler, Term
from .site_operator import SiteOperator, SpinDescriptor
from .symmetry import Index

# local basis (index = position in the dense 4x4 matrices below)
STATES = [(0, 0), (1, 0), (0, 1), (1, 1)]
EMPTY, UP, DN, UPDN = range(4)


def phys_index() -> Index:
    """Physical basis of one orbital, descending: (1,1), (1,0), (0,1), (0,0)."""
    return Index([((1, 1), 1), ((1, 0), 1), ((0, 1), 1), ((0, 0), 1)])


def _ladder() -> Dict[str, np.ndarray]:
    """Dense physical matrices <out|O|in> of the local operators."""
    cu = np.zeros((4, 4))
    cu[UP, EMPTY] = 1.0      # c+_up |0> = |up>
    cu[UPDN, DN] = 1.0       # c+_up |dn> = c+_up c+_dn |0> = |updn>
    cd = np.zeros((4, 4))
    cd[DN, EMPTY] = 1.0      # c+_dn |0> = |dn>
    cd[UPDN, UP] = -1.0      # c+_dn |up> = c+_dn c+_up |0> = -|updn>
    fill = np.diag([1.0, -1.0, -1.0, 1.0])
    return {"cu": cu, "cd": cd, "du": cu.T.copy(), "dd": cd.T.copy(), "F": fill, "I": np.eye(4)}


def dense_to_op(m: np.ndarray) -> SiteOperator:
    """SiteOperator (blocks keyed (phys_in, phys_out)) of a dense <out|O|in> matrix."""
    bm = BlockMatrix()
    for i in range(4):
        for o in range(4):
            if m[o, i] != 0.0:
                bm.insert_block(np.array([[float(m[o, i])]]), STATES[i], STATES[o])
    return SiteOperator(bm, SpinDescriptor(), {})


class _OpRegistry:
    """Local operators by their dense matrix: a product equal to a registered one up to
    a scale reuses its tag (the scale goes into the term's coefficient); every new
    operator is registered together with its transpose (its Hermitian partner), so
    the partner of a tag is exactly its adjoint."""

    def __init__(self, th: TagHandler):
        self.th = th
        self.by_key: Dict[bytes, Tuple[int, float]] = {}
        self.dense: List[np.ndarray] = []

    @staticmethod
    def _key(m: np.ndarray) -> Tuple[bytes, float]:
        flat = m.ravel()
        nz = np.flatnonzero(flat)
        first = flat[nz[0]]
        return np.round(m / first, 12).tobytes(), first

    def tag(self, m: np.ndarray, fermionic: bool) -> Tuple[int, float]:
        """(tag, scale) with m = scale * operator(tag)."""
        k, first = self._key(m)
        if k in self.by_key:
            t, f0 = self.by_key[k]
            return t, first / f0
        t = self.th.register_op(dense_to_op(m), FERMIONIC if fermionic else BOSONIC)
        self.by_key[k] = (t, first)
        self.dense.append(m)
        mt = m.T.copy()
        kt, firstt = self._key(mt)
        if kt not in self.by_key:
            tt = self.th.register_op(dense_to_op(mt), FERMIONIC if fermionic else BOSONIC)
            self.by_key[kt] = (tt, firstt)
            self.th.hermitian_pair(t, tt)
        return t, 1.0


def expand_integrals(L: int, ints) -> Tuple[np.ndarray, np.ndarray, float, Dict]:
    """Full t_pq, (pq|rs) and the core energy of an 8-fold-symmetric integral map, and
    for every full index the map key it came from (provenance of the coefficients)."""
    t = np.zeros((L, L))
    V = np.zeros((L, L, L, L))
    core = 0.0
    src: Dict = {}
    for key, v in ints.items():
        i, j, k, l = key
        if i == 0 and j == 0 and k == 0 and l == 0:
            core += v
            src[()] = key
        elif k == 0 and l == 0:
            for a, b in ((i - 1, j - 1), (j - 1, i - 1)):
                t[a, b] = v
                src[(a, b)] = key
        else:
            i, j, k, l = i - 1, j - 1, k - 1, l - 1
            for idx in [(i, j, k, l), (j, i, k, l), (i, j, l, k), (j, i, l, k),
                        (k, l, i, j), (l, k, i, j), (k, l, j, i), (l, k, j, i)]:
                V[idx] = v
                src[idx] = key
    return t, V, core, src


class TwoU1Model:
    """The TwoU1 quantum-chemistry model: ``L`` orbitals, ``n_up`` and ``n_down``
    electrons (the reference's ``u1_total_charge1`` / ``u1_total_charge2``)."""

    symmetry = "2u1"

    def __init__(self, L: int, integrals: Dict[Tuple[int, int, int, int], float], n_up: int, n_down: int,
                 integral_cutoff: float = 1e-20):
        self.L = L
        self.n_up, self.n_down = n_up, n_down
        self.nelec = n_up + n_down
        self.right_end = (n_up, n_down)
        self.phys = phys_index()
        self.integrals = integrals
        self.integral_cutoff = integral_cutoff
        self.tag_handler = TagHandler()
        self._reg = _OpRegistry(self.tag_handler)
        lad = _ladder()
        self._lad = lad
        self.ops = Operators()
        self.ops.ident, _ = self._reg.tag(lad["I"], False)
        self.ops.ident_full = self.ops.ident
        self.ops.fill, _ = self._reg.tag(lad["F"], False)
        self.terms: List[Term] = []
        self._create_terms()

    def _site_ops(self, ladder: List[Tuple[int, str]]):
        """One (site, local matrix, fermionic) per site of a product of ladder operators
        given in operator order as (site, name), or None if the product vanishes."""
        lad = self._lad
        sites = sorted({s for s, _ in ladder})
        out = []
        for k in sites:
            m = np.eye(4)
            nferm = 0
            for s, name in ladder:
                if s == k:
                    m = m @ lad[name]
                    nferm += 1
                elif s > k:
                    m = m @ lad["F"]
            if not np.any(m != 0.0):
                return None
            out.append((k, m, nferm % 2 == 1))
        return out

    def _create_terms(self):
        L = self.L
        t, V, core, src = expand_integrals(L, self.integrals)
        merged: Dict[Tuple, Term] = {}

        def add(coeff: float, ladder, key):
            if abs(coeff) <= 0.0:
                return
            so = self._site_ops(ladder)
            if so is None:
                return
            term = Term(coeff, False)
            scale = 1.0
            for k, m, ferm in so:
                tag, sc = self._reg.tag(m, ferm)
                scale *= sc
                term.push(k, tag)
            term.coeff = coeff * scale
            term.src = {key: scale * (coeff / self._unit[key]) if self._unit[key] != 0.0 else scale}
            sig = tuple(term.ops)
            if sig in merged:
                merged[sig].coeff += term.coeff
                for u, f in term.src.items():
                    merged[sig].src[u] = merged[sig].src.get(u, 0.0) + f
            else:
                merged[sig] = term

        self._unit = {k: v for k, v in self.integrals.items()}
        cut = self.integral_cutoff
        for p in range(L):
            for q in range(L):
                if abs(t[p, q]) > cut:
                    for c, d in (("cu", "du"), ("cd", "dd")):
                        add(t[p, q], [(p, c), (q, d)], src[(p, q)])
        cre = {0: "cu", 1: "cd"}
        ann = {0: "du", 1: "dd"}
        for p in range(L):
            for q in range(L):
                for r in range(L):
                    for s in range(L):
                        v = V[p, q, r, s]
                        if abs(v) <= cut:
                            continue
                        for sa in (0, 1):
                            for sb in (0, 1):
                                add(0.5 * v, [(p, cre[sa]), (r, cre[sb]), (s, ann[sb]), (q, ann[sa])],
                                    src[(p, q, r, s)])
        if core != 0.0 or () in src:
            term = Term(core, False)
            term.push(0, self.ops.ident)
            term.src = {src[()]: 1.0} if () in src else {}
            self.terms.append(term)
        self.terms.extend(x for x in merged.values() if x.coeff != 0.0)


__all__ = ["TwoU1Model", "phys_index", "expand_integrals", "dense_to_op"]
