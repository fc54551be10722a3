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


def dense_to_op(m: np.ndarray, states=STATES) -> SiteOperator:
    """SiteOperator (blocks keyed (phys_in, phys_out)) of a dense <out|O|in> matrix over
    a local basis of one state per charge (``states``: the charge of each position)."""
    bm = BlockMatrix()
    d = len(states)
    for i in range(d):
        for o in range(d):
            if m[o, i] != 0.0:
                bm.insert_block(np.array([[float(m[o, i])]]), states[i], states[o])
    return SiteOperator(bm, SpinDescriptor(), {})


class _OpRegistry:
    """Local operators by their dense matrix: a product equal to a registered one up to
    a scale reuses its tag (the scale goes into the term's coefficient); every new
    operator is registered together with its transpose (its Hermitian partner), so
    the partner of a tag is exactly its adjoint."""

    def __init__(self, th: TagHandler, states=STATES):
        self.th = th
        self.states = states
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
        t = self.th.register_op(dense_to_op(m, self.states), FERMIONIC if fermionic else BOSONIC)
        self.by_key[k] = (t, first)
        self.dense.append(m)
        mt = m.T.copy()
        kt, firstt = self._key(mt)
        if kt not in self.by_key:
            tt = self.th.register_op(dense_to_op(mt, self.states), FERMIONIC if fermionic else BOSONIC)
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


class AbelianChemModel:
    """The terms of the quantum-chemistry Hamiltonian over an abelian group, from its
    spin-orbital operator form.  A subclass fixes the local basis (``states``: the
    charge of each local state, one state per charge), the local matrices
    (``_ladder``: identity "I", fill "F" and the ladder operators) and where a spin
    orbital lives (``_so``); the spin orbitals are ordered for the Jordan-Wigner
    string as the sites are, and within a site in ``_so``'s order."""

    symmetry = ""
    states: List = []
    _memo_enabled = True   # memoised local operators (``_site_tags``); False: recomputed for every term

    def _so(self, p: int, spin: int, create: bool) -> Tuple[int, str]:
        """(site, ladder name) of c+_{p spin} (``create``) or c_{p spin}."""
        raise NotImplementedError

    def _ladder(self) -> Dict[str, np.ndarray]:
        raise NotImplementedError

    def _init_operators(self):
        self.tag_handler = TagHandler()
        self._reg = _OpRegistry(self.tag_handler, self.states)
        lad = self._ladder()
        self._lad = lad
        self.ops = Operators()
        self.ops.ident, _ = self._reg.tag(lad["I"], False)
        self.ops.ident_full = self.ops.ident
        self.ops.fill, _ = self._reg.tag(lad["F"], False)
        self.terms: List[Term] = []
        self._memo: Dict[Tuple, Tuple] = {}

    def _site_ops(self, ladder: List[Tuple[int, str]]):
        """One (site, local matrix, fermionic) per site of a product of ladder operators
        given in operator order as (site, name), or None if the product vanishes."""
        lad = self._lad
        d = len(self.states)
        sites = sorted({s for s, _ in ladder})
        out = []
        for k in sites:
            m = np.eye(d)
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

    def _site_tags(self, ladder: List[Tuple[int, str]]):
        """(site, tag, scale) per site of a product of ladder operators, or None if the
        product vanishes -- ``_site_ops`` followed by the registry lookup, memoised
        per site on the operator pattern that fixes the local matrix there (the
        names of the operators on the site and a filling for every later operator,
        in operator order).  The first appearance of a pattern registers its
        operator exactly as the unmemoised form does, so tags come out the same."""
        if not self._memo_enabled:
            so = self._site_ops(ladder)
            if so is None:
                return None
            return [(k, *self._reg.tag(m, ferm)) for k, m, ferm in so]
        out = []
        for k in sorted({s for s, _ in ladder}):
            sig = tuple(name if s == k else "F" for s, name in ladder if s >= k)
            hit = self._memo.get(sig)
            if hit is None:
                lad = self._lad
                m = np.eye(len(self.states))
                nferm = 0
                for name in sig:
                    m = m @ lad[name]
                    nferm += name != "F"
                if not np.any(m != 0.0):
                    hit = (None, 0.0)
                else:
                    hit = self._reg.tag(m, nferm % 2 == 1)
                self._memo[sig] = hit
            if hit[0] is None:
                return None
            out.append((k, hit[0], hit[1]))
        return out

    def _create_terms(self, norb: int):
        """H = sum_pq t_pq sum_s c+_ps c_qs + 1/2 sum_pqrs (pq|rs) sum_st c+_ps c+_rt c_ts c_qs
        + E_core over ``norb`` spatial orbitals."""
        t, V, core, src = expand_integrals(norb, self.integrals)
        merged: Dict[Tuple, Term] = {}

        def add(coeff: float, ladder, key):
            if abs(coeff) <= 0.0:
                return
            st = self._site_tags(ladder)
            if st is None:
                return
            term = Term(coeff, False)
            scale = 1.0
            for k, tag, sc in st:
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
        for p in range(norb):
            for q in range(norb):
                if abs(t[p, q]) > cut:
                    for sp in (0, 1):
                        add(t[p, q], [self._so(p, sp, True), self._so(q, sp, False)], src[(p, q)])
        for p in range(norb):
            for q in range(norb):
                for r in range(norb):
                    for s in range(norb):
                        v = V[p, q, r, s]
                        if abs(v) <= cut:
                            continue
                        for sa in (0, 1):
                            for sb in (0, 1):
                                add(0.5 * v, [self._so(p, sa, True), self._so(r, sb, True),
                                              self._so(s, sb, False), self._so(q, sa, False)],
                                    src[(p, q, r, s)])
        if core != 0.0 or () in src:
            term = Term(core, False)
            term.push(0, self.ops.ident)
            term.src = {src[()]: 1.0} if () in src else {}
            self.terms.append(term)
        self.terms.extend(x for x in merged.values() if x.coeff != 0.0)


class TwoU1Model(AbelianChemModel):
    """The TwoU1 quantum-chemistry model: ``L`` orbitals, ``n_up`` and ``n_down``
    electrons (the reference's ``u1_total_charge1`` / ``u1_total_charge2``)."""

    symmetry = "2u1"
    states = STATES

    def __init__(self, L: int, integrals: Dict[Tuple[int, int, int, int], float], n_up: int, n_down: int,
                 integral_cutoff: float = 1e-20):
        self.L = L
        self.n_up, self.n_down = n_up, n_down
        self.nelec = n_up + n_down
        self.right_end = (n_up, n_down)
        self.phys = phys_index()
        self.integrals = integrals
        self.integral_cutoff = integral_cutoff
        self._init_operators()
        self._create_terms(L)

    def _ladder(self) -> Dict[str, np.ndarray]:
        return _ladder()

    def _so(self, p: int, spin: int, create: bool) -> Tuple[int, str]:
        return p, ("c" if create else "d") + ("u" if spin == 0 else "d")


__all__ = ["AbelianChemModel", "TwoU1Model", "phys_index", "expand_integrals", "dense_to_op"]
