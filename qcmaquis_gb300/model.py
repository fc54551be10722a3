"""Quantum-chemistry Hamiltonian in SU2U1 symmetry: site operators and terms.

Restates, for the spin-adapted (SU2U1) chemistry model:

* the operator table of ``TermMakerSU2::construct_operators``
  (``dmrg/framework/dmrg/models/chem/su2u1/term_maker.h:120-395``), registered
  in the same order so operator tags -- which order the MPO bond labels -- agree;
* ``TagHandler`` registration, Hermitian pairing and scale-aware de-duplication
  (``models/OperatorHandlers/TagHandler.hpp:33-96``, ``OpTable.hpp:10-35``,
  ``models/tag_detail.h:55-120``);
* term generation ``qc_su2::create_terms`` (``models/chem/su2u1/model.hpp:50-300``)
  with ``SpinSumSU2`` (``term_maker.h:548-793``) and the term collapse of
  ``ChemHelperSU2`` (``models/chem/su2u1/chem_helper.h:17-100``);
* integral index canonicalisation ``align`` (``dmrg/framework/dmrg/utils/align.h:19-27``).

Only real FP64 integrals and a single orbital type (all ``site_types`` 0,
i.e. no point-group labels) are supported, which covers every workload here.
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Tuple

import numpy as np

from .block_matrix import BlockMatrix
from .site_operator import SiteOperator, SpinDescriptor, op_equal
from .symmetry import Index

A = (2, 0)
B = (1, 1)
C = (1, -1)
D = (0, 0)

BOSONIC = 0
FERMIONIC = 1


def phys_index() -> Index:
    """Physical basis of one orbital: {(2,0),(1,1),(1,-1),(0,0)}, one state each."""
    return Index([(A, 1), (B, 1), (C, 1), (D, 1)])


def _op(entries, spin: SpinDescriptor = None) -> SiteOperator:
    op = SiteOperator(BlockMatrix(), spin if spin is not None else SpinDescriptor())
    for v, lc, rc in entries:
        op.insert_block(v, lc, rc)
    return op


class TagHandler:
    """Operator table with tags, fermion signs and Hermitian partners."""

    def __init__(self):
        self.ops: List[SiteOperator] = []
        self.sign: List[int] = []
        self.herm: List[int] = []

    def register_op(self, op: SiteOperator, kind: int) -> int:
        self.ops.append(op)
        self.sign.append(kind)
        self.herm.append(len(self.ops) - 1)
        return len(self.ops) - 1

    def checked_register(self, op: SiteOperator, kind: int):
        for t, ref in enumerate(self.ops):
            ok, scale = op_equal(ref, op)
            if ok:
                return t, scale
        return self.register_op(op, kind), 1.0

    def hermitian_pair(self, t1: int, t2: int):
        if self.herm[t1] == t2 and self.herm[t2] == t1:
            return
        assert self.herm[t1] == t1 and self.herm[t2] == t2
        self.herm[t1], self.herm[t2] = self.herm[t2], self.herm[t1]

    def herm_conj(self, t: int) -> int:
        return self.herm[t]

    def is_fermionic(self, t: int) -> bool:
        return bool(self.sign[t])

    def get_op(self, t: int) -> SiteOperator:
        return self.ops[t]


class Operators:
    pass


class Bundle:
    __slots__ = ("couple_up", "couple_down", "fill_couple_up", "fill_couple_down", "no_couple", "fill_no_couple")

    def __init__(self):
        for s in self.__slots__:
            setattr(self, s, None)


def construct_operators(th: TagHandler) -> Operators:
    s2 = math.sqrt(2.0)
    half_up = SpinDescriptor(1, 0, 1)
    half_down = SpinDescriptor(1, 1, 0)
    one_up = SpinDescriptor(2, 0, 2)
    one_flat = SpinDescriptor(2, 1, 1)
    one_down = SpinDescriptor(2, 2, 0)

    ops = {}
    ops["ident"] = _op([(1, A, A), (1, B, B), (1, C, C), (1, D, D)])
    ops["ident_full"] = _op([(1, A, A), (1, D, D), (1, B, B), (1, C, C), (1, B, C), (1, C, B)])
    ops["fill"] = _op([(1, A, A), (1, D, D), (-1, B, B), (-1, C, C), (-1, B, C), (-1, C, B)])
    ops["create_fill"] = _op([(s2, B, A), (s2, C, A), (1, D, B), (1, D, C)], half_up)
    ops["destroy"] = _op([(1, A, B), (1, A, C), (s2, B, D), (s2, C, D)], half_down)
    ops["destroy_fill"] = _op([(1, A, B), (1, A, C), (-s2, B, D), (-s2, C, D)], half_up)
    ops["create"] = _op([(s2, B, A), (s2, C, A), (-1, D, B), (-1, D, C)], half_down)

    def respin(name, sd):
        o = ops[name].copy()
        o.spin = sd
        return o

    ops["create_fill_couple_down"] = respin("create_fill", half_down)
    ops["destroy_fill_couple_down"] = respin("destroy_fill", half_down)
    ops["create_couple_up"] = respin("create", half_up)
    ops["destroy_couple_up"] = respin("destroy", half_up)

    ops["create_fill_count"] = _op([(s2, B, A), (s2, C, A)], half_up)
    ops["destroy_count"] = _op([(1, A, B), (1, A, C)], half_down)
    ops["destroy_fill_count"] = _op([(1, A, B), (1, A, C)], half_up)
    ops["create_count"] = _op([(s2, B, A), (s2, C, A)], half_down)

    ops["count"] = _op([(2, A, A), (1, B, B), (1, C, C)])
    ops["docc"] = _op([(1, A, A)])
    ops["e2d"] = _op([(1, D, A)])
    ops["d2e"] = _op([(1, A, D)])
    ops["count_fill"] = _op([(2, A, A), (-1, B, B), (-1, C, C), (-1, B, C), (-1, C, B)])

    f = math.sqrt(3.0 / 2.0)
    ops["flip_to_S2"] = _op([(f, B, B), (f, C, C), (f, B, C), (f, C, B)], one_up)
    ops["flip_to_S0"] = respin("flip_to_S2", one_down)
    ops["flip_S0"] = respin("flip_to_S2", one_flat)

    order = [
        ("ident", BOSONIC), ("ident_full", BOSONIC), ("fill", BOSONIC),
        ("create_fill", FERMIONIC), ("create", FERMIONIC), ("destroy_fill", FERMIONIC), ("destroy", FERMIONIC),
        ("create_fill_couple_down", FERMIONIC), ("destroy_fill_couple_down", FERMIONIC),
        ("create_couple_up", FERMIONIC), ("destroy_couple_up", FERMIONIC),
        ("create_fill_count", FERMIONIC), ("create_count", FERMIONIC),
        ("destroy_fill_count", FERMIONIC), ("destroy_count", FERMIONIC),
        ("count", BOSONIC), ("docc", BOSONIC), ("e2d", BOSONIC), ("d2e", BOSONIC),
        ("flip_S0", BOSONIC), ("flip_to_S2", BOSONIC), ("flip_to_S0", BOSONIC), ("count_fill", BOSONIC),
    ]
    tags = Operators()
    for name, kind in order:
        t, scale = th.checked_register(ops[name], kind)
        assert abs(scale - 1.0) == 0.0, name
        setattr(tags, name, t)

    for a, b in [("create_fill", "destroy_fill"), ("create", "destroy"), ("e2d", "d2e"),
                 ("create_fill_count", "destroy_fill_count"), ("create_count", "destroy_count"),
                 ("create_fill_couple_down", "destroy_fill_couple_down"),
                 ("create_couple_up", "destroy_couple_up")]:
        th.hermitian_pair(getattr(tags, a), getattr(tags, b))
    return tags


def construct_collection(t: Operators):
    col = Operators()
    for name in ["ident", "ident_full", "fill", "create", "destroy", "count", "flip", "e2d", "d2e",
                 "docc", "create_count", "destroy_count"]:
        setattr(col, name, Bundle())
    col.create.couple_up = t.create_couple_up
    col.create.couple_down = t.create
    col.create.fill_couple_up = t.create_fill
    col.create.fill_couple_down = t.create_fill_couple_down
    col.destroy.couple_up = t.destroy_couple_up
    col.destroy.couple_down = t.destroy
    col.destroy.fill_couple_up = t.destroy_fill
    col.destroy.fill_couple_down = t.destroy_fill_couple_down
    col.create_count.couple_down = t.create_count
    col.create_count.fill_couple_up = t.create_fill_count
    col.destroy_count.couple_down = t.destroy_count
    col.destroy_count.fill_couple_up = t.destroy_fill_count
    col.ident.no_couple = t.ident
    col.ident_full.no_couple = t.ident_full
    col.fill.no_couple = t.fill
    col.count.no_couple = t.count
    col.count.fill_no_couple = t.count_fill
    col.e2d.no_couple = t.e2d
    col.d2e.no_couple = t.d2e
    col.docc.no_couple = t.docc
    col.flip.no_couple = t.flip_S0
    col.flip.couple_up = t.flip_to_S2
    col.flip.couple_down = t.flip_to_S0
    return col


class Term:
    """``term_descriptor``: list of (position, tag) with a coefficient.  ``src`` records
    the coefficient as a linear combination of integral values,
    coeff = sum_u src[u] * integral[u] (keys of the integral map)."""
    __slots__ = ("ops", "coeff", "is_fermionic", "src")

    def __init__(self, coeff=1.0, fermionic=False):
        self.ops: List[Tuple[int, int]] = []
        self.coeff = coeff
        self.is_fermionic = fermionic
        self.src: Dict = {}

    def push(self, pos, tag):
        self.ops.append((pos, tag))

    def canonical_order(self):
        self.ops.sort(key=lambda x: x[0])

    def position(self, i):
        return self.ops[i][0]

    def tag(self, i):
        return self.ops[i][1]

    def __len__(self):
        return len(self.ops)

    def __repr__(self):
        return f"Term({self.coeff:+.6g}, {self.ops})"


def sgn4(i, j, k, l) -> bool:
    idx = [i, j, k, l]
    inv = 0
    for c1 in range(3):
        for c2 in range(c1 + 1, 4):
            if idx[c1] > idx[c2]:
                inv += 1
    return inv % 2 != 0


def align(i, j, k, l):
    """Canonical integral index order (``utils/align.h:19-27``)."""
    if i < j:
        i, j = j, i
    if k < l:
        k, l = l, k
    if i < k:
        i, k = k, i
        j, l = l, j
    if i == k and j < l:
        j, l = l, j
    return (i, j, k, l)


# ---------------------------------------------------------------- TermMaker
def tm_two_term(sign, scale, i, j, op1, op2):
    t = Term(scale, sign)
    t.push(i, op1)
    t.push(j, op2)
    return t


def tm_positional_two_term(sign, scale, i, j, op1, op1_fill, op2, op2_fill):
    t = Term(scale, sign)
    op1_use = op1_fill if i < j else op2_fill
    op2_use = op2 if i < j else op1
    if j < i and sign:
        t.coeff = -t.coeff
    start, end = min(i, j), max(i, j)
    t.push(start, op1_use)
    t.push(end, op2_use)
    return t


def tm_three_term(scale, pb, p1, p2, boson_op, boson_op_fill, op1, op1_fill, op2, op2_fill):
    t = Term(scale, True)
    op1_use = op1_fill if p1 < p2 else op2_fill
    op2_use = op2 if p1 < p2 else op1
    if (p1 < pb < p2) or (p2 < pb < p1):
        boson_use = boson_op_fill
    else:
        boson_use = boson_op
    if p2 < p1:
        t.coeff = -t.coeff
    start, end = min(p1, p2), max(p1, p2)
    t.push(pb, boson_use)
    t.push(start, op1_use)
    t.push(end, op2_use)
    t.canonical_order()
    return t


def tm_four_term(max_two_S, scale, i, j, k, l, op_i: Bundle, op_k: Bundle):
    t = Term(scale, True)
    if sgn4(i, j, k, l):
        t.coeff = -t.coeff
    st = sorted([(i, op_i), (j, op_i), (k, op_k), (l, op_k)], key=lambda x: x[0])
    if max_two_S == 2:
        t.push(st[0][0], st[0][1].fill_couple_up)
        t.push(st[1][0], st[1][1].couple_up)
        t.push(st[2][0], st[2][1].fill_couple_down)
        t.push(st[3][0], st[3][1].couple_down)
    else:
        t.push(st[0][0], st[0][1].fill_couple_up)
        t.push(st[1][0], st[1][1].couple_down)
        t.push(st[2][0], st[2][1].fill_couple_up)
        t.push(st[3][0], st[3][1].couple_down)
    return t


# ---------------------------------------------------------------- SpinSumSU2
class SpinSum:
    def __init__(self, col):
        self.c = col

    def V_term(self, me, i, k, l, j):
        n_unique = len(set([i, k, l, j]))
        if n_unique == 4:
            return self.four_term(me, i, k, l, j)
        if n_unique == 3:
            return self.three_term(me, i, k, l, j)
        if n_unique == 2:
            return self.two_term(me, i, k, l, j)
        t = Term(2.0 * me)
        t.push(i, self.c.docc.no_couple)
        return [t]

    def two_term(self, me, i, k, l, j):
        c = self.c
        if i == j and k == l and j != k:
            return [tm_two_term(False, me, i, k, c.count.no_couple, c.count.no_couple)]
        if i == k and j == l and j != k:
            return [tm_two_term(False, 2.0 * me, i, j, c.e2d.no_couple, c.d2e.no_couple)]
        if i == l and j == k and i != j:
            return [tm_positional_two_term(False, math.sqrt(3.0) * me, i, j, c.flip.couple_down, c.flip.couple_up,
                                           c.flip.couple_down, c.flip.couple_up),
                    tm_two_term(False, -0.5 * me, i, j, c.count.no_couple, c.count.no_couple)]
        if (i == k == l) or (k == l == j) or (i == l == j) or (i == k == j):
            if i == k and k == l:
                s, p = i, j
            elif k == l and l == j:
                s, p = j, i
            elif i == l and l == j:
                s, p = i, k
            else:
                s, p = i, l
            if i == k:
                return [tm_positional_two_term(True, math.sqrt(2.0) * me, s, p, c.create_count.couple_down,
                                               c.create_count.fill_couple_up, c.destroy.couple_down,
                                               c.destroy.fill_couple_up)]
            return [tm_positional_two_term(True, -math.sqrt(2.0) * me, s, p, c.destroy_count.couple_down,
                                           c.destroy_count.fill_couple_up, c.create.couple_down,
                                           c.create.fill_couple_up)]
        raise RuntimeError("Unexpected index arrangement for V_ijjj term")

    def three_term(self, me, i, k, l, j):
        if i == j or k == l:
            return self.three_termA(me, i, k, l, j)
        return self.three_termB(me, i, k, l, j)

    def four_term(self, me, i, k, l, j):
        c = self.c
        i_, j_, k_, l_ = align(i, j, k, l)
        ret = []
        if k_ > l_ and l_ > j_:
            ret.append(tm_four_term(2, -math.sqrt(3.0) * me, i, k, l, j, c.create, c.destroy))
            ret.append(tm_four_term(1, me, i, k, l, j, c.create, c.destroy))
        elif k_ > j_ and j_ > l_:
            le = -me if sgn4(i, k, l, j) else me
            ret.append(tm_four_term(2, math.sqrt(3.0) * le, i, k, l, j, c.create, c.destroy))
            ret.append(tm_four_term(1, le, i, k, l, j, c.create, c.destroy))
        elif j_ > k_ and k_ > l_:
            ret.append(tm_four_term(1, 2.0 * me, i, k, l, j, c.create, c.destroy))
        else:
            raise RuntimeError("unexpected index arrangment in V_ijkl term")
        return ret

    def three_termA(self, me, i, k, l, j):
        c = self.c
        same = None
        if i == j:
            same = i
        if k == l:
            same = k
            k = i
            l = j
        return [tm_three_term(math.sqrt(2.0) * me, same, k, l, c.count.no_couple, c.count.fill_no_couple,
                              c.create.couple_down, c.create.fill_couple_up,
                              c.destroy.couple_down, c.destroy.fill_couple_up)]

    def three_termB(self, me, i, k, l, j):
        c = self.c
        ret = []
        if i == k:
            same, p1, p2 = i, min(l, j), max(l, j)
            ret.append(tm_three_term(-math.sqrt(2.0) * me, same, p1, p2, c.e2d.no_couple, c.e2d.no_couple,
                                     c.destroy.couple_down, c.destroy.fill_couple_up,
                                     c.destroy.couple_down, c.destroy.fill_couple_up))
        if j == l:
            same, p1, p2 = j, min(i, k), max(i, k)
            ret.append(tm_three_term(-math.sqrt(2.0) * me, same, p1, p2, c.d2e.no_couple, c.d2e.no_couple,
                                     c.create.couple_down, c.create.fill_couple_up,
                                     c.create.couple_down, c.create.fill_couple_up))
        if j == k or i == l:
            if j == k:
                same, p1, p2 = j, l, i
            else:
                same, p1, p2 = i, j, k
            phase = -1.0 if sgn4(i, k, l, j) else 1.0
            if same < min(p1, p2):
                ret.append(tm_three_term(phase * math.sqrt(3.0) * me, same, p1, p2, c.flip.couple_up, c.flip.couple_up,
                                         c.create.couple_down, c.create.fill_couple_down,
                                         c.destroy.couple_down, c.destroy.fill_couple_down))
                ret.append(tm_three_term(-0.5 * math.sqrt(2.0) * me, same, p1, p2, c.count.no_couple, c.count.no_couple,
                                         c.create.couple_down, c.create.fill_couple_up,
                                         c.destroy.couple_down, c.destroy.fill_couple_up))
            elif same > max(p1, p2):
                ret.append(tm_three_term(phase * math.sqrt(3.0) * me, same, p1, p2, c.flip.couple_down,
                                         c.flip.couple_down, c.create.couple_up, c.create.fill_couple_up,
                                         c.destroy.couple_up, c.destroy.fill_couple_up))
                ret.append(tm_three_term(-0.5 * math.sqrt(2.0) * me, same, p1, p2, c.count.no_couple, c.count.no_couple,
                                         c.create.couple_down, c.create.fill_couple_up,
                                         c.destroy.couple_down, c.destroy.fill_couple_up))
            else:
                ret.append(tm_three_term(phase * math.sqrt(3.0) * me, same, p1, p2, c.flip.no_couple, c.flip.no_couple,
                                         c.create.couple_down, c.create.fill_couple_up,
                                         c.destroy.couple_down, c.destroy.fill_couple_up))
                ret.append(tm_three_term(-0.5 * math.sqrt(2.0) * me, same, p1, p2, c.count.fill_no_couple,
                                         c.count.fill_no_couple, c.create.couple_down, c.create.fill_couple_up,
                                         c.destroy.couple_down, c.destroy.fill_couple_up))
        return ret


class QCModel:
    """The SU2U1 quantum-chemistry model of ``models/chem/su2u1/model.hpp``."""

    def __init__(self, L: int, integrals: Dict[Tuple[int, int, int, int], float], nelec: int,
                 integral_cutoff: float = 1e-20, native: bool = True):
        """``native``: the terms come from the library's generator (``qcm_chem_terms``,
        kept as flat arrays that the native MPO maker reads directly; ``terms`` is
        built from them on first use); else from the Python restatement below.
        Both give the same terms, coefficients and provenance in the same order."""
        self.L = L
        self.nelec = nelec
        self.tag_handler = TagHandler()
        self.ops = construct_operators(self.tag_handler)
        self.col = construct_collection(self.ops)
        self.phys = phys_index()
        self.integrals = integrals
        self.integral_cutoff = integral_cutoff
        self._terms: Optional[List[Term]] = None
        self.term_arrays = None
        if native:
            from . import native as N
            self.term_arrays = N.chem_terms(L, nelec, integrals, integral_cutoff, self.ops, self.col)
        else:
            self._terms = []
            self._create_terms()

    @property
    def terms(self) -> List[Term]:
        if self._terms is None:
            self._terms = self._terms_from_arrays()
        return self._terms

    def _terms_from_arrays(self) -> List[Term]:
        a = self.term_arrays
        ptr, pos, tag = a.term_ptr.tolist(), a.pos.tolist(), a.tag.tolist()
        coeff, ferm = a.coeff.tolist(), a.fermionic.tolist()
        sptr, sidx, sval = a.src_ptr.tolist(), a.src_idx.tolist(), a.src_val.tolist()
        keys = a.keys
        out = []
        for t in range(len(coeff)):
            term = Term(coeff[t], bool(ferm[t]))
            term.ops = list(zip(pos[ptr[t]:ptr[t + 1]], tag[ptr[t]:ptr[t + 1]]))
            term.src = {keys[sidx[q]]: sval[q] for q in range(sptr[t], sptr[t + 1])}
            out.append(term)
        return out

    # parse_integrals (models/chem/parse_integrals.h:43-214), identity orbital order
    def _parsed(self):
        out = []
        for key, val in self.integrals.items():
            if abs(val) > self.integral_cutoff:
                i, j, k, l = [x - 1 for x in key]
                out.append((align(i, j, k, l), float(val), key))
        return out

    def _create_terms(self):
        N = self.nelec
        c = self.col
        ss = SpinSum(c)
        two_terms: Dict = {}
        three_terms: Dict = {}
        four_terms: Dict = {}

        def add(store, key, term):
            if key in store:
                store[key].coeff += term.coeff
                for u, f in term.src.items():
                    store[key].src[u] = store[key].src.get(u, 0.0) + f
            else:
                store[key] = term

        def add2(term):
            add(two_terms, (term.position(0), term.position(1), term.tag(0), term.tag(1)), term)

        def add3(term):
            add(three_terms, (term.position(0), term.position(1), term.position(2),
                              term.tag(0), term.tag(1), term.tag(2)), term)

        def add4(term):
            add(four_terms, tuple(term.position(x) for x in range(4)) + tuple(term.tag(x) for x in range(4)), term)

        for (i, j, k, l), me, ukey in self._parsed():
            terms = list(self._integral_terms(i, j, k, l, me, ss, N))
            # the terms of a unit integral give the coefficient per unit of this
            # integral (also for a value of zero, kept when the cutoff admits it)
            units = terms if me != 0.0 else list(self._integral_terms(i, j, k, l, 1.0, ss, N))
            for (kind, t), (_, tu) in zip(terms, units):
                # the coefficient per unit of this integral, before terms are merged
                t.src = {ukey: t.coeff / me if me != 0.0 else tu.coeff}
                if kind == 1:
                    self.terms.append(t)
                elif kind == 2:
                    add2(t)
                elif kind == 3:
                    add3(t)
                else:
                    add4(t)
        for key in sorted(two_terms):
            self.terms.append(two_terms[key])
        for key in sorted(three_terms):
            self.terms.append(three_terms[key])
        for key in sorted(four_terms):
            self.terms.append(four_terms[key])

    def _integral_terms(self, i, j, k, l, me, ss, N):
        """The terms of one integral as (kind, term): kind 1 = kept as is, 2/3/4 =
        merged with equal two-/three-/four-operator terms (``model.hpp:96-139``)."""
        out = []
        if i == -1 and j == -1 and k == -1 and l == -1:
            t = Term(me)
            t.push(0, self.ops.ident)
            out.append((1, t))
        elif i == j and k == -1 and l == -1:
            t = Term(me)
            t.push(i, self.ops.count)
            out.append((1, t))
        elif k == -1 and l == -1:
            if N == 1:
                raise NotImplementedError("one-electron systems are not supported")
            f = me * (1.0 / (N - 1))
            terms = []
            for kk in range(self.L):
                if kk == j or kk == i:
                    continue
                terms += ss.three_term(f, i, kk, kk, j)
                terms += ss.three_term(f, j, kk, kk, i)
            out += [(3, t) for t in terms]
            terms = []
            terms += ss.V_term(f, i, i, i, j)
            terms += ss.V_term(f, j, i, i, i)
            terms += ss.V_term(f, i, j, j, j)
            terms += ss.V_term(f, j, j, j, i)
            out += [(2, t) for t in terms]
        elif i == j == k == l:
            t = Term(me)
            t.push(i, self.ops.docc)
            out.append((1, t))
        elif (i == j and j == k and k != l) or (i != j and j == k and k == l):
            if i == j:
                s, p = i, l
            elif k == l:
                s, p = l, i
            else:
                raise RuntimeError("V_ijjj")
            out += [(2, t) for t in ss.two_term(me, s, s, s, p) + ss.two_term(me, s, p, s, s)]
        elif i == j and k == l and j != k:
            out += [(2, t) for t in ss.two_term(me, i, k, k, i)]
        elif i == k and j == l and i != j:
            terms = ss.two_term(0.5 * me, i, i, j, j) + ss.two_term(0.5 * me, j, j, i, i) + \
                ss.two_term(me, i, j, i, j)
            out += [(2, t) for t in terms]
        elif (i == j and j != k and k != l) or (k == l and i != j and j != k):
            if i == j:
                terms = ss.three_term(me, i, k, l, i) + ss.three_term(me, i, l, k, i)
            else:
                terms = ss.three_term(me, i, k, k, j) + ss.three_term(me, j, k, k, i)
            out += [(3, t) for t in terms]
        elif ((i == k and j != l) or j == k or (j == l and i != k)) and (i != j and k != l):
            terms = (ss.three_term(me, i, k, l, j) + ss.three_term(me, i, l, k, j)
                     + ss.three_term(me, j, k, l, i) + ss.three_term(me, j, l, k, i))
            out += [(3, t) for t in terms]
        elif i != j and j != k and k != l and i != k and j != l:
            terms = (ss.four_term(me, i, k, l, j) + ss.four_term(me, i, l, k, j)
                     + ss.four_term(me, j, k, l, i) + ss.four_term(me, j, l, k, i))
            out += [(4, t) for t in terms]
        return out


__all__ = ["QCModel", "TagHandler", "phys_index", "align", "Term"]
