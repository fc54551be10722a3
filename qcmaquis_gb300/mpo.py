"""MPO tensors and the tagged MPO builder for the chemistry Hamiltonian.

* ``MPOTensor`` restates ``mp_tensors/mpotensor.h:23-107`` /
  ``mpotensor.hpp:10-75``: a column-major sparse matrix of (tag, scale) lists,
  row/column non-zero counts, left/right bond spins and the Hermitian pairing
  ``Hermitian`` of ``mp_tensors/mpotensor_detail.h:124-170``.
* ``TaggedMPOMaker`` restates
  ``models/generate_mpo/tagged_mpo_maker_optim.hpp:97-735``: prempo keys,
  fork/merge insertion, filling strings, bond numbering in key order,
  bond spins and Hermitian-conjugate bond pairs with their phases.
* ``make_twosite_mpo`` restates ``mp_tensors/ts_ops.h:36-125`` (two-site MPO as
  spin-coupled Kronecker products of neighbouring tensors).
"""
from __future__ import annotations

import itertools
from typing import Dict, List, Optional, Tuple

import numpy as np

from .model import QCModel, TagHandler, Term
from .site_operator import SiteOperator, SpinDescriptor, allowed_spins, op_kron_su2
from .symmetry import Index, particle_number

TRIVIAL_LEFT, BULK, BULK_NO_MERGE, TRIVIAL_RIGHT = 0, 1, 2, 3
KEY_TL = (TRIVIAL_LEFT, (), 0)
KEY_TR = (TRIVIAL_RIGHT, (), 0)


def bulk_key(pos_op):
    return (BULK, tuple(pos_op), 0)


class Hermitian:
    def __init__(self, left_herm, right_herm, left_phase, right_phase):
        self.LeftHerm = list(left_herm)
        self.RightHerm = list(right_herm)
        self.LeftPhase = list(left_phase)
        self.RightPhase = list(right_phase)

    @classmethod
    def identity(cls, ld, rd):
        return cls(range(ld), range(rd), [1] * ld, [1] * rd)

    def left_skip(self, b):
        return self.LeftHerm[b] < b

    def right_skip(self, b):
        return self.RightHerm[b] < b

    def left_conj(self, b):
        return self.LeftHerm[b]

    def right_conj(self, b):
        return self.RightHerm[b]

    def left_phase(self, b):
        return self.LeftPhase[b]

    def right_phase(self, b):
        return self.RightPhase[b]

    def __mul__(self, other: "Hermitian") -> "Hermitian":
        return Hermitian(self.LeftHerm, other.RightHerm, self.LeftPhase, other.RightPhase)


class MPOTensor:
    """Sparse (b1, b2) -> [(op, scale), ...] tensor with SU(2) bond spins (all 0 for
    an abelian group; ``symmetry`` names the group: "su2u1", "2u1" or "u1")."""

    symmetry = "su2u1"

    def __init__(self, ld: int, rd: int, prempo: List[Tuple[int, int, int, float]], op_table: List[SiteOperator],
                 herm: Optional[Hermitian], left_spins: List[SpinDescriptor], right_spins: List[SpinDescriptor]):
        self.row_dim = ld
        self.col_dim = rd
        self.op_table = op_table
        self.left_spins = list(left_spins)
        self.right_spins = list(right_spins)
        # element lists: later entries (in column-major order) are prepended
        # entries (b1, b2, tag, scale[, label]); a label names the model term whose
        # coefficient the scale is (kept parallel to the element lists in ``labels``)
        entries = sorted(prempo, key=lambda t: (t[1], t[0]))
        self.elements: Dict[Tuple[int, int], List[Tuple[int, float]]] = {}
        self.labels: Dict[Tuple[int, int], List] = {}
        self.row_index: List[set] = [set() for _ in range(ld)]
        for ent in entries:
            b1, b2, tag, scale = ent[:4]
            label = ent[4] if len(ent) > 4 else None
            key = (b1, b2)
            if key not in self.elements:
                self.elements[key] = [(tag, scale)]
                self.labels[key] = [label]
                self.row_index[b1].add(b2)
            else:
                self.elements[key].insert(0, (tag, scale))
                self.labels[key].insert(0, label)
        self.cols: List[List[int]] = [[] for _ in range(rd)]
        for (b1, b2) in sorted(self.elements, key=lambda k: (k[1], k[0])):
            self.cols[b2].append(b1)
        self.row_nnz = [0] * ld
        self.col_nnz = [0] * rd
        for (b1, b2) in self.elements:
            self.row_nnz[b1] += 1
            self.col_nnz[b2] += 1
        self.num_one_rows = sum(1 for x in self.row_nnz if x == 1)
        self.num_one_cols = sum(1 for x in self.col_nnz if x == 1)
        if herm is not None and len(herm.LeftHerm) == ld and len(herm.RightHerm) == rd:
            self.herm = herm
        else:
            self.herm = Hermitian.identity(ld, rd)
        self._sparse_cache: Dict[int, list] = {}

    @classmethod
    def from_elements(cls, ld: int, rd: int, op_table: List[SiteOperator], herm: Optional[Hermitian],
                      left_spins: List[SpinDescriptor], right_spins: List[SpinDescriptor], elem_b1, elem_b2, elem_ptr,
                      term_tag, term_scale, term_label) -> "MPOTensor":
        """The tensor from column-major elements whose term lists are already in
        this class's order (as the native maker writes them); the same object
        the constructor builds from the equivalent entry list."""
        t = cls.__new__(cls)
        t.row_dim, t.col_dim = ld, rd
        t.op_table = op_table
        t.left_spins = list(left_spins)
        t.right_spins = list(right_spins)
        terms = list(zip(term_tag, term_scale))
        labs = [None if x < 0 else x for x in term_label]
        keys = list(zip(elem_b1, elem_b2))
        ptr = elem_ptr
        t.elements = {k: terms[ptr[e]:ptr[e + 1]] for e, k in enumerate(keys)}
        t.labels = {k: labs[ptr[e]:ptr[e + 1]] for e, k in enumerate(keys)}
        b1 = np.asarray(elem_b1, dtype=np.int64)
        b2 = np.asarray(elem_b2, dtype=np.int64)
        cb = np.searchsorted(b2, np.arange(rd + 1)).tolist()          # elements are column-major
        t.cols = [elem_b1[cb[c]:cb[c + 1]] for c in range(rd)]
        order = np.lexsort((b2, b1))
        rb = np.searchsorted(b1[order], np.arange(ld + 1)).tolist()
        by_row = b2[order].tolist()
        t.row_index = [set(by_row[rb[r]:rb[r + 1]]) for r in range(ld)]
        t.row_nnz = np.bincount(b1, minlength=ld).tolist()
        t.col_nnz = np.bincount(b2, minlength=rd).tolist()
        t.num_one_rows = sum(1 for x in t.row_nnz if x == 1)
        t.num_one_cols = sum(1 for x in t.col_nnz if x == 1)
        if herm is not None and len(herm.LeftHerm) == ld and len(herm.RightHerm) == rd:
            t.herm = herm
        else:
            t.herm = Hermitian.identity(ld, rd)
        t._sparse_cache = {}
        return t

    def has(self, b1, b2) -> bool:
        return (b1, b2) in self.elements

    def at(self, b1, b2) -> List[Tuple[int, float]]:
        return self.elements[(b1, b2)]

    def labels_at(self, b1, b2) -> List:
        return self.labels.get((b1, b2), [None] * len(self.elements[(b1, b2)]))

    def column(self, b2) -> List[int]:
        return self.cols[b2]

    def row(self, b1) -> List[int]:
        return sorted(self.row_index[b1])

    def left_spin(self, b) -> SpinDescriptor:
        return self.left_spins[b]

    def right_spin(self, b) -> SpinDescriptor:
        return self.right_spins[b]

    def op(self, tag) -> SiteOperator:
        return self.op_table[tag]

    def sparse(self, tag):
        s = self._sparse_cache.get(tag)
        if s is None:
            s = self.op_table[tag].sparse()
            self._sparse_cache[tag] = s
        return s


class MPO(list):
    core_energy: float = 0.0
    core_labels: list = []   # model terms folded into core_energy


class TaggedMPOMaker:
    """``merge_site_terms=False`` keeps every one-site term as its own (tag, scale)
    entry instead of one summed operator per site (the same operator; used where
    each term's coefficient must stay a separate MPO scale, as for gradients).
    Every coefficient-carrying scale is labelled with its model term's index."""

    def __init__(self, model: QCModel, merge_site_terms: bool = True, native: bool = True):
        self.L = model.L
        self.symmetry = getattr(model, "symmetry", "su2u1")
        self.th: TagHandler = model.tag_handler
        self.identity = model.ops.ident
        self.identity_full = model.ops.ident_full
        self.filling = model.ops.fill
        self.prempo: List[Dict] = [dict() for _ in range(self.L)]
        self.site_terms: Dict[int, SiteOperator] = {}
        self.leftmost_right = self.L
        self.rightmost_left = 0
        self.core_energy = 0.0
        self.finalized = False
        self.merge_site_terms = merge_site_terms
        self.site_term_lists: Dict[int, list] = {}
        self.core_labels: List[int] = []
        self._label = None
        self.native = native
        if native:
            self._collect_native(model)
        else:
            for idx, t in enumerate(model.terms):
                self._label = idx
                self.add_term(t)
        self._label = None

    def _collect_native(self, model: QCModel):
        """The native maker's input: one-site terms are added here (they need the
        operator algebra), the terms of two or more operators are flattened for
        ``qcm_mpo_maker_add_terms``."""
        arrays = getattr(model, "term_arrays", None)
        if arrays is not None and getattr(model, "_terms", None) is None:
            return self._collect_arrays(arrays)
        ptr, flat, coeff, label = [0], [], [], []
        lr, rl = self.L, 0
        for idx, t in enumerate(model.terms):
            ops = t.ops
            if len(ops) == 1:
                self._label = idx
                self._add_1term(t)
                p = ops[0][0]
                lr, rl = min(lr, p), max(rl, p)
                continue
            flat.extend(ops)
            ptr.append(len(flat))
            coeff.append(t.coeff)
            label.append(idx)
        pt = np.fromiter(itertools.chain.from_iterable(flat), dtype=np.int32, count=2 * len(flat)).reshape(-1, 2)
        pos, tag = np.ascontiguousarray(pt[:, 0]), np.ascontiguousarray(pt[:, 1])
        if len(coeff):
            starts = np.asarray(ptr[:-1], dtype=np.int64)
            lr = min(lr, int(np.maximum.reduceat(pos, starts).min()))
            rl = max(rl, int(np.minimum.reduceat(pos, starts).max()))
        self._native_terms = (np.asarray(ptr, dtype=np.int32), pos, tag, np.asarray(coeff, dtype=np.float64),
                              np.asarray(label, dtype=np.int32))
        self.leftmost_right, self.rightmost_left = lr, rl
        self._native_terms = (ptr, pos, tag, coeff, label)

    # -- prempo helpers ------------------------------------------------------
    def _insert(self, p, kk, val, attach):
        d = self.prempo[p]
        if attach:
            if kk not in d:
                d[kk] = [val]
        else:
            d.setdefault(kk, []).append(val)
        return kk[1]

    def _insert_filling(self, i, j, k, trivial_fill, spin_gt_one):
        for s in range(i, j):
            use_ident = self.identity_full if spin_gt_one else self.identity
            op = use_ident if trivial_fill else self.filling
            d = self.prempo[s]
            kk = (k, k)
            if kk not in d:
                d[kk] = [(op, 1.0, None)]
            elif d[kk][0][:2] != (op, 1.0):
                raise RuntimeError(f"Pre-existing term at site {s}")

    def add_term(self, term: Term):
        term.ops.sort(key=lambda x: x[0])
        n = len(term)
        if n == 1:
            self._add_1term(term)
        elif n == 2:
            self._add_2term(term)
        else:
            self._add_generic_term(term)
        self.leftmost_right = min(self.leftmost_right, term.ops[-1][0])
        self.rightmost_left = max(self.rightmost_left, term.ops[0][0])

    def _add_1term(self, term):
        if term.tag(0) == self.identity:
            self.core_energy += term.coeff
            self.core_labels.append(self._label)
        elif not self.merge_site_terms:
            self.site_term_lists.setdefault(term.position(0), []).append((term.tag(0), term.coeff, self._label))
        else:
            op = self.th.get_op(term.tag(0)).scaled(term.coeff)
            p = term.position(0)
            if p in self.site_terms:
                self.site_terms[p].iadd(op)
            else:
                cur = SiteOperator()
                cur.iadd(op)
                self.site_terms[p] = cur

    def _add_2term(self, term):
        th = self.th
        nferm = sum(1 for i in range(2) if th.is_fermionic(term.tag(i)))
        mpo_spin = SpinDescriptor()
        k1 = KEY_TL
        mpo_spin = mpo_spin.couple(th.get_op(term.tag(0)).spin)
        k2 = bulk_key([term.ops[1]])
        k1 = self._insert(term.position(0), (k1, k2), (term.tag(0), term.coeff, self._label), attach=False)
        if th.is_fermionic(term.tag(0)):
            nferm -= 1
        trivial = (nferm % 2 == 0)
        self._insert_filling(term.position(0) + 1, term.position(1), k1, trivial, mpo_spin.get() > 1)
        mpo_spin = mpo_spin.couple(th.get_op(term.tag(1)).spin)
        self._insert(term.position(1), (k1, KEY_TR), (term.tag(1), 1.0, None), attach=True)
        assert mpo_spin.get() == 0

    def _add_generic_term(self, term):
        th = self.th
        nops = len(term)
        nferm = sum(1 for i in range(nops) if th.is_fermionic(term.tag(i)))
        mpo_spin = SpinDescriptor()
        thresh = nops // 2  # prefer_fork
        ops_left = []
        k1 = KEY_TL
        for i in range(thresh):
            mpo_spin = mpo_spin.couple(th.get_op(term.tag(i)).spin)
            ops_left.append(term.ops[i])
            k2 = bulk_key(ops_left)
            k1 = self._insert(term.position(i), (k1, k2), (term.tag(i), 1.0, None), attach=True)
            if th.is_fermionic(term.tag(i)):
                nferm -= 1
            self._insert_filling(term.position(i) + 1, term.position(i + 1), k1, nferm % 2 == 0, mpo_spin.get() > 1)
        ops_right = [term.ops[j] for j in range(thresh + 1, nops)]
        k2 = bulk_key(ops_right)
        mpo_spin = mpo_spin.couple(th.get_op(term.tag(thresh)).spin)
        k1 = self._insert(term.position(thresh), (k1, k2), (term.tag(thresh), term.coeff, self._label), attach=False)
        if th.is_fermionic(term.tag(thresh)):
            nferm -= 1
        self._insert_filling(term.position(thresh) + 1, term.position(thresh + 1), k1, nferm % 2 == 0,
                             mpo_spin.get() > 1)
        for i in range(thresh + 1, nops):
            if i == nops - 1:
                k2 = KEY_TR
            else:
                k2 = bulk_key([term.ops[j] for j in range(i + 1, nops)])
            mpo_spin = mpo_spin.couple(th.get_op(term.tag(i)).spin)
            k1 = self._insert(term.position(i), (k1, k2), (term.tag(i), 1.0, None), attach=True)
            if th.is_fermionic(term.tag(i)):
                nferm -= 1
            if i != nops - 1:
                self._insert_filling(term.position(i) + 1, term.position(i + 1), k1, nferm % 2 == 0,
                                     mpo_spin.get() > 1)
        assert mpo_spin.get() == 0

    def _finalize(self):
        kk = (KEY_TL, KEY_TR)
        for p in sorted(self.site_terms):
            tag = self.th.register_op(self.site_terms[p], 0)
            d = self.prempo[p]
            if kk in d:
                raise RuntimeError("another site term already existing!")
            d[kk] = [(tag, 1.0, None)]
        for p in sorted(self.site_term_lists):
            d = self.prempo[p]
            if kk in d:
                raise RuntimeError("another site term already existing!")
            d[kk] = list(self.site_term_lists[p])
        for p in range(self.rightmost_left):
            d = self.prempo[p]
            d.setdefault((KEY_TL, KEY_TL), []).append((self.identity, 1.0, None))
        for p in range(self.leftmost_right + 1, self.L):
            d = self.prempo[p]
            d.setdefault((KEY_TR, KEY_TR), []).append((self.identity, 1.0, None))
        self.finalized = True

    def _conjugate_key(self, k, p):
        th = self.th
        kind, pos_op, off = k
        conj = (kind, tuple((pp, th.herm_conj(t)) for pp, t in pos_op), off)
        phase = (1, 1)
        if self.symmetry != "su2u1":
            # abelian groups: a partner bond's boundary is the plain transpose
            return conj, phase
        if len(pos_op) == 1:
            op1 = th.get_op(pos_op[0][1])
            if p < pos_op[0][0]:
                pdiff = particle_number(op1.bm.keys[0][0]) - particle_number(op1.bm.keys[0][1])
                if pdiff == 1:
                    phase = (1, -1)
                elif pdiff == -1:
                    phase = (-1, 1)
            else:
                if op1.spin.get() == 1:
                    phase = (-1, 1)
        if len(pos_op) == 2:
            op1 = th.get_op(pos_op[0][1])
            op2 = th.get_op(pos_op[1][1])
            d1 = particle_number(op1.bm.keys[0][0]) - particle_number(op1.bm.keys[0][1])
            d2 = particle_number(op2.bm.keys[0][0]) - particle_number(op2.bm.keys[0][1])
            if op1.spin.get() == 1 and op2.spin.get() == 1 and op2.spin.action() == -1 and d1 == -d2:
                phase = (-1, -1)
            if op1.spin.get() == 1 and op2.spin.get() == 1 and op2.spin.action() == 1 and d1 == d2:
                phase = (-1, -1)
        return conj, phase

    def _collect_arrays(self, a):
        """``_collect_native`` from the model's flat term arrays (the native term
        generator's output), without Python term objects."""
        nops = np.diff(a.term_ptr.astype(np.int64))
        one = np.nonzero(nops == 1)[0]
        lr, rl = self.L, 0
        for idx in one.tolist():
            q = int(a.term_ptr[idx])
            t = Term(float(a.coeff[idx]), bool(a.fermionic[idx]))
            t.push(int(a.pos[q]), int(a.tag[q]))
            self._label = idx
            self._add_1term(t)
            lr, rl = min(lr, t.position(0)), max(rl, t.position(0))
        if np.any(nops < 1):
            raise RuntimeError("a model term without operators")
        multi = np.nonzero(nops >= 2)[0]
        op_mask = np.repeat(nops >= 2, nops)
        pos = np.ascontiguousarray(a.pos[op_mask], dtype=np.int32)
        tag = np.ascontiguousarray(a.tag[op_mask], dtype=np.int32)
        ptr = np.zeros(len(multi) + 1, dtype=np.int32)
        np.cumsum(nops[multi], out=ptr[1:])
        if len(multi):
            starts = ptr[:-1].astype(np.int64)
            lr = min(lr, int(np.maximum.reduceat(pos, starts).min()))
            rl = max(rl, int(np.minimum.reduceat(pos, starts).max()))
        self.leftmost_right, self.rightmost_left = lr, rl
        self._native_terms = (ptr, pos, tag, np.ascontiguousarray(a.coeff[multi], dtype=np.float64),
                              multi.astype(np.int32))

    def _create_native(self) -> MPO:
        """create_mpo through the native maker (``qcm_mpo_maker_*``): the same
        tensors as the Python restatement below, element for element."""
        from . import native as N
        site_terms = {}
        for p in sorted(self.site_terms):
            site_terms[p] = [(self.th.register_op(self.site_terms[p], 0), 1.0, None)]
        for p in sorted(self.site_term_lists):
            site_terms[p] = list(self.site_term_lists[p])
        self.finalized = True
        tags = N.FTagTable(self.th, self.identity, self.identity_full, self.filling, self.symmetry)
        sites = N.mpo_maker_sites(self.L, tags, self._native_terms, site_terms, self.leftmost_right,
                                  self.rightmost_left)
        mpo = MPO()
        table = self.th.ops
        left_spins = [SpinDescriptor()]
        LeftHerm, LeftPhase = [0], [1]
        for (ld, rd, eb1, eb2, eptr, ttag, tscale, tlabel, rspin, rherm, rphase) in sites:
            right_spins = [SpinDescriptor.raw(a, b) for a, b in rspin]
            h = Hermitian(LeftHerm, rherm, LeftPhase, rphase)
            t = MPOTensor.from_elements(ld, rd, table, h, left_spins, right_spins, eb1, eb2, eptr, ttag, tscale,
                                        tlabel)
            t.symmetry = self.symmetry
            mpo.append(t)
            left_spins, LeftHerm, LeftPhase = right_spins, rherm, rphase
        mpo.core_energy = self.core_energy
        mpo.core_labels = list(self.core_labels)
        return mpo

    def create_mpo(self) -> MPO:
        if self.native:
            return self._create_native()
        if not self.finalized:
            self._finalize()
        mpo = MPO()
        left = {KEY_TL: 0}
        left_spins = [SpinDescriptor()]
        LeftHerm = [0]
        LeftPhase = [1]
        L = self.L
        table = self.th.ops
        for p in range(L):
            pre = []
            herm_pairs = {}
            herm_phases = {}
            right = {}
            r = 2
            for kk in sorted(self.prempo[p], key=lambda x: (x[1], x[0])):
                k1, k2 = kk
                for val in self.prempo[p][kk]:
                    if k1 not in left:
                        raise RuntimeError("k1 not found!")
                    ll = left[k1]
                    if k2 not in right:
                        if k2 == KEY_TL:
                            right[k2] = 0
                        elif k2 == KEY_TR:
                            right[k2] = 1
                        else:
                            right[k2] = r
                            r += 1
                    rr_dim = 0 if p == L - 1 else right[k2]
                    pre.append((ll, rr_dim, val[0], val[1], val[2]))
                    ck2, phase = self._conjugate_key(k2, p)
                    if k2 != ck2:
                        herm_pairs[k2] = ck2
                        herm_phases[k2] = phase
            ldim = max(x[0] for x in pre) + 1
            rdim = max(x[1] for x in pre) + 1
            right_spins = [SpinDescriptor() for _ in range(rdim)]
            for (b1, b2, tag, _, _) in pre:
                out_spin = left_spins[b1].couple(table[tag].spin)
                assert right_spins[b2].get() == 0 or right_spins[b2].get() == out_spin.get()
                right_spins[b2] = out_spin
            RightHerm = list(range(rdim))
            RightPhase = [1] * rdim
            for hk in sorted(herm_pairs):
                romeo = right.get(hk, 0)
                julia = right.get(herm_pairs[hk], 0)
                if romeo < julia:
                    RightHerm[romeo], RightHerm[julia] = RightHerm[julia], RightHerm[romeo]
                    RightPhase[romeo] = herm_phases[hk][0]
                    RightPhase[julia] = herm_phases[hk][1]
            h = Hermitian(LeftHerm, RightHerm, LeftPhase, RightPhase)
            if p == 0:
                t = MPOTensor(1, rdim, pre, table, h, left_spins, right_spins)
            elif p == L - 1:
                t = MPOTensor(ldim, 1, pre, table, h, left_spins, right_spins)
            else:
                t = MPOTensor(ldim, rdim, pre, table, h, left_spins, right_spins)
            t.symmetry = self.symmetry
            mpo.append(t)
            left = right
            left_spins = right_spins
            LeftHerm = RightHerm
            LeftPhase = RightPhase
        mpo.core_energy = self.core_energy
        mpo.core_labels = list(self.core_labels)
        return mpo


def make_mpo(model: QCModel) -> MPO:
    return TaggedMPOMaker(model).create_mpo()


def _merge_spins(dst: List[int], src: List[int]):
    """``extend_spin_basis``: grow ``dst`` to ``src``'s length, non-zero entries of src win."""
    if len(dst) < len(src):
        dst.extend([0] * (len(src) - len(dst)))
    for i, v in enumerate(src):
        if v != 0:
            dst[i] = v


def make_twosite_mpo(mpo1: MPOTensor, mpo2: MPOTensor, phys1: Index, phys2: Index) -> MPOTensor:
    """Two-site MPO tensor W(b1,b3) = sum_b2 W1(b1,b2) (x) W2(b2,b3) per operator spin
    (``make_twosite_mpo``, ``mp_tensors/ts_ops.h:78-152``).  The spin-coupled
    Kronecker product depends only on the two operators and the three bond spins,
    so each distinct (op1, op2, spins, product spin) is formed once and reused
    scaled.  Only the non-zero (b1, b2, b3) chains are visited (b2 in row b1 of W1,
    b3 in row b2 of W2), and every (b1, b3, spin) sum runs over its summands in the
    reference's order, block by block, with the reference's additions."""
    assert mpo1.col_dim == mpo2.row_dim
    table: List[SiteOperator] = []
    prempo = []
    kron: Dict[tuple, SiteOperator] = {}
    rows2 = [mpo2.row(b2) for b2 in range(mpo2.row_dim)]
    for b1 in range(mpo1.row_dim):
        chains: Dict[int, List[int]] = {}
        for b2 in mpo1.row(b1):
            for b3 in rows2[b2]:
                chains.setdefault(b3, []).append(b2)
        j = mpo1.left_spin(b1).get()
        for b3 in sorted(chains):
            jp = mpo2.right_spin(b3).get()
            # per product spin: block sums keyed (lc, rc), the spin basis, the first summand's spin
            acc: Dict[int, list] = {}
            for b2 in chains[b3]:
                jpp = mpo1.right_spin(b2).get()
                for tag1, s1 in mpo1.at(b1, b2):
                    op1 = mpo1.op(tag1)
                    for tag2, s2 in mpo2.at(b2, b3):
                        op2 = mpo2.op(tag2)
                        for sp in allowed_spins(j, jp, op1.spin.get(), op2.spin.get()):
                            key = (tag1, tag2, j, jpp, jp, sp)
                            prod = kron.get(key)
                            if prod is None:
                                prod = op_kron_su2(phys1, phys2, op1, op2, mpo1.left_spin(b1),
                                                   mpo1.right_spin(b2), mpo2.right_spin(b3),
                                                   SpinDescriptor(sp, j, jp))
                                prod.remove_empty_blocks()
                                kron[key] = prod
                            c = s1 * s2
                            a = acc.get(sp)
                            if a is None:
                                a = acc[sp] = [{}, {}, None, set()]
                            blocks, basis = a[0], a[1]
                            if not blocks:   # SiteOperator += takes the spin while empty
                                a[2] = (prod.spin.twoS, prod.spin.diff)
                            for bk, blk in zip(prod.bm.keys, prod.bm.blocks):
                                cur = blocks.get(bk)
                                blocks[bk] = blk * c if cur is None else cur + blk * c
                            # a basis spin is a function of its position (the spin of that
                            # product state), so merging one product's spin basis again
                            # changes nothing: once per distinct product
                            if key not in a[3]:
                                a[3].add(key)
                                for bk, (rr, cc) in prod.spin_basis.items():
                                    d = basis.get(bk)
                                    if d is None:
                                        basis[bk] = (list(rr), list(cc))
                                    else:
                                        _merge_spins(d[0], rr)
                                        _merge_spins(d[1], cc)
            for sp in sorted(acc):
                blocks, basis, spin_raw, _ = acc[sp]
                op = SiteOperator(spin_basis=basis)
                if spin_raw is not None:
                    op.spin = SpinDescriptor.raw(*spin_raw)
                for (lc, rc), blk in blocks.items():
                    op.bm.insert_block(blk, lc, rc)
                table.append(op)
                prempo.append((b1, b3, len(table) - 1, 1.0))
    return MPOTensor(mpo1.row_dim, mpo2.col_dim, prempo, table, mpo1.herm * mpo2.herm,
                     mpo1.left_spins, mpo2.right_spins)


def _twosite_job(args):
    a, b, phys = args
    return make_twosite_mpo(a, b, phys, phys)


def make_ts_cache_mpo(mpo: MPO, phys: Index, workers: int = 1) -> List[MPOTensor]:
    """Two-site MPO tensors of every site pair (``make_ts_cache_mpo``,
    ``mp_tensors/ts_ops.h``).  ``workers`` > 1 builds them in that many spawned
    processes (host work only; spawn, so it is safe after CUDA is initialised)."""
    jobs = [(mpo[p], mpo[p + 1], phys) for p in range(len(mpo) - 1)]
    if workers <= 1 or len(jobs) < 2:
        return [_twosite_job(j) for j in jobs]
    import multiprocessing as mp
    from concurrent.futures import ProcessPoolExecutor
    with ProcessPoolExecutor(max_workers=min(workers, len(jobs)), mp_context=mp.get_context("spawn")) as ex:
        return list(ex.map(_twosite_job, jobs))


__all__ = ["MPOTensor", "MPO", "Hermitian", "TaggedMPOMaker", "make_mpo", "make_twosite_mpo",
           "make_ts_cache_mpo"]
