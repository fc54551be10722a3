"""The oracle's own two-site MPO tensors (test infrastructure).

Restates, independently of the product package:

* ``make_twosite_mpo`` / ``mpo_couple`` / ``allowed_spins``
  (``mt/ts_ops.h:19-152``): W(b1, b3) = sum over the b2 that row b1 of W1 and
  column b3 of W2 share, of the spin-coupled Kronecker products of every
  (op1, op2) pair, one output operator per product spin s allowed by the bond
  spins, accumulated per s in ascending b2 order (``std::set``);
* the abelian ``op_kron`` (``bm/site_operator_algorithms.h:167-205``) for TwoU1
  tensors, and the SU(2) ``op_kron`` (``:215-318``) with the
  identity expansion, the per-block 9j coupling ``mod_coupling(j1, j2, J, k1,
  k2, k, j1', j2', J')``, the product-state spins of ``productSpin``
  (``bm/symmetry/spin_descriptor.h:106-117``) and the overall 6j factor;
* ``SiteOperator::operator+=`` with ``extend_spin_basis``
  (``bm/site_operator.hpp:58-102``), ``tag_detail::remove_empty_blocks``
  (``models/tag_detail.h:22-46``);
* the sparse form of an SU(2) site operator (``SparseOperator::update`` with
  ``check_spin_basis``, ``bm/sparse_operator.h:127-160``,
  ``bm/site_operator.hpp:318-341``): per block, the non-zero entries
  (row, col, row spin, col spin, value) in row-major order.

The single-site MPO tensors are inputs here (built by the model builder
outside the path); the oracle reads their bond spins, Hermitian partner data
and operator blocks.
"""
from __future__ import annotations

from typing import Dict, List, Tuple

import numpy as np

from .qn import BlockMatrix, ProductBasis, fuse, spin
from .su2 import mod_coupling, sixj


class OSpin:
    """``SpinDescriptor<SU2Tag>``: the operator rank 2S and its action out - in."""

    __slots__ = ("twoS", "diff")

    def __init__(self, twoS: int = 0, inp: int = 0, out: int = 0):
        self.twoS = twoS
        self.diff = out - inp

    def get(self) -> int:
        return self.twoS


class OOp:
    """An SU(2) site operator: its block matrix, its spin descriptor and its spin basis
    {(lc, rc): (row spins, column spins)}."""

    __slots__ = ("bm", "spin", "spin_basis")

    def __init__(self, bm=None, sp=None, spin_basis=None):
        self.bm = bm if bm is not None else BlockMatrix()
        self.spin = sp if sp is not None else OSpin()
        self.spin_basis = spin_basis if spin_basis is not None else {}


_SPARSE_CACHE: Dict[int, tuple] = {}


def sparse_of(op) -> List[List[tuple]]:
    """Per block of ``op.bm``, the entries (row, col, row spin, col spin, value) != 0.
    An empty spin basis takes |spin| of the block's charges for every row and column."""
    hit = _SPARSE_CACHE.get(id(op))
    if hit is not None and hit[0] is op:
        return hit[1]
    sb = getattr(op, "spin_basis", None) or {}
    out = []
    for (lc, rc), b in zip(op.bm.keys, op.bm.blocks):
        if sb:
            rs, cs = sb[(lc, rc)]
        else:
            rs, cs = [abs(spin(lc))] * b.shape[0], [abs(spin(rc))] * b.shape[1]
        ents = []
        for i in range(b.shape[0]):
            for j in range(b.shape[1]):
                v = float(b[i, j])
                if v != 0.0:
                    ents.append((i, j, rs[i], cs[j], v))
        out.append(ents)
    _SPARSE_CACHE[id(op)] = (op, out)
    return out


def allowed_spins(left: int, right: int, k1: int, k2: int) -> List[int]:
    """Product ranks s in |k1-k2| .. k1+k2 with |s - left| <= right <= s + left."""
    return [s for s in range(abs(k1 - k2), abs(k1 + k2) + 1, 2) if abs(s - left) <= right <= abs(s + left)]


def product_spin(a, b) -> int:
    sa, sb = spin(a), spin(b)
    return 2 if (sa == -1 and sb == 1) else abs(sa + sb)


def _op_blocks(op) -> BlockMatrix:
    bm = BlockMatrix()
    for (lc, rc), b in zip(op.bm.keys, op.bm.blocks):
        bm.insert_block(np.array(b, dtype=np.float64), lc, rc)
    return bm


def op_kron_su2(phys_a, phys_b, op_a, op_b, j: int, jpp: int, jp: int, k: int) -> OOp:
    """Spin-coupled Kronecker product of two site operators, product rank k, bond spins
    j (left of site a), jpp (between), jp (right of site b)."""
    A, B = _op_blocks(op_a), _op_blocks(op_b)
    k1, k2 = op_a.spin.get(), op_b.spin.get()
    # the identity of a site is stored on its (N,2S) diagonal only; a rank > 0 partner
    # needs its spin-flipping pair (1,1) <-> (1,-1) as well
    if k1 > 0 and k2 == 0:
        cb, cc = tuple(phys_b[1][0]), tuple(phys_b[2][0])
        if not B.has_block(cb, cc):
            B.insert_block(np.ones((1, 1)), cb, cc)
            B.insert_block(np.ones((1, 1)), cc, cb)
    if k1 == 0 and k2 > 0:
        cb, cc = tuple(phys_a[1][0]), tuple(phys_a[2][0])
        if not A.has_block(cb, cc):
            A.insert_block(np.ones((1, 1)), cb, cc)
            A.insert_block(np.ones((1, 1)), cc, cb)
    pb = ProductBasis(phys_a, phys_b)
    blocks = BlockMatrix()
    basis: Dict = {}
    for (ia, oa), a in zip(A.keys, A.blocks):
        for (ib, ob), b in zip(B.keys, B.blocks):
            nl, nr = fuse(ia, ib), fuse(oa, ob)
            tmp = np.zeros((pb.size(nl), pb.size(nr)))
            r0, c0 = pb(ia, ib), pb(oa, ob)
            tmp[r0:r0 + a.shape[0] * b.shape[0], c0:c0 + a.shape[1] * b.shape[1]] = np.kron(a, b)
            J, Jp = product_spin(ia, ib), product_spin(oa, ob)
            tmp *= mod_coupling(abs(spin(ia)), abs(spin(ib)), J, k1, k2, k, abs(spin(oa)), abs(spin(ob)), Jp)
            blocks.match_and_add_block(tmp, nl, nr)
            rs, cs = basis.get((nl, nr), ([], []))
            rs = rs + [0] * (tmp.shape[0] - len(rs))
            cs = cs + [0] * (tmp.shape[1] - len(cs))
            rs[r0] = J
            cs[c0] = Jp
            basis[(nl, nr)] = (rs, cs)
    c = np.sqrt((jpp + 1.0) * (k + 1.0)) * sixj(j, jp, k, k2, k1, jpp)
    if ((j + jp + k1 + k2) // 2) % 2:
        c = -c
    blocks.scale(c)
    return OOp(blocks, OSpin(k, j, jp), basis)


def op_kron_abelian(phys_a, phys_b, op_a, op_b) -> OOp:
    """``op_kron`` of an abelian group (``bm/site_operator_algorithms.h:167-205``): the
    Kronecker product placed at ProductBasis(phys_a, phys_b) offsets, block pair by
    block pair, no couplings and no spins."""
    A, B = _op_blocks(op_a), _op_blocks(op_b)
    pb = ProductBasis(phys_a, phys_b)
    blocks = BlockMatrix()
    for (ia, oa), a in zip(A.keys, A.blocks):
        for (ib, ob), b in zip(B.keys, B.blocks):
            nl, nr = fuse(ia, ib), fuse(oa, ob)
            tmp = np.zeros((pb.size(nl), pb.size(nr)))
            r0, c0 = pb(ia, ib), pb(oa, ob)
            tmp[r0:r0 + a.shape[0] * b.shape[0], c0:c0 + a.shape[1] * b.shape[1]] = np.kron(a, b)
            blocks.match_and_add_block(tmp, nl, nr)
    return OOp(blocks, OSpin(), {})


def _remove_empty_blocks(op: OOp):
    k = 0
    while k < op.bm.n_blocks():
        if not np.any(op.bm.blocks[k] != 0.0):
            op.bm.remove_block(k)
        else:
            k += 1


def _add_into(dst: OOp, src: OOp, scale: float):
    """dst += scale * src (``SiteOperator::operator+=``)."""
    if dst.bm.n_blocks() == 0:
        dst.spin = src.spin
    for (lc, rc), b in zip(src.bm.keys, src.bm.blocks):
        k = dst.bm.find_block(lc, rc)
        if k < dst.bm.n_blocks():
            dst.bm.blocks[k] = dst.bm.blocks[k] + b * scale
        else:
            dst.bm.insert_block(b * scale, lc, rc)
    for key, (rr, cc) in src.spin_basis.items():
        cur_r, cur_c = dst.spin_basis.get(key, ([], []))
        cur_r = cur_r + [0] * max(0, len(rr) - len(cur_r))
        cur_c = cur_c + [0] * max(0, len(cc) - len(cur_c))
        for i, v in enumerate(rr):
            if v != 0:
                cur_r[i] = v
        for i, v in enumerate(cc):
            if v != 0:
                cur_c[i] = v
        dst.spin_basis[key] = (cur_r, cur_c)


class OHerm:
    """Hermitian partner data of a tensor: partner bond and phase per left/right bond."""

    def __init__(self, left_herm, right_herm, left_phase, right_phase):
        self.LeftHerm, self.RightHerm = list(left_herm), list(right_herm)
        self.LeftPhase, self.RightPhase = list(left_phase), list(right_phase)

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


class OTensor:
    """An MPO tensor: element (b1, b2) -> [(operator index, scale)], operators, bond spins;
    ``symmetry`` "su2u1", or "2u1" / "u1" (abelian)."""

    symmetry = "su2u1"

    def __init__(self, row_dim, col_dim, elements: Dict[Tuple[int, int], List[Tuple[int, float]]], ops: List[OOp],
                 herm: OHerm, left_spins, right_spins):
        self.row_dim, self.col_dim = row_dim, col_dim
        self.elements = elements
        self.op_table = ops
        self.herm = herm
        self.left_spins, self.right_spins = list(left_spins), list(right_spins)
        self._rows: List[List[int]] = [[] for _ in range(row_dim)]
        self._cols: List[List[int]] = [[] for _ in range(col_dim)]
        for (b1, b2) in sorted(elements, key=lambda e: (e[1], e[0])):
            self._cols[b2].append(b1)
        for (b1, b2) in sorted(elements):
            self._rows[b1].append(b2)
        self.num_one_rows = sum(1 for r in self._rows if len(r) == 1)
        self.num_one_cols = sum(1 for c in self._cols if len(c) == 1)

    def has(self, b1, b2):
        return (b1, b2) in self.elements

    def at(self, b1, b2):
        return self.elements[(b1, b2)]

    def row(self, b1):
        return self._rows[b1]

    def column(self, b2):
        return self._cols[b2]

    def left_spin(self, b):
        return self.left_spins[b]

    def right_spin(self, b):
        return self.right_spins[b]

    def op(self, tag):
        return self.op_table[tag]

    def sparse(self, tag):
        return sparse_of(self.op_table[tag])


def make_twosite_mpo(mpo1, mpo2, phys1, phys2) -> OTensor:
    """The two-site tensor of a neighbouring pair of single-site MPO tensors (abelian
    Kronecker products when the tensors are of an abelian group, "2u1" or "u1", where
    every spin is 0)."""
    assert mpo1.col_dim == mpo2.row_dim
    group = getattr(mpo1, "symmetry", "su2u1")
    abelian = group != "su2u1"
    ops: List[OOp] = []
    elements: Dict[Tuple[int, int], List[Tuple[int, float]]] = {}
    for b1 in range(mpo1.row_dim):
        row1 = mpo1.row(b1)
        j = mpo1.left_spin(b1).get()
        for b3 in range(mpo2.col_dim):
            summands = sorted(b2 for b2 in row1 if mpo2.has(b2, b3))
            if not summands:
                continue
            jp = mpo2.right_spin(b3).get()
            per_s: Dict[int, OOp] = {}
            for b2 in summands:
                jpp = mpo1.right_spin(b2).get()
                for t1, s1 in mpo1.at(b1, b2):
                    o1 = mpo1.op(t1)
                    for t2, s2 in mpo2.at(b2, b3):
                        o2 = mpo2.op(t2)
                        for s in allowed_spins(j, jp, o1.spin.get(), o2.spin.get()):
                            if abelian:
                                prod = op_kron_abelian(phys1, phys2, o1, o2)
                            else:
                                prod = op_kron_su2(phys1, phys2, o1, o2, j, jpp, jp, s)
                            _remove_empty_blocks(prod)
                            _add_into(per_s.setdefault(s, OOp()), prod, s1 * s2)
            for s in sorted(per_s):
                ops.append(per_s[s])
                elements.setdefault((b1, b3), []).append((len(ops) - 1, 1.0))
    h1, h2 = mpo1.herm, mpo2.herm
    herm = OHerm(h1.LeftHerm, h2.RightHerm, h1.LeftPhase, h2.RightPhase)
    t = OTensor(mpo1.row_dim, mpo2.col_dim, elements, ops, herm, mpo1.left_spins, mpo2.right_spins)
    t.symmetry = group
    return t


def make_ts_cache_mpo(mpo, phys) -> List[OTensor]:
    """Two-site tensors of every neighbouring pair (``make_ts_cache_mpo``, ``mt/ts_ops.h:164-180``)."""
    return [make_twosite_mpo(mpo[p], mpo[p + 1], phys, phys) for p in range(len(mpo) - 1)]


__all__ = ["OSpin", "OOp", "OHerm", "OTensor", "sparse_of", "allowed_spins", "product_spin", "op_kron_su2",
           "op_kron_abelian",
           "make_twosite_mpo", "make_ts_cache_mpo"]
