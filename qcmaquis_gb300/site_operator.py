"""SU(2) site operators: a small block matrix plus spin bookkeeping.

Restates ``SiteOperator`` (``block_matrix/site_operator.h``,
``site_operator.hpp:93-117, 310-341``), the SU2 ``SpinDescriptor``
(``block_matrix/symmetry/spin_descriptor.h:44-110``), the SU2 ``SparseOperator``
entry list (``block_matrix/sparse_operator.h:105-168``) and the SU2 ``op_kron``
(``block_matrix/site_operator_algorithms.h:214-321``).

Operator blocks are stored as ``(phys_in, phys_out)``: block ``(B, A)`` of the
creator maps a singly-occupied input state ``B`` to the doubly-occupied output
``A`` -- the orientation in which the contraction kernels read them.
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Tuple

import numpy as np

from .block_matrix import BlockMatrix
from .symmetry import Charge, Index, ProductBasis, fuse, spin, triangle
from .wigner import mod_coupling, wigner6j


class SpinDescriptor:
    """(2S, action) of an operator or an MPO bond (``spin_descriptor.h:44-90``)."""

    __slots__ = ("twoS", "diff")

    def __init__(self, twoS: int = 0, inp: int = 0, out: int = 0):
        self.twoS = twoS
        self.diff = out - inp

    @classmethod
    def raw(cls, twoS, diff):
        s = cls()
        s.twoS = twoS
        s.diff = diff
        return s

    def get(self) -> int:
        return self.twoS

    def action(self) -> int:
        return self.diff

    def couple(self, rhs: "SpinDescriptor") -> "SpinDescriptor":
        """Apply the action of ``rhs`` (not symmetric)."""
        return SpinDescriptor.raw(self.twoS + rhs.diff, self.diff)

    def __eq__(self, o):
        return isinstance(o, SpinDescriptor) and self.twoS == o.twoS and self.diff == o.diff

    def __hash__(self):
        return hash((self.twoS, self.diff))

    def __repr__(self):
        return f"Spin({self.twoS},{self.diff})"


class SiteOperator:
    __slots__ = ("bm", "spin", "spin_basis")

    def __init__(self, bm: Optional[BlockMatrix] = None, spin_desc: Optional[SpinDescriptor] = None,
                 spin_basis: Optional[Dict] = None):
        self.bm = bm if bm is not None else BlockMatrix()
        self.spin = spin_desc if spin_desc is not None else SpinDescriptor()
        self.spin_basis: Dict[Tuple[Charge, Charge], Tuple[List[int], List[int]]] = dict(spin_basis or {})

    def copy(self) -> "SiteOperator":
        return SiteOperator(self.bm.copy(), SpinDescriptor.raw(self.spin.twoS, self.spin.diff),
                            {k: (list(v[0]), list(v[1])) for k, v in self.spin_basis.items()})

    def insert_block(self, value, lc, rc):
        self.bm.insert_block(np.array([[float(value)]]), lc, rc)

    def n_blocks(self):
        return self.bm.n_blocks()

    def scaled(self, s: float) -> "SiteOperator":
        o = self.copy()
        o.bm.scale(s)
        return o

    def iadd(self, rhs: "SiteOperator") -> "SiteOperator":
        """``SiteOperator::operator+=`` incl. ``extend_spin_basis``."""
        if self.bm.n_blocks() == 0:
            self.spin = SpinDescriptor.raw(rhs.spin.twoS, rhs.spin.diff)
        self.bm.iadd(rhs.bm)
        for key, (rr, cc) in rhs.spin_basis.items():
            sbr, sbl = self.spin_basis.get(key, ([], []))
            sbr = list(sbr) + [0] * max(0, len(rr) - len(sbr))
            sbl = list(sbl) + [0] * max(0, len(cc) - len(sbl))
            for i in range(min(len(sbr), len(rr))):
                if rr[i] != 0:
                    sbr[i] = rr[i]
            for i in range(min(len(sbl), len(cc))):
                if cc[i] != 0:
                    sbl[i] = cc[i]
            self.spin_basis[key] = (sbr, sbl)
        return self

    def checked_spin_basis(self):
        """``check_spin_basis``: default row/col spins |spin(charge)| if empty."""
        if len(self.spin_basis) == 0:
            sb = {}
            for (lc, rc), b in zip(self.bm.keys, self.bm.blocks):
                sb[(lc, rc)] = ([abs(spin(lc))] * b.shape[0], [abs(spin(rc))] * b.shape[1])
            return sb
        return self.spin_basis

    def sparse(self):
        """Per-block entry lists (row, col, row_spin, col_spin, coeff)."""
        sb = self.checked_spin_basis()
        out = []
        for (lc, rc), b in zip(self.bm.keys, self.bm.blocks):
            ls, rs = sb[(lc, rc)]
            ents = []
            for i in range(b.shape[0]):
                for j in range(b.shape[1]):
                    if b[i, j] != 0.0:
                        ents.append((i, j, ls[i], rs[j], float(b[i, j])))
            out.append(ents)
        return out

    def remove_empty_blocks(self):
        k = 0
        while k < self.bm.n_blocks():
            if not np.any(self.bm.blocks[k] != 0.0):
                self.bm.remove_block(k)
            else:
                k += 1

    def __repr__(self):
        return f"SiteOperator({self.spin}, {self.bm})"


def shape_equal(a: SiteOperator, b: SiteOperator) -> bool:
    return a.bm.basis() == b.bm.basis() and a.spin == b.spin


def op_equal(reference: SiteOperator, sample: SiteOperator):
    """``tag_detail::equal`` (``models/tag_detail.h:55-120``): equal up to a scale."""
    if not shape_equal(reference, sample):
        return False, 0.0
    if sample.bm.n_blocks() == 0:
        return True, 1.0

    def first_inv(m):
        flat = m.ravel(order="C")  # row loop outer, col inner
        for v in flat:
            if abs(v) > 1e-50:
                return 1.0 / v
        return None

    inv1 = first_inv(reference.bm.blocks[0])
    inv2 = first_inv(sample.bm.blocks[0])
    if inv1 is None or inv2 is None:
        return False, 0.0
    for b1, b2 in zip(reference.bm.blocks, sample.bm.blocks):
        if np.any(np.abs(b1 * inv1 - b2 * inv2) > 1e-12):
            return False, 0.0
    return True, inv1 / inv2


def product_spin(a: Charge, b: Charge) -> int:
    """``productSpin`` (``spin_descriptor.h:97-110``)."""
    sa, sb = spin(a), spin(b)
    if sa == -1 and sb == 1:
        return 2
    return abs(sa + sb)


def allowed_spins(left: int, right: int, k1: int, k2: int) -> List[int]:
    """``ts_ops_detail::allowed_spins`` (``mp_tensors/ts_ops.h:21-35``)."""
    ops = list(range(abs(k1 - k2), abs(k1 + k2) + 1, 2))
    return [s for s in ops if abs(s - left) <= right <= abs(s + left)]


def op_kron_su2(phys_A: Index, phys_B: Index, Ao: SiteOperator, Bo: SiteOperator,
                lspin: SpinDescriptor, mspin: SpinDescriptor, rspin: SpinDescriptor,
                target_spin: Optional[SpinDescriptor] = None) -> SiteOperator:
    """Spin-coupled Kronecker product of two site operators (SU2 ``op_kron``)."""
    pb = ProductBasis(phys_A, phys_B)
    A = Ao.copy()
    B = Bo.copy()
    # expand the small identity to the full one (site_operator_algorithms.h:238-256)
    if A.spin.get() > 0 and B.spin.get() == 0:
        cb, cc = phys_B[1][0], phys_B[2][0]
        if not B.bm.has_block(cb, cc):
            B.bm.insert_block(np.ones((1, 1)), cb, cc)
            B.bm.insert_block(np.ones((1, 1)), cc, cb)
    if A.spin.get() == 0 and B.spin.get() > 0:
        cb, cc = phys_A[1][0], phys_A[2][0]
        if not A.bm.has_block(cb, cc):
            A.bm.insert_block(np.ones((1, 1)), cb, cc)
            A.bm.insert_block(np.ones((1, 1)), cc, cb)

    k1, k2 = A.spin.get(), B.spin.get()
    j = lspin.get()
    jpp = mspin.get()
    jp = rspin.get()
    pspins = allowed_spins(j, jp, k1, k2)
    if target_spin is not None and target_spin.get() > -1:
        k = target_spin.get()
    else:
        k = pspins[0]

    blocks = BlockMatrix()
    basis_spins: Dict = {}
    for i in range(A.bm.n_blocks()):
        inA, outA = A.bm.keys[i]
        a_blk = A.bm.blocks[i]
        for jj in range(B.bm.n_blocks()):
            inB, outB = B.bm.keys[jj]
            b_blk = B.bm.blocks[jj]
            new_left = fuse(inA, inB)
            new_right = fuse(outA, outB)
            tmp = np.zeros((pb.size(new_left), pb.size(new_right)))
            in_off = pb(inA, inB)
            out_off = pb(outA, outB)
            # maquis::dmrg::detail::op_kron: out(l1*ld2+l2, r1*rd2+r2) = B(l2,r2)*A(l1,r1)
            for l1 in range(a_blk.shape[0]):
                for r1 in range(a_blk.shape[1]):
                    for l2 in range(b_blk.shape[0]):
                        for r2 in range(b_blk.shape[1]):
                            tmp[in_off + l1 * b_blk.shape[0] + l2, out_off + r1 * b_blk.shape[1] + r2] = \
                                b_blk[l2, r2] * a_blk[l1, r1]
            j1, j2, J = abs(spin(inA)), abs(spin(inB)), product_spin(inA, inB)
            j1p, j2p, Jp = abs(spin(outA)), abs(spin(outB)), product_spin(outA, outB)
            coupling = mod_coupling(j1, j2, J, k1, k2, k, j1p, j2p, Jp)
            tmp = tmp * coupling
            blocks.match_and_add_block(tmp, new_left, new_right)
            key = (new_left, new_right)
            rs, cs = basis_spins.get(key, ([], []))
            rs = list(rs) + [0] * max(0, tmp.shape[0] - len(rs))
            cs = list(cs) + [0] * max(0, tmp.shape[1] - len(cs))
            rs[in_off] = J
            cs[out_off] = Jp
            basis_spins[key] = (rs, cs)

    coupling = math.sqrt((jpp + 1) * (k + 1)) * wigner6j(j, jp, k, k2, k1, jpp)
    if ((j + jp + k1 + k2) // 2) % 2:
        coupling = -coupling
    blocks.scale(coupling)
    C = SiteOperator(blocks, SpinDescriptor(k, j, jp), basis_spins)
    return C


def op_kron_abelian(phys_A: Index, phys_B: Index, Ao: SiteOperator, Bo: SiteOperator) -> SiteOperator:
    """``op_kron`` of an abelian group (``block_matrix/site_operator_algorithms.h:167-205``):
    the Kronecker product of the two operators in ProductBasis(phys_A, phys_B), block
    pair by block pair summed into the fused sectors (no couplings, no spins)."""
    pb = ProductBasis(phys_A, phys_B)
    blocks = BlockMatrix()
    for (inA, outA), a_blk in zip(Ao.bm.keys, Ao.bm.blocks):
        for (inB, outB), b_blk in zip(Bo.bm.keys, Bo.bm.blocks):
            new_left, new_right = fuse(inA, inB), fuse(outA, outB)
            tmp = np.zeros((pb.size(new_left), pb.size(new_right)))
            in_off, out_off = pb(inA, inB), pb(outA, outB)
            for l1 in range(a_blk.shape[0]):
                for r1 in range(a_blk.shape[1]):
                    for l2 in range(b_blk.shape[0]):
                        for r2 in range(b_blk.shape[1]):
                            tmp[in_off + l1 * b_blk.shape[0] + l2, out_off + r1 * b_blk.shape[1] + r2] = \
                                b_blk[l2, r2] * a_blk[l1, r1]
            blocks.match_and_add_block(tmp, new_left, new_right)
    return SiteOperator(blocks, SpinDescriptor(), {})


__all__ = ["SpinDescriptor", "SiteOperator", "op_equal", "shape_equal", "product_spin",
           "allowed_spins", "op_kron_su2", "op_kron_abelian"]
