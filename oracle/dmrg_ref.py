"""Numpy restatement of QCMaquis's SU2U1 two-site DMRG step (oracle; tests only).

Block-sparse tensors, indices and couplings are the oracle's own
(``oracle.qn``, ``oracle.su2``, ``oracle.ts_mpo``), written from the reference
and not from the product package; every algorithm below is written against the
reference files cited in its docstring.  Arithmetic is FP64 throughout.  Work counters (``FLOPS``)
record the algorithmic floating-point work of each GEMM/axpy the reference
algorithm issues, which the benchmark uses as the roofline numerator.
"""
from __future__ import annotations

import math
from typing import Dict, List, Optional, Tuple

import numpy as np

from .qn import (BlockMatrix, Index, ProductBasis, adjoin, bm_gemm, common_subset, fuse, fuse_neg_first,
                 index_product, neg, spin, triangle)
from .su2 import conjugate_correction, mod_coupling, set_coupling, wigner6j
from .ts_mpo import sparse_of

LEFT_PAIRED, RIGHT_PAIRED = 0, 1


class Counters:
    def __init__(self):
        self.reset()

    def reset(self):
        self.gemm_flops = 0
        self.axpy_flops = 0
        self.axpy_bytes = 0

    def gemm(self, m, n, k):
        self.gemm_flops += 2 * m * n * k

    def axpy(self, n):
        self.axpy_flops += 2 * n
        self.axpy_bytes += 24 * n


FLOPS = Counters()


# --------------------------------------------------------------------------- reshapes
def reshape_right_to_left(phys: Index, left_i: Index, right_i: Index, m1: BlockMatrix) -> BlockMatrix:
    """``reshape_right_to_left_new`` (``mp_tensors/reshapes.h:290-338``)."""
    m2 = BlockMatrix()
    in_right = ProductBasis(phys, right_i, fuse_neg_first)
    out_left = ProductBasis(phys, left_i)
    for blk in range(m1.n_blocks()):
        l = left_i.position(m1.left_charge(blk))
        if l == len(left_i):
            continue
        in_l, in_r = left_i[l][0], m1.right_charge(blk)
        for s in range(len(phys)):
            r = right_i.position(fuse(in_r, phys[s][0]))
            if r == len(right_i):
                continue
            out_l = fuse(phys[s][0], in_l)
            out_r = right_i[r][0]
            if not m2.has_block(out_l, out_r):
                m2.insert_block(np.zeros((out_left.size(out_l), right_i[r][1])), out_l, out_r)
            iro = in_right(phys[s][0], out_r)
            olo = out_left(phys[s][0], in_l)
            ob = m2.blocks[m2.find_block(out_l, out_r)]
            ib = m1.blocks[blk]
            sd, ld, rd = phys[s][1], left_i[l][1], right_i[r][1]
            for ss in range(sd):
                ob[olo + ss * ld: olo + (ss + 1) * ld, :rd] = ib[:ld, iro + ss * rd: iro + (ss + 1) * rd]
    return m2


def reshape_left_to_right(phys: Index, left_i: Index, right_i: Index, m1: BlockMatrix) -> BlockMatrix:
    """``reshape_left_to_right_new`` (``mp_tensors/reshapes.h:178-221``)."""
    m2 = BlockMatrix()
    in_left = ProductBasis(phys, left_i)
    out_right = ProductBasis(phys, right_i, fuse_neg_first)
    for blk in range(m1.n_blocks()):
        r = right_i.position(m1.right_charge(blk))
        if r == len(right_i):
            continue
        in_r = right_i[r][0]
        for s in range(len(phys)):
            l = left_i.position(fuse(m1.left_charge(blk), neg(phys[s][0])))
            if l == len(left_i):
                continue
            out_l = left_i[l][0]
            out_r = fuse(neg(phys[s][0]), in_r)
            if not m2.has_block(out_l, out_r):
                m2.insert_block(np.zeros((left_i[l][1], out_right.size(out_r))), out_l, out_r)
            ilo = in_left(phys[s][0], left_i[l][0])
            oro = out_right(phys[s][0], in_r)
            ob = m2.blocks[m2.find_block(out_l, out_r)]
            ib = m1.blocks[blk]
            sd, ld, rd = phys[s][1], left_i[l][1], right_i[r][1]
            for ss in range(sd):
                ob[:ld, oro + ss * rd: oro + (ss + 1) * rd] = ib[ilo + ss * ld: ilo + (ss + 1) * ld, :rd]
    return m2


# --------------------------------------------------------------------------- MPSTensor
class MPSTensor:
    """``MPSTensor`` (``mp_tensors/mpstensor.hpp:25-330``) with lazy pairing."""

    def __init__(self, phys: Index, left_i: Index, right_i: Index, data: BlockMatrix, layout: int):
        self.phys_i = phys
        self.left_i = left_i
        self.right_i = right_i
        self.data = data
        self.layout = layout

    @classmethod
    def from_block(cls, phys, left_i, right_i, block: BlockMatrix, layout: int):
        """Constructor from a block_matrix (``mpstensor.hpp:63-96``)."""
        if layout == LEFT_PAIRED:
            new_right = block.right_basis()
            possible_left = index_product(adjoin(phys), new_right)
            old_left = left_i.copy()
            common_subset(old_left, possible_left)
            return cls(phys, old_left, new_right, block, layout)
        new_left = block.left_basis()
        possible_right = index_product(phys, new_left)
        old_right = right_i.copy()
        common_subset(old_right, possible_right)
        return cls(phys, new_left, old_right, block, layout)

    def copy(self):
        return MPSTensor(self.phys_i, self.left_i.copy(), self.right_i.copy(), self.data.copy(), self.layout)

    def make_left_paired(self):
        if self.layout == LEFT_PAIRED:
            return self
        self.data = reshape_right_to_left(self.phys_i, self.left_i, self.right_i, self.data)
        self.layout = LEFT_PAIRED
        return self

    def make_right_paired(self):
        if self.layout == RIGHT_PAIRED:
            return self
        self.data = reshape_left_to_right(self.phys_i, self.left_i, self.right_i, self.data)
        self.layout = RIGHT_PAIRED
        return self

    # vector-space operations used by the eigensolver (both operands left-paired)
    def dot(self, other: "MPSTensor") -> float:
        """``scalar_overlap`` (``mpstensor.hpp:365-380``, ``block_matrix.hpp:575-590``)."""
        self.make_left_paired()
        other.make_left_paired()
        s = 0.0
        for (k, b) in zip(self.data.keys, self.data.blocks):
            p = other.data.find_block(*k)
            if p < other.data.n_blocks():
                s += float(np.vdot(b, other.data.blocks[p]))
        return s

    def norm(self) -> float:
        return self.data.norm()

    def scaled(self, a: float) -> "MPSTensor":
        out = self.copy()
        out.data.scale(a)
        return out

    def axpy(self, a: float, x: "MPSTensor") -> "MPSTensor":
        """self += a * x (block-matched, missing blocks inserted)."""
        self.make_left_paired()
        x.make_left_paired()
        for (k, b) in zip(x.data.keys, x.data.blocks):
            p = self.data.find_block(*k)
            if p < self.data.n_blocks():
                self.data.blocks[p] = self.data.blocks[p] + a * b
            else:
                self.data.insert_block(a * b, *k)
        return self


# --------------------------------------------------------------------------- QR / LQ
def block_qr(M: BlockMatrix):
    """Thin QR per block (``block_matrix_algorithms.h:442-466``)."""
    Q, R = BlockMatrix(), BlockMatrix()
    for (lc, rc), b in zip(M.keys, M.blocks):
        q, r = np.linalg.qr(b, mode="reduced")
        Q.insert_block(q, lc, rc)
        R.insert_block(r, rc, rc)
    return Q, R


def block_lq(M: BlockMatrix):
    """Thin LQ per block (``block_matrix_algorithms.h:468-492``)."""
    Lm, Q = BlockMatrix(), BlockMatrix()
    for (lc, rc), b in zip(M.keys, M.blocks):
        q, r = np.linalg.qr(b.T, mode="reduced")
        Lm.insert_block(r.T, lc, lc)
        Q.insert_block(q.T, lc, rc)
    return Lm, Q


def left_normalize_and_return(t: MPSTensor) -> BlockMatrix:
    """``leftNormalizeAndReturn`` with QR (``mpstensor.hpp:219-238, 283-292``)."""
    t.make_left_paired()
    Q, R = block_qr(t.data)
    t.data = Q
    t.right_i = Q.right_basis()
    return R


def right_normalize_and_return(t: MPSTensor) -> BlockMatrix:
    """``rightNormalizeAndReturn`` with LQ (``mpstensor.hpp:240-258, 294-302``)."""
    t.make_right_paired()
    Lm, Q = block_lq(t.data)
    t.data = Q
    t.left_i = Q.left_basis()
    return Lm


def multiply_from_left(t: MPSTensor, N: BlockMatrix):
    """``multiply_from_left`` (``mpstensor.hpp:323-330``)."""
    t.make_right_paired()
    tmp = bm_gemm(N, t.data)
    new = MPSTensor.from_block(t.phys_i, t.left_i, t.right_i, tmp, RIGHT_PAIRED)
    t.left_i, t.right_i, t.data, t.layout = new.left_i, new.right_i, new.data, RIGHT_PAIRED


def multiply_from_right(t: MPSTensor, N: BlockMatrix):
    """``multiply_from_right`` (``mpstensor.hpp:312-320``)."""
    t.make_left_paired()
    tmp = bm_gemm(t.data, N)
    new = MPSTensor.from_block(t.phys_i, t.left_i, t.right_i, tmp, LEFT_PAIRED)
    t.left_i, t.right_i, t.data, t.layout = new.left_i, new.right_i, new.data, LEFT_PAIRED


# --------------------------------------------------------------------------- MPS init
def allowed_sectors(L: int, phys: Index, right_end, Mmax: int, abelian: bool = False) -> List[Index]:
    """``allowed_sectors`` (``mp_tensors/mps_sectors.h:23-112``), one site type; the
    test that a sector's spin is not negative (``ChargeDetailClass::physical``) is
    SU(2)'s and is skipped for an abelian group."""
    physc = phys.copy()
    physc.sort()
    cmax, cmin = physc[0][0], physc[len(physc) - 1][0]
    if cmin > cmax:
        cmax, cmin = cmin, cmax
    maxt, mint = (0, 0), (0, 0)
    for _ in range(L):
        maxt = fuse(maxt, cmax)
        mint = fuse(mint, cmin)
    left = [None] * (L + 1)
    right = [None] * (L + 1)
    left[0] = Index([((0, 0), 1)])
    right[L] = Index([(right_end, 1)])
    cmaxi, cmini = maxt, mint
    for i in range(1, L + 1):
        li = index_product(phys, left[i - 1])
        cmaxi = fuse(cmaxi, neg(cmax))
        cmini = fuse(cmini, neg(cmin))
        keep = []
        for c, s in li:
            if fuse(c, cmaxi) < right_end:
                continue
            if fuse(c, cmini) > right_end:
                continue
            if not abelian and spin(c) < 0:
                continue
            keep.append([c, min(Mmax, s)])
        li.data = keep
        left[i] = li
    cmaxi, cmini = maxt, mint
    for i in range(L - 1, -1, -1):
        ri = index_product(adjoin(phys), right[i + 1])
        cmaxi = fuse(cmaxi, neg(cmax))
        cmini = fuse(cmini, neg(cmin))
        keep = []
        for c, s in ri:
            if fuse(c, neg(cmaxi)) > (0, 0):
                continue
            if fuse(c, neg(cmini)) < (0, 0):
                continue
            if not abelian and spin(c) < 0:
                continue
            keep.append([c, min(Mmax, s)])
        ri.data = keep
        right[i] = ri
        common_subset(left[i], right[i])
    allowed = []
    for i in range(L + 1):
        a = left[i].copy()
        b = right[i].copy()
        common_subset(a, b)
        a.data = [[c, min(Mmax, left[i].size_of_block(c), right[i].size_of_block(c))] for c, _ in a]
        allowed.append(a)
    return allowed


def new_mps_tensor(phys: Index, ld: Index, rd: Index, rng: Optional[np.random.Generator]) -> MPSTensor:
    """Random MPSTensor (``mpstensor.hpp:25-60``); blocks filled column-major."""
    lb = index_product(phys, ld)
    rb = rd.copy()
    common_subset(lb, rb)
    right_i = rb.copy()
    possible_rp = index_product(adjoin(phys), right_i)
    left_i = ld.copy()
    common_subset(left_i, possible_rp)
    data = BlockMatrix.from_indices(lb, rb)
    if rng is not None:
        for k in range(data.n_blocks()):
            b = data.blocks[k]
            data.blocks[k] = rng.random(b.size).reshape(b.shape, order="F")
    return MPSTensor(phys, left_i, right_i, data, LEFT_PAIRED)


def default_mps_init(L, phys, right_end, init_bond_dimension, seed, abelian: bool = False) -> List[MPSTensor]:
    """``default_mps_init`` (``mp_tensors/mps_initializers.h:34-81``).

    The element stream comes from numpy's PCG64 seeded with ``seed`` rather
    than boost's mt19937, so the initial MPS is this repository's own.
    """
    rng = np.random.default_rng(seed)
    allowed = allowed_sectors(L, phys, right_end, init_bond_dimension, abelian)
    mps = []
    for i in range(L):
        t = new_mps_tensor(phys, allowed[i], allowed[i + 1], rng)
        t.data.scale(1.0 / t.norm())
        mps.append(t)
    return mps


def normalize_right(mps: List[MPSTensor]):
    """``MPS::normalize_right`` = canonize(0) then LQ of site 0 (``mps.hpp:117-128``)."""
    L = len(mps)
    for i in range(L - 1, 0, -1):
        t = right_normalize_and_return(mps[i])
        multiply_from_right(mps[i - 1], t)
    nf = right_normalize_and_return(mps[0])
    if nf.trace() < 0:
        mps[0].data.scale(-1.0)


def left_boundary(mps0: MPSTensor) -> List[BlockMatrix]:
    """``MPS::left_boundary`` (``mps.hpp:242-254``): ones on the diagonal blocks."""
    i = mps0.left_i
    return [BlockMatrix.from_indices(i, i, fill=1.0)]


def right_boundary(mpsL: MPSTensor) -> List[BlockMatrix]:
    i = mpsL.right_i
    return [BlockMatrix.from_indices(i, i, fill=1.0)]


# --------------------------------------------------------------------------- SU2 gemms
def conjugate_phases(bm: BlockMatrix, mpo, k, left: bool, forward: bool) -> List[float]:
    """``conjugate_phases`` (``ct/common/boundary_times_mps.hpp:19-43``)."""
    S = mpo.left_spin(k).get() if left else mpo.right_spin(k).get()
    h = mpo.herm
    if forward:
        ph = h.left_phase(h.left_conj(k)) if left else h.right_phase(h.right_conj(k))
    else:
        ph = h.left_phase(k) if left else h.right_phase(k)
    return [conjugate_correction(spin(lc), spin(rc), S) * ph for (lc, rc) in bm.keys]


def gemm_trim_left(A: BlockMatrix, B: BlockMatrix, ref: Index, scales=None) -> BlockMatrix:
    """``SU2::gemm_trim_left`` (``ct/non-abelian/gemm.hpp:78-115``)."""
    if scales is None or len(scales) != A.n_blocks():
        scales = [1.0] * A.n_blocks()
    C = BlockMatrix()
    for k in range(A.n_blocks()):
        if not ref.has(A.left_charge(k)):
            continue
        ar = A.right_charge(k)
        it = B.left_lower_bound(ar)
        while it < B.n_blocks() and B.keys[it][0] == ar:
            lc, rc = A.left_charge(k), B.keys[it][1]
            prod = scales[k] * (A.blocks[k] @ B.blocks[it])
            FLOPS.gemm(A.blocks[k].shape[0], B.blocks[it].shape[1], A.blocks[k].shape[1])
            p = C.find_block(lc, rc)
            if p < C.n_blocks():
                C.blocks[p] = C.blocks[p] + prod
            else:
                C.insert_block(prod, lc, rc)
            it += 1
    return C


def gemm_trim_right(A: BlockMatrix, B: BlockMatrix, ref: Index, scales=None) -> BlockMatrix:
    """``SU2::gemm_trim_right`` (``ct/non-abelian/gemm.hpp:144-176``)."""
    if scales is None or len(scales) != B.n_blocks():
        scales = [1.0] * B.n_blocks()
    C = BlockMatrix()
    for k in range(A.n_blocks()):
        ar = A.right_charge(k)
        it = B.left_lower_bound(ar)
        while it < B.n_blocks() and B.keys[it][0] == ar:
            if not ref.has(B.keys[it][1]):
                it += 1
                continue
            lc, rc = A.left_charge(k), B.keys[it][1]
            prod = scales[it] * (A.blocks[k] @ B.blocks[it])
            FLOPS.gemm(A.blocks[k].shape[0], B.blocks[it].shape[1], A.blocks[k].shape[1])
            p = C.find_block(lc, rc)
            if p < C.n_blocks():
                C.blocks[p] = C.blocks[p] + prod
            else:
                C.insert_block(prod, lc, rc)
            it += 1
    return C


def gemm_trim(A: BlockMatrix, B: BlockMatrix, scales, conjugate_a: bool) -> BlockMatrix:
    """``SU2::gemm_trim`` (``ct/non-abelian/gemm.hpp:178-204``)."""
    C = BlockMatrix()
    for k in range(A.n_blocks()):
        al, ar = A.keys[k]
        m = B.find_block(ar, al)
        if m == B.n_blocks():
            continue
        s = scales[k] if conjugate_a else scales[m]
        prod = s * (A.blocks[k] @ B.blocks[m])
        FLOPS.gemm(A.blocks[k].shape[0], B.blocks[m].shape[1], A.blocks[k].shape[1])
        p = C.find_block(al, al)
        if p < C.n_blocks():
            C.blocks[p] = C.blocks[p] + prod
        else:
            C.insert_block(prod, al, al)
    return C


def su2_gemm(A: BlockMatrix, B: BlockMatrix, spin_filter: int) -> BlockMatrix:
    """``SU2::gemm`` with triangle filter (``ct/non-abelian/gemm.hpp:48-75``)."""
    C = BlockMatrix()
    for k in range(A.n_blocks()):
        ar = A.right_charge(k)
        it = B.left_lower_bound(ar)
        while it < B.n_blocks() and B.keys[it][0] == ar:
            if spin_filter != -1 and not triangle(spin(A.left_charge(k)), spin_filter, spin(B.keys[it][1])):
                it += 1
                continue
            lc, rc = A.left_charge(k), B.keys[it][1]
            prod = A.blocks[k] @ B.blocks[it]
            FLOPS.gemm(A.blocks[k].shape[0], B.blocks[it].shape[1], A.blocks[k].shape[1])
            p = C.find_block(lc, rc)
            if p < C.n_blocks():
                C.blocks[p] = C.blocks[p] + prod
            else:
                C.insert_block(prod, lc, rc)
            it += 1
    return C


# --------------------------------------------------------------------------- boundary x MPS
def boundary_mps_product(ket_rp: BlockMatrix, left: List[BlockMatrix], mpo, ref: Index,
                         is_hermitian=True) -> List[BlockMatrix]:
    """``BoundaryMPSProduct::populateData`` + ``at`` (``boundary_times_mps.hpp:163-209``).

    All rows are evaluated eagerly; the reference defers single-use rows to
    ``at()``, which computes the same product.
    """
    out = []
    h = mpo.herm
    for b1 in range(len(left)):
        if h.left_skip(b1) and is_hermitian:
            lc = left[h.left_conj(b1)]
            scales = conjugate_phases(lc, mpo, b1, True, False)
            out.append(gemm_trim_left(lc, ket_rp, ref, scales))
        else:
            out.append(gemm_trim_left(left[b1].transpose(), ket_rp, ref))
    return out


def mps_boundary_product(ket_lp: BlockMatrix, right: List[BlockMatrix], mpo, ref: Index,
                         is_hermitian=True) -> List[BlockMatrix]:
    """``MPSBoundaryProduct::populateData`` + ``at`` (``boundary_times_mps.hpp:226-385``)."""
    out = []
    h = mpo.herm
    for b2 in range(len(right)):
        if h.right_skip(b2) and is_hermitian:
            trv = right[h.right_conj(b2)].transpose()
            scales = conjugate_phases(trv, mpo, b2, False, True)
            out.append(gemm_trim_right(ket_lp, trv, ref, scales))
        else:
            out.append(gemm_trim_right(ket_lp, right[b2], ref))
    return out


# --------------------------------------------------------------------------- lbtm / rbtm kernels
def lbtm_kernel(b2, T: List[BlockMatrix], mpo, right_i: Index, out_left_i: Index,
                in_right_pb: ProductBasis, out_left_pb: ProductBasis) -> BlockMatrix:
    """``SU2::lbtm_kernel`` + ``detail::lbtm`` (``apply_op.hpp:23-101``, ``micro_kernels.hpp:19-45``).

    The ket basis is block-diagonal, so the ket charge matched to a T block's
    right charge is that charge itself.
    """
    ret = BlockMatrix()
    for b1 in mpo.column(b2):
        Tb = T[b1]
        for tag, scale in mpo.at(b1, b2):
            W = mpo.op(tag)
            wsparse = sparse_of(mpo.op(tag))
            a = mpo.left_spin(b1).get()
            k = W.spin.get()
            ap = mpo.right_spin(b2).get()
            for t in range(Tb.n_blocks()):
                lc, rc = Tb.keys[t]
                mc = rc
                iblock = Tb.blocks[t]
                l_size = iblock.shape[0]
                for wb in range(W.bm.n_blocks()):
                    phys_in, phys_out = W.bm.keys[wb]
                    out_r = fuse(rc, phys_in)
                    rb = right_i.position(out_r)
                    if rb == len(right_i):
                        continue
                    out_l = fuse(lc, phys_out)
                    if not triangle(spin(out_r), ap, spin(out_l)):
                        continue
                    if not out_left_i.has(out_l):
                        continue
                    r_size = right_i[rb][1]
                    o = ret.find_block(out_l, out_r)
                    if o == ret.n_blocks():
                        o = ret.insert_block(np.zeros((out_left_i.size_of_block(out_l), r_size)), out_l, out_r)
                    i, ip = spin(lc), spin(out_l)
                    j, jp = spin(mc), spin(out_r)
                    cpl = set_coupling(j, abs(j - jp), jp, a, k, ap, i, abs(i - ip), ip, scale)
                    iro = in_right_pb(phys_in, out_r)
                    olo = out_left_pb(phys_out, lc)
                    ob = ret.blocks[o]
                    for (ss1, ss2, rspin, cspin, coeff) in wsparse[wb]:
                        case = 3 if (rspin == 2 and cspin == 2) else (1 if rspin == 2 else (2 if cspin == 2 else 0))
                        alfa = coeff * cpl[case]
                        ob[olo + ss2 * l_size: olo + (ss2 + 1) * l_size, :r_size] += \
                            alfa * iblock[:, iro + ss1 * r_size: iro + (ss1 + 1) * r_size]
                        FLOPS.axpy(l_size * r_size)
    return ret


def rbtm_tasks_apply(b1, t: List[BlockMatrix], mpo, left_i: Index, out_right_i: Index,
                     in_left_pb: ProductBasis, out_right_pb: ProductBasis):
    """``SU2::rbtm_tasks`` + ``task_axpy`` (``apply_op.hpp:114-209``, ``micro_kernels.hpp:182-198``).

    Returns {(out_l, out_r): buffer}, each buffer l_size x size(out_r).  The
    reference splits each stripe into cache-sized chunks; the sums are equal.
    """
    bufs: Dict = {}
    for b2 in mpo.row(b1):
        Tb = t[b2]
        for tag, scale in mpo.at(b1, b2):
            W = mpo.op(tag)
            wsparse = sparse_of(mpo.op(tag))
            a = mpo.left_spin(b1).get()
            k = W.spin.get()
            ap = mpo.right_spin(b2).get()
            for tb in range(Tb.n_blocks()):
                lc, rc = Tb.keys[tb]
                mc = lc
                iblock = Tb.blocks[tb]
                for wb in range(W.bm.n_blocks()):
                    phys_in, phys_out = W.bm.keys[wb]
                    out_l = fuse(lc, neg(phys_in))
                    lb = left_i.position(out_l)
                    if lb == len(left_i):
                        continue
                    out_r = fuse(rc, neg(phys_out))
                    if not triangle(spin(out_l), a, spin(out_r)):
                        continue
                    if not out_right_i.has(out_r):
                        continue
                    l_size = left_i[lb][1]
                    i, ip = spin(out_r), spin(rc)
                    j, jp = spin(out_l), spin(mc)
                    cpl = set_coupling(j, abs(j - jp), jp, a, k, ap, i, abs(i - ip), ip, scale)
                    ilo = in_left_pb(phys_in, out_l)
                    oro = out_right_pb(phys_out, rc)
                    r_size = iblock.shape[1]
                    key = (out_l, out_r)
                    if key not in bufs:
                        bufs[key] = np.zeros((l_size, out_right_i.size_of_block(out_r)))
                    buf = bufs[key]
                    for (ss1, ss2, rspin, cspin, coeff) in wsparse[wb]:
                        case = 3 if (rspin == 2 and cspin == 2) else (1 if rspin == 2 else (2 if cspin == 2 else 0))
                        alfa = coeff * cpl[case]
                        buf[:, oro + ss2 * r_size: oro + (ss2 + 1) * r_size] += \
                            alfa * iblock[ilo + ss1 * l_size: ilo + (ss1 + 1) * l_size, :r_size]
                        FLOPS.axpy(l_size * r_size)
    return bufs


# --------------------------------------------------------------------------- site Hamiltonian
def site_hamil_lbtm(ket: MPSTensor, left: List[BlockMatrix], right: List[BlockMatrix], mpo,
                    is_hermitian=True) -> MPSTensor:
    """``site_hamil_lbtm`` (``ct/non-abelian/site_hamil.hpp:57-147``); bra = ket."""
    ket = ket.copy()
    bra = ket
    phys = ket.phys_i
    left_i = bra.left_i
    right_i = ket.right_i
    out_left_i = index_product(phys, left_i)
    rib = bra.right_i.copy()
    common_subset(out_left_i, rib)
    out_left_pb = ProductBasis(phys, left_i)
    in_right_pb = ProductBasis(phys, right_i, fuse_neg_first)
    ket.make_right_paired()
    ref = ket.data.left_basis()
    T = boundary_mps_product(ket.data, left, mpo, ref, is_hermitian)
    h = mpo.herm
    out = BlockMatrix()
    for b2 in range(mpo.col_dim):
        contr = lbtm_kernel(b2, T, mpo, right_i, out_left_i, in_right_pb, out_left_pb)
        if h.right_skip(b2) and is_hermitian:
            Radj = right[h.right_conj(b2)].transpose()
            phases = conjugate_phases(Radj, mpo, b2, False, True)
            tmp = gemm_trim(contr, Radj, phases, False)
        else:
            tmp = gemm_trim(contr, right[b2], [1.0] * contr.n_blocks(), True)
        for k in range(tmp.n_blocks()):
            out.match_and_add_block(tmp.blocks[k], *tmp.keys[k])
    return MPSTensor(phys, bra.left_i, bra.right_i, out, LEFT_PAIRED)


def site_hamil_rbtm(ket: MPSTensor, left: List[BlockMatrix], right: List[BlockMatrix], mpo,
                    is_hermitian=True) -> MPSTensor:
    """``site_hamil_rbtm`` (``ct/non-abelian/site_hamil.hpp:149-204``) with
    ``rbtm_axpy_gemm`` / ``charge_gemm`` (``apply_op.hpp:257-298``); bra = ket."""
    ket = ket.copy()
    bra = ket
    ket.make_left_paired()
    ref = ket.data.left_basis()
    t = mps_boundary_product(ket.data, right, mpo, ref, is_hermitian)
    phys = ket.phys_i
    right_i = bra.right_i
    left_i = ket.left_i
    out_right_i = index_product(adjoin(phys), right_i)
    lik = ket.left_i.copy()
    common_subset(out_right_i, lik)
    in_left_pb = ProductBasis(phys, left_i)
    out_right_pb = ProductBasis(phys, right_i, fuse_neg_first)
    collector = BlockMatrix()
    h = mpo.herm
    for b1 in range(mpo.row_dim):
        bufs = rbtm_tasks_apply(b1, t, mpo, left_i, out_right_i, in_left_pb, out_right_pb)
        if h.left_skip(b1) and is_hermitian:
            left_b1 = left[h.left_conj(b1)]
            phases = conjugate_phases(left_b1, mpo, b1, True, False)
        else:
            left_b1 = left[b1].transpose()
            phases = [1.0] * left_b1.n_blocks()
        prod = BlockMatrix()
        for (out_l, out_r) in sorted(bufs, reverse=True):
            k = left_b1.find_block(out_r, out_l)
            if k == left_b1.n_blocks():
                continue
            g = phases[k] * (left_b1.blocks[k] @ bufs[(out_l, out_r)])
            FLOPS.gemm(left_b1.blocks[k].shape[0], bufs[(out_l, out_r)].shape[1], left_b1.blocks[k].shape[1])
            prod.match_and_add_block(g, out_r, out_r)
        for k in range(prod.n_blocks()):
            collector.match_and_add_block(prod.blocks[k], *prod.keys[k])
    data = reshape_right_to_left(phys, left_i, right_i, collector)
    return MPSTensor(phys, bra.left_i, bra.right_i, data, LEFT_PAIRED)


def site_hamil2(ket: MPSTensor, left, right, mpo, is_hermitian=True, force=None) -> MPSTensor:
    """``Engine::site_hamil2`` dispatch (``ct/non-abelian/site_hamil.hpp:28-38``)."""
    use_lbtm = (mpo.row_dim - mpo.num_one_rows) < (mpo.col_dim - mpo.num_one_cols)
    if force == "lbtm" or (force is None and use_lbtm):
        return site_hamil_lbtm(ket, left, right, mpo, is_hermitian)
    return site_hamil_rbtm(ket, left, right, mpo, is_hermitian)


def zerosite_hamil(bond: BlockMatrix, left: List[BlockMatrix], right: List[BlockMatrix], mpo_left, mpo_right,
                   is_hermitian=True) -> BlockMatrix:
    """``zerosite_hamil_lbtm_kernel`` (``ct/non-abelian/zero_site_hamil.hpp:44-79``), bra = ket.

    ``bond`` is the bond matrix C between sites i and i+1, ``left`` = L[i+1],
    ``right`` = R[i+1], ``mpo_left`` = W[i], ``mpo_right`` = W[i+1].  For every bond
    index b: T[b] = L[b]^T C (``BoundaryMPSProduct`` over C with
    ``correctConjugate = false``: a Hermitian partner enters as L[conj b] with no
    phase), then sigma += T[b] R[b] (``gemm_trim`` with unit scales; a partner as
    R[conj b]^T, again with no phase).  The skip test is W[i+1]'s left one, the
    right partner index W[i]'s right one, as in the reference."""
    ref = bond.left_basis()
    hr, hl = mpo_right.herm, mpo_left.herm
    out = BlockMatrix()
    for b in range(mpo_right.row_dim):
        conj = is_hermitian and hr.left_skip(b)
        if conj:
            T = gemm_trim_left(left[hr.left_conj(b)], bond, ref)
            Radj = right[hl.right_conj(b)].transpose()
            tmp = gemm_trim(T, Radj, [1.0] * Radj.n_blocks(), False)
        else:
            T = gemm_trim_left(left[b].transpose(), bond, ref)
            tmp = gemm_trim(T, right[b], [1.0] * T.n_blocks(), True)
        for k in range(tmp.n_blocks()):
            out.match_and_add_block(tmp.blocks[k], *tmp.keys[k])
    return out


def diagonal_hamiltonian(left: List[BlockMatrix], right: List[BlockMatrix], mpo, x: MPSTensor) -> BlockMatrix:
    """``SU2::diagonal_hamiltonian`` + ``lbtm_diag_kernel`` (``ct/non-abelian/h_diag.hpp:13-158``):
    the diagonal of H_eff in x's left-paired layout.  Reads L[b1] and R[b2] for
    every bond index (no Hermitian partners), so the boundaries must hold every b.
    Per b2 and every MPO term of its column, the diagonal entries (row == col) of
    the operator add coeff * coupling * diag(L[b1](lc, lc)) to the rows of
    (phys, lc) in every column of the output block; the per-b2 block is then
    scaled column by column by diag(R[b2](rc, rc)) and added in, when R[b2]
    has that block."""
    phys = x.phys_i
    xs = x.copy().make_left_paired()
    right_i = xs.right_i.copy()
    out_left_i = index_product(phys, xs.left_i)
    common_subset(out_left_i, right_i)
    left_pb = ProductBasis(phys, xs.left_i)
    ret = BlockMatrix()
    for b2 in range(len(right)):
        lb2 = BlockMatrix()
        ap = mpo.right_spin(b2).get()
        for b1 in mpo.column(b2):
            a = mpo.left_spin(b1).get()
            for tag, scale in mpo.at(b1, b2):
                W = mpo.op(tag)
                wsparse = sparse_of(mpo.op(tag))
                k = W.spin.get()
                for blk in range(len(right_i)):
                    in_charge = right_i[blk][0]
                    o = lb2.find_block(in_charge, in_charge)
                    if o == lb2.n_blocks():
                        o = lb2.insert_block(np.zeros((out_left_i[blk][1], right_i[blk][1])), in_charge, in_charge)
                    for pc, _pd in phys:
                        lin = fuse(in_charge, neg(pc))
                        if not xs.left_i.has(lin):
                            continue
                        l = xs.left_i.position(lin)
                        lc, ld = xs.left_i[l]
                        lk = left[b1].find_block(lc, lc)
                        if lk == left[b1].n_blocks():
                            continue
                        ldiag = np.diagonal(left[b1].blocks[lk])[:ld]
                        loff = left_pb(pc, lc)
                        for wb in range(W.bm.n_blocks()):
                            p_in, p_out = W.bm.keys[wb]
                            if pc != p_in or p_in != p_out:
                                continue
                            i, ip, j, jp = spin(lc), spin(in_charge), spin(lc), spin(in_charge)
                            pref = math.sqrt((ip + 1.0) * (j + 1.0) / ((i + 1.0) * (jp + 1.0))) * scale
                            c0 = pref * mod_coupling(j, abs(j - jp), jp, a, k, ap, i, abs(i - ip), ip)
                            c1 = pref * mod_coupling(j, 2, jp, a, k, ap, i, 2, ip)
                            for (ss1, ss2, rspin, _cspin, coeff) in wsparse[wb]:
                                if ss1 != ss2:
                                    continue
                                alfa = coeff * (c1 if rspin == 2 else c0)
                                lb2.blocks[o][loff + ss1 * ld:loff + (ss1 + 1) * ld, :] += (alfa * ldiag)[:, None]
        for (lc, rc), blk in zip(lb2.keys, lb2.blocks):
            rk = right[b2].find_block(rc, rc)
            if rk == right[b2].n_blocks():
                continue
            rdiag = np.diagonal(right[b2].blocks[rk])[:blk.shape[1]]
            ret.match_and_add_block(blk * rdiag[None, :], rc, rc)
    return ret


# --------------------------------------------------------------------------- boundary steps
def overlap_mpo_left_step(bra: MPSTensor, ket: MPSTensor, left: List[BlockMatrix], mpo,
                          is_hermitian=True) -> List[BlockMatrix]:
    """``overlap_mpo_left_step`` (``ct/common/move_boundary.hpp:128-187``)."""
    bra = bra.copy()
    ket = ket.copy()
    bra.make_right_paired()
    bra_basis_idx = bra.data.left_basis()
    ket.make_right_paired()
    T = boundary_mps_product(ket.data, left, mpo, bra_basis_idx, is_hermitian)
    left_i = bra.left_i
    right_i = ket.right_i
    out_left_i = index_product(bra.phys_i, left_i)
    bri = bra.right_i.copy()
    common_subset(out_left_i, bri)
    out_left_pb = ProductBasis(bra.phys_i, left_i)
    in_right_pb = ProductBasis(ket.phys_i, right_i, fuse_neg_first)
    bra.make_left_paired()
    bra_conj = bra.data
    h = mpo.herm
    ret = [BlockMatrix() for _ in range(mpo.col_dim)]
    for b2 in range(mpo.col_dim):
        if h.right_skip(b2) and is_hermitian:
            continue
        contr = lbtm_kernel(b2, T, mpo, right_i, out_left_i, in_right_pb, out_left_pb)
        ret[b2] = su2_gemm(contr.transpose(), bra_conj, mpo.right_spin(b2).get())
    return ret


def overlap_mpo_right_step(bra: MPSTensor, ket: MPSTensor, right: List[BlockMatrix], mpo,
                           is_hermitian=True) -> List[BlockMatrix]:
    """``overlap_mpo_right_step`` (``ct/common/move_boundary.hpp:189-229``)."""
    bra = bra.copy()
    ket = ket.copy()
    phys = ket.phys_i
    right_i = bra.right_i
    left_i = ket.left_i
    out_right_i = index_product(adjoin(phys), right_i)
    bra.make_left_paired()
    index_for_trim = bra.data.right_basis()
    ket.make_left_paired()
    t = mps_boundary_product(ket.data, right, mpo, index_for_trim, is_hermitian)
    bli = bra.left_i.copy()
    common_subset(out_right_i, bli)
    in_left_pb = ProductBasis(phys, left_i)
    out_right_pb = ProductBasis(phys, right_i, fuse_neg_first)
    bra.make_right_paired()
    bra_conj_T = bra.data.transpose()
    h = mpo.herm
    ret = [BlockMatrix() for _ in range(mpo.row_dim)]
    for b1 in range(mpo.row_dim):
        if h.left_skip(b1) and is_hermitian:
            continue
        bufs = rbtm_tasks_apply(b1, t, mpo, left_i, out_right_i, in_left_pb, out_right_pb)
        blk = BlockMatrix()
        for key in bufs:
            blk.insert_block(bufs[key], *key)
        ret[b1] = su2_gemm(blk, bra_conj_T, mpo.left_spin(b1).get())
    return ret


# --------------------------------------------------------------------------- overlap boundaries
def overlap_left_step(bra: MPSTensor, ket: MPSTensor, left: BlockMatrix) -> BlockMatrix:
    """``common::overlap_left_step`` with ``SU2::gemm`` (``ct/common/move_boundary.hpp:20-40``):
    the MPO-free left step of <bra|ket>; blocks keyed (bra charge, ket charge)."""
    k = ket.copy().make_right_paired()
    t1 = su2_gemm(left, k.data, -1)
    t3 = reshape_right_to_left(k.phys_i, bra.left_i, k.right_i, t1)
    b = bra.copy().make_left_paired()
    return su2_gemm(b.data.transpose(), t3, -1)


def overlap_right_step(bra: MPSTensor, ket: MPSTensor, right: BlockMatrix) -> BlockMatrix:
    """``common::overlap_right_step`` (``ct/common/move_boundary.hpp:45-62``)."""
    k = ket.copy().make_left_paired()
    t1 = su2_gemm(k.data, right.transpose(), -1)
    t3 = reshape_left_to_right(k.phys_i, k.left_i, bra.right_i, t1)
    b = bra.copy().make_right_paired()
    return su2_gemm(b.data, t3.transpose(), -1)


def reshape_and_pad_left(phys: Index, in_left_i: Index, in_right_i: Index, out_left_i: Index,
                         m1: BlockMatrix, m2: BlockMatrix) -> BlockMatrix:
    """``reshape_and_pad_left`` (``mp_tensors/reshapes.h:228-278``): m2 zeroed, then every
    (phys, left) stripe of m1 that m2's layout holds copied to its place in m2."""
    out = BlockMatrix()
    for key, blk in zip(m2.keys, m2.blocks):
        out.insert_block(np.zeros_like(blk), *key)
    in_left = ProductBasis(phys, in_left_i)
    out_left = ProductBasis(phys, out_left_i)
    for (lc, rc), blk in zip(m1.keys, m1.blocks):
        for s in range(len(phys)):
            pc, pd = phys[s]
            if not in_right_i.has(rc):
                continue
            r = in_right_i.position(rc)
            l_in = fuse(lc, neg(pc))
            if not in_left_i.has(l_in):
                continue
            l = in_left_i.position(l_in)
            ldim = in_left_i[l][1]
            if not out_left_i.has(l_in):
                continue
            k2 = out.find_block(lc, rc)
            if k2 == out.n_blocks():
                continue
            io, oo = in_left(pc, l_in), out_left(pc, l_in)
            nr = in_right_i[r][1]
            out.blocks[k2][oo:oo + pd * ldim, :nr] = blk[io:io + pd * ldim, :nr]
    return out


def site_ortho_boundaries(mps: MPSTensor, ortho: MPSTensor, o_left: BlockMatrix, o_right: BlockMatrix) -> MPSTensor:
    """``site_ortho_boundaries`` (``ct/abelian/special.hpp:16-43``): the state ``ortho``
    seen through the overlap boundaries of the sites around ``mps`` -- its
    projection onto the variational space of ``mps``, in ``mps``'s left-paired layout."""
    o = ortho.copy().make_right_paired()
    t = bm_gemm(o_left, o.data)
    t2 = reshape_right_to_left(mps.phys_i, o_left.left_basis(), o.right_i, t)
    t3 = bm_gemm(t2, o_right.transpose())
    m = mps.copy().make_left_paired()
    data = reshape_and_pad_left(mps.phys_i, o_left.left_basis(), o_right.left_basis(), m.left_i, t3, m.data)
    return MPSTensor(mps.phys_i, mps.left_i, mps.right_i, data, LEFT_PAIRED)


# --------------------------------------------------------------------------- two-site tensor
def two_site_theta(A: MPSTensor, B: MPSTensor) -> BlockMatrix:
    """``TwoSiteTensor(mps1, mps2)``: theta = A(lp) . B(rp) (``twositetensor.hpp:22-31``)."""
    A = A.copy().make_left_paired()
    B = B.copy().make_right_paired()
    return bm_gemm(A.data, B.data)


def _reshape_both_to_right(p1: Index, p2: Index, left_i: Index, right_i: Index, m1: BlockMatrix) -> BlockMatrix:
    """``ts_reshape::reshape_both_to_right`` (``mp_tensors/ts_reshape.h:231-290``)."""
    phys2 = index_product(p1, p2)
    phys_pb = ProductBasis(p1, p2)
    in_left = ProductBasis(p1, left_i)
    in_right = ProductBasis(p2, right_i, fuse_neg_first)
    out_right = ProductBasis(phys2, right_i, fuse_neg_first)
    m2 = BlockMatrix()
    for blk in range(m1.n_blocks()):
        for s1 in range(len(p1)):
            l = left_i.position(fuse(m1.left_charge(blk), neg(p1[s1][0])))
            if l == len(left_i):
                continue
            for s2 in range(len(p2)):
                r = right_i.position(fuse(m1.right_charge(blk), p2[s2][0]))
                if r == len(right_i):
                    continue
                s_charge = fuse(p1[s1][0], p2[s2][0])
                out_l = left_i[l][0]
                out_r = fuse(neg(s_charge), right_i[r][0])
                if not m2.has_block(out_l, out_r):
                    m2.insert_block(np.zeros((left_i[l][1], out_right.size(out_r))), out_l, out_r)
                ob = m2.blocks[m2.find_block(out_l, out_r)]
                ib = m1.blocks[blk]
                ilo = in_left(p1[s1][0], left_i[l][0])
                iro = in_right(p2[s2][0], right_i[r][0])
                oro = out_right(s_charge, right_i[r][0])
                opo = phys_pb(p1[s1][0], p2[s2][0])
                sd1, sd2, ld, rd = p1[s1][1], p2[s2][1], left_i[l][1], right_i[r][1]
                for ss1 in range(sd1):
                    for ss2 in range(sd2):
                        ss_out = opo + ss1 * sd2 + ss2
                        ob[:ld, oro + ss_out * rd: oro + (ss_out + 1) * rd] = \
                            ib[ilo + ss1 * ld: ilo + (ss1 + 1) * ld, iro + ss2 * rd: iro + (ss2 + 1) * rd]
    return m2


def _reshape_left_to_both(p1: Index, p2: Index, left_i: Index, right_i: Index, m1: BlockMatrix) -> BlockMatrix:
    """``ts_reshape::reshape_left_to_both`` (``mp_tensors/ts_reshape.h:89-145``)."""
    phys2 = index_product(p1, p2)
    phys_pb = ProductBasis(p1, p2)
    in_left = ProductBasis(phys2, left_i)
    out_right = ProductBasis(p2, right_i, fuse_neg_first)
    out_left = ProductBasis(p1, left_i)
    m2 = BlockMatrix()
    for blk in range(m1.n_blocks()):
        r = right_i.position(m1.right_charge(blk))
        if r == len(right_i):
            raise RuntimeError("m1 matrix inconsistent with right_i.")
        for s1 in range(len(p1)):
            for s2 in range(len(p2)):
                s_charge = fuse(p1[s1][0], p2[s2][0])
                l = left_i.position(fuse(m1.left_charge(blk), neg(s_charge)))
                if l == len(left_i):
                    continue
                out_l = fuse(p1[s1][0], left_i[l][0])
                out_r = fuse(neg(p2[s2][0]), right_i[r][0])
                o = m2.find_block(out_l, out_r)
                if o == m2.n_blocks():
                    o = m2.insert_block(np.zeros((out_left.size(out_l), out_right.size(out_r))), out_l, out_r)
                ob = m2.blocks[o]
                ib = m1.blocks[blk]
                ilo = in_left(s_charge, left_i[l][0])
                ipo = phys_pb(p1[s1][0], p2[s2][0])
                olo = out_left(p1[s1][0], left_i[l][0])
                oro = out_right(p2[s2][0], right_i[r][0])
                sd1, sd2, ld, rd = p1[s1][1], p2[s2][1], left_i[l][1], right_i[r][1]
                for ss1 in range(sd1):
                    for ss2 in range(sd2):
                        ss_in = ipo + ss1 * sd2 + ss2
                        ob[olo + ss1 * ld: olo + (ss1 + 1) * ld, oro + ss2 * rd: oro + (ss2 + 1) * rd] = \
                            ib[ilo + ss_in * ld: ilo + (ss_in + 1) * ld, :rd]
    return m2


def reduce_right(p1: Index, p2: Index, left_i: Index, right_i: Index, m1: BlockMatrix):
    """``ts_reduction::reduce_right`` (``mp_tensors/ts_reduction.h:42-141``)."""
    phys2 = index_product(p1, p2)
    phys_pb = ProductBasis(p1, p2)
    in_right = ProductBasis(phys2, right_i, fuse_neg_first)
    m2 = BlockMatrix()
    for blk in range(m1.n_blocks()):
        lc = m1.left_charge(blk)
        left_size = m1.blocks[blk].shape[0]
        in_r = m1.right_charge(blk)
        o = m2.insert_block(np.zeros(m1.blocks[blk].shape), lc, in_r)
        ib = m1.blocks[blk]
        ob = m2.blocks[o]
        for s in range(len(phys2)):
            s_charge = phys2[s][0]
            r = right_i.position(fuse(in_r, s_charge))
            if r == len(right_i):
                continue
            iro = in_right(s_charge, right_i[r][0])
            rs = right_i[r][1]
            for s1 in range(len(p1)):
                for s2 in range(len(p2)):
                    c1, c2 = p1[s1][0], p2[s2][0]
                    if s_charge != fuse(c1, c2):
                        continue
                    ipo = phys_pb(c1, c2)
                    S1, S2 = abs(spin(c1)), abs(spin(c2))
                    jl = spin(lc)
                    jm = spin(lc) + spin(c1)
                    jr = spin(right_i[r][0])
                    if jm < 0:
                        continue
                    if jl == jr and jl > 0 and S1 == 1 and S2 == 1:
                        base = ipo if spin(c1) == 1 else ipo - 1
                        for j in range(abs(S1 - S2), abs(S1 + S2) + 1, 2):
                            opo = base + j // 2
                            cc = math.sqrt((j + 1) * (jm + 1)) * wigner6j(jl, jr, j, S2, S1, jm)
                            if ((jl + jr + S1 + S2) // 2) % 2:
                                cc = -cc
                            _reduce_r(ob, ib, cc, iro, ipo, opo, p1[s1][1], p2[s2][1], left_size, rs)
                    else:
                        j = abs(spin(c1) + spin(c2))
                        cc = math.sqrt((j + 1) * (jm + 1)) * wigner6j(jl, jr, j, S2, S1, jm)
                        if ((jl + jr + S1 + S2) // 2) % 2:
                            cc = -cc
                        _reduce_r(ob, ib, cc, iro, ipo, ipo, p1[s1][1], p2[s2][1], left_size, rs)
    return phys2, m2


def _reduce_r(out, inp, scale, iro, ipo, opo, sd1, sd2, ld, rd):
    for ss1 in range(sd1):
        for ss2 in range(sd2):
            si = ipo + ss1 * sd2 + ss2
            so = opo + ss1 * sd2 + ss2
            out[:ld, iro + so * rd: iro + (so + 1) * rd] += scale * inp[:ld, iro + si * rd: iro + (si + 1) * rd]
            FLOPS.axpy(ld * rd)


def unreduce_left(p1: Index, p2: Index, left_i: Index, right_i: Index, m1: BlockMatrix):
    """``ts_reduction::unreduce_left`` (``mp_tensors/ts_reduction.h:143-251``)."""
    phys2 = index_product(p1, p2)
    phys_pb = ProductBasis(p1, p2)
    in_left = ProductBasis(phys2, left_i)
    m2 = BlockMatrix()
    for blk in range(m1.n_blocks()):
        rc = m1.right_charge(blk)
        right_size = m1.blocks[blk].shape[1]
        in_l = m1.left_charge(blk)
        o = m2.insert_block(np.zeros(m1.blocks[blk].shape), in_l, rc)
        ib = m1.blocks[blk]
        ob = m2.blocks[o]
        for s in range(len(phys2)):
            s_charge = phys2[s][0]
            l = left_i.position(fuse(in_l, neg(s_charge)))
            if l == len(left_i):
                continue
            ilo = in_left(s_charge, left_i[l][0])
            for s1 in range(len(p1)):
                for s2 in range(len(p2)):
                    c1, c2 = p1[s1][0], p2[s2][0]
                    if s_charge != fuse(c1, c2):
                        continue
                    ipo = phys_pb(c1, c2)
                    S1, S2 = abs(spin(c1)), abs(spin(c2))
                    jl = spin(left_i[l][0])
                    jr = spin(rc)
                    ld = left_i[l][1]
                    if jl == jr and jl > 0 and S1 == 1 and S2 == 1:
                        j = 0 if spin(c1) == 1 else 2
                        base = ipo if j == 0 else ipo - 1
                        for jm in (jl - 1, jl + 1):
                            opo = base + 1 if jm == jl - 1 else base
                            cc = math.sqrt((j + 1) * (jm + 1)) * wigner6j(jl, jr, j, S2, S1, jm)
                            if ((jl + jr + S1 + S2) // 2) % 2:
                                cc = -cc
                            _reduce_l(ob, ib, cc, ilo, ipo, opo, p1[s1][1], p2[s2][1], ld, right_size)
                    else:
                        j = abs(spin(c1) + spin(c2))
                        jm = jl + spin(c1)
                        if jm < 0:
                            continue
                        cc = math.sqrt((j + 1) * (jm + 1)) * wigner6j(jl, jr, j, S2, S1, jm)
                        if ((jl + jr + S1 + S2) // 2) % 2:
                            cc = -cc
                        _reduce_l(ob, ib, cc, ilo, ipo, ipo, p1[s1][1], p2[s2][1], ld, right_size)
    return phys2, m2


def _reduce_l(out, inp, scale, ilo, ipo, opo, sd1, sd2, ld, rd):
    for ss1 in range(sd1):
        for ss2 in range(sd2):
            si = ipo + ss1 * sd2 + ss2
            so = opo + ss1 * sd2 + ss2
            out[ilo + so * ld: ilo + (so + 1) * ld, :rd] += scale * inp[ilo + si * ld: ilo + (si + 1) * ld, :rd]
            FLOPS.axpy(ld * rd)


def make_two_site_mps(A: MPSTensor, B: MPSTensor) -> MPSTensor:
    """``SweepMPSContainer::getMPSTensor``: theta, both-paired -> right-paired, SU2-reduced
    (``twositetensor.hpp:132-139``)."""
    theta = two_site_theta(A, B)
    rp = _reshape_both_to_right(A.phys_i, B.phys_i, A.left_i, B.right_i, theta)
    phys2, red = reduce_right(A.phys_i, B.phys_i, A.left_i, B.right_i, rp)
    return MPSTensor.from_block(phys2, A.left_i, B.right_i, red, RIGHT_PAIRED)


# --------------------------------------------------------------------------- truncation
class TruncationResults:
    def __init__(self, bond_dimension, truncated_weight, truncated_fraction, smallest_ev):
        self.bond_dimension = bond_dimension
        self.truncated_weight = truncated_weight
        self.truncated_fraction = truncated_fraction
        self.smallest_ev = smallest_ev


def svd_truncate(M: BlockMatrix, rel_tol: float, Mmax: int):
    """``svd_truncate`` + ``estimate_truncation`` (``block_matrix_algorithms.h:163-333``).

    Keeps every singular value >= evalscut = max(cutoff*s0, s[Mmax]), so
    Mmax+1 values survive when there is no tie -- as in the reference.
    """
    U, S, V = BlockMatrix(), [], BlockMatrix()
    svals = []
    for (lc, rc), b in zip(M.keys, M.blocks):
        u, s, vt = np.linalg.svd(b, full_matrices=False)
        U.insert_block(u, lc, rc)
        V.insert_block(vt, rc, rc)
        svals.append(s)
    allevals = np.sort(np.concatenate(svals))[::-1]
    evalscut = rel_tol * allevals[0]
    if allevals.size > Mmax:
        evalscut = max(evalscut, allevals[Mmax])
    smallest_ev = evalscut / allevals[0]
    disc = allevals[allevals < evalscut]
    truncated_fraction = float(disc.sum() / allevals.sum())
    truncated_weight = float((disc * disc).sum() / (allevals * allevals).sum())
    # reference keeps the leading run of values >= evalscut (values are sorted descending per block)
    keeps = [int(np.argmax(s < evalscut)) if np.any(s < evalscut) else s.size for s in svals]
    Ut, Vt, St = BlockMatrix(), BlockMatrix(), []
    for k in range(len(svals)):
        kk = keeps[k]
        if kk == 0:
            continue
        lc, rc = U.keys[k]
        Ut.insert_block(U.blocks[k][:, :kk], lc, rc)
        Vt.insert_block(V.blocks[k][:kk, :], *V.keys[k])
        St.append((rc, svals[k][:kk]))
    bond_dimension = sum(keeps)
    return Ut, St, Vt, TruncationResults(bond_dimension, truncated_weight, truncated_fraction, smallest_ev)


def split_mps(tst_lp: BlockMatrix, p1, p2, left_i, right_i, Mmax, cutoff, l2r: bool):
    """``TwoSiteTensor::split_mps_l2r/r2l`` (``twositetensor.hpp:141-180``)."""
    both = _reshape_left_to_both(p1, p2, left_i, right_i, tst_lp)
    U, S, V, trunc = svd_truncate(both, cutoff, Mmax)
    sdict = {c: s for c, s in S}
    if l2r:
        A = MPSTensor.from_block(p1, left_i, U.right_basis(), U, LEFT_PAIRED)
        SV = BlockMatrix()
        for (lc, rc), b in zip(V.keys, V.blocks):
            SV.insert_block(sdict[lc][:, None] * b, lc, rc)
        Bt = MPSTensor.from_block(p2, SV.left_basis(), right_i, SV, RIGHT_PAIRED)
    else:
        Bt = MPSTensor.from_block(p2, V.left_basis(), right_i, V, RIGHT_PAIRED)
        US = BlockMatrix()
        for (lc, rc), b in zip(U.keys, U.blocks):
            US.insert_block(b * sdict[rc][None, :], lc, rc)
        A = MPSTensor.from_block(p1, left_i, US.right_basis(), US, LEFT_PAIRED)
    return A, Bt, trunc


def left_boundary_tensor_mpo(mps: MPSTensor, left: List[BlockMatrix], mpo) -> List[BlockMatrix]:
    """``left_boundary_tensor_mpo`` (``ct/common/move_boundary.hpp:66-97``): the left
    boundary x MPS x MPO contraction without the bra, one block matrix per right
    MPO bond.  The boundary product is trimmed to the ket's left index, every b2
    is computed and the output rows are phys x left (no restriction)."""
    mps = mps.copy()
    phys, left_i, right_i = mps.phys_i, mps.left_i, mps.right_i
    out_left_i = index_product(phys, left_i)
    mps.make_right_paired()
    T = boundary_mps_product(mps.data, left, mpo, left_i, True)
    out_left_pb = ProductBasis(phys, left_i)
    in_right_pb = ProductBasis(phys, right_i, fuse_neg_first)
    return [lbtm_kernel(b2, T, mpo, right_i, out_left_i, in_right_pb, out_left_pb) for b2 in range(mpo.col_dim)]


def right_boundary_tensor_mpo(mps: MPSTensor, right: List[BlockMatrix], mpo) -> List[BlockMatrix]:
    """``right_boundary_tensor_mpo`` (``ct/common/move_boundary.hpp:99-126``), one block
    matrix per left MPO bond.  ``MPSBoundaryProduct(mps, right, mpo)`` trims its
    products to the ket's *left* index (``boundary_times_mps.hpp:258-261``); the
    output columns are adjoin(phys) x right (no restriction)."""
    mps = mps.copy()
    phys, left_i, right_i = mps.phys_i, mps.left_i, mps.right_i
    mps.make_left_paired()
    t = mps_boundary_product(mps.data, right, mpo, left_i, True)
    out_right_i = index_product(adjoin(phys), right_i)
    in_left_pb = ProductBasis(phys, left_i)
    out_right_pb = ProductBasis(phys, right_i, fuse_neg_first)
    ret = []
    for b1 in range(mpo.row_dim):
        bufs = rbtm_tasks_apply(b1, t, mpo, left_i, out_right_i, in_left_pb, out_right_pb)
        blk = BlockMatrix()
        for key in bufs:
            blk.insert_block(bufs[key], *key)
        ret.append(blk)
    return ret


def heev_truncate(M: BlockMatrix, cutoff: float, Mmax: int):
    """``heev_truncate`` + ``estimate_truncation`` (``block_matrix_algorithms.h:188-200,
    211-251, 388-440``): per-block eigendecomposition, eigenvalues reordered
    descending with their vectors (``algorithms.hpp:402-421``), one global cut on
    the eigenvalues.  The result carries the truncated fraction in both weight
    fields, as the reference returns it (``block_matrix_algorithms.h:439``)."""
    U, evs = BlockMatrix(), []
    for (lc, rc), b in zip(M.keys, M.blocks):
        w, v = np.linalg.eigh(b)
        U.insert_block(v[:, ::-1].copy(), lc, rc)
        evs.append(w[::-1].copy())
    allevals = np.sort(np.concatenate(evs))[::-1]
    evalscut = cutoff * allevals[0]
    if allevals.size > Mmax:
        evalscut = max(evalscut, allevals[Mmax])
    smallest_ev = evalscut / allevals[0]
    disc = allevals[allevals < evalscut]
    truncated_fraction = float(disc.sum() / allevals.sum())
    keeps = [int(np.argmax(e < evalscut)) if np.any(e < evalscut) else e.size for e in evs]
    Ut, St = BlockMatrix(), []
    for k, kk in enumerate(keeps):
        if kk == 0:
            continue
        lc, rc = U.keys[k]
        Ut.insert_block(U.blocks[k][:, :kk].copy(), lc, rc)
        St.append((rc, evs[k][:kk]))
    return Ut, St, TruncationResults(sum(keeps), truncated_fraction, truncated_fraction, smallest_ev)


def predict_split_mps(tst_lp: BlockMatrix, p1, p2, left_i, right_i, Mmax, cutoff, l2r: bool,
                      alpha: float = 0.0, boundary=None, mpo=None, perturb: bool = True):
    """``TwoSiteTensor::predict_split_l2r/r2l`` (``twositetensor.hpp:184-297``).

    l2r: rho = theta theta^T (+ alpha sum_b h_b h_b^T, h = left_boundary_tensor_mpo of
    theta seen as one site with right index adjoin(p2) x right, ``boundary`` =
    left boundary of the pair, ``mpo`` = MPO tensor of the left site); the kept
    eigenvectors U give A = U and B = U^T theta.
    r2l: rho = theta^T theta (+ alpha sum_b h_b^T h_b from right_boundary_tensor_mpo
    with left index p1 x left, the right boundary and the right site's MPO
    tensor); B = U^T and A = theta U.  Only perturbation blocks whose charges
    theta holds are added (``twositetensor.hpp:207-221``)."""
    both = _reshape_left_to_both(p1, p2, left_i, right_i, tst_lp)
    bt = both.transpose()
    dm = bm_gemm(both, bt) if l2r else bm_gemm(bt, both)
    if perturb and boundary is not None:
        if l2r:
            tmp = MPSTensor.from_block(p1, left_i, index_product(adjoin(p2), right_i), both, LEFT_PAIRED)
            half = left_boundary_tensor_mpo(tmp, boundary, mpo)
        else:
            tmp = MPSTensor.from_block(p2, index_product(p1, left_i), right_i, both, RIGHT_PAIRED)
            half = right_boundary_tensor_mpo(tmp, boundary, mpo)
        for h in half:
            ht = h.transpose()
            tdm = bm_gemm(h, ht) if l2r else bm_gemm(ht, h)
            for (lc, rc), b in zip(tdm.keys, tdm.blocks):
                if both.find_block(lc, rc) == both.n_blocks():
                    continue
                p = dm.find_block(lc, rc)
                if p == dm.n_blocks():
                    dm.insert_block(alpha * b, lc, rc)
                else:
                    dm.blocks[p] = dm.blocks[p] + alpha * b
    U, S, trunc = heev_truncate(dm, cutoff, Mmax)
    if l2r:
        A = MPSTensor.from_block(p1, left_i, U.right_basis(), U, LEFT_PAIRED)
        V = bm_gemm(U.transpose(), both)
        Bt = MPSTensor.from_block(p2, V.left_basis(), right_i, V, RIGHT_PAIRED)
    else:
        Ut = U.transpose()
        Bt = MPSTensor.from_block(p2, Ut.left_basis(), right_i, Ut, RIGHT_PAIRED)
        V = bm_gemm(both, U)
        A = MPSTensor.from_block(p1, left_i, V.right_basis(), V, LEFT_PAIRED)
    return A, Bt, trunc


def predict_new_state(mps: MPSTensor, mpo, left, right, alpha: float, cutoff: float, Mmax: int, l2r: bool):
    """``predict_new_state_l2r_sweep`` / ``predict_new_state_r2l_sweep`` with the
    density-matrix perturbation (``ct/common/prediction.hpp:19-125``) and the zero-site
    factor of ``getZeroSiteTensorL2R/R2L`` (``prediction.hpp:62-73, 126-136``).

    l2r: rho = M M^T + alpha sum_b h_b h_b^T (M left-paired, h = left_boundary_tensor_mpo),
    the kept eigenvectors U are the new left-normalised site, the zero-site factor is
    U^T M.  r2l: rho = M^T M + alpha sum_b h_b^T h_b (M right-paired,
    h = right_boundary_tensor_mpo), the new site is U^T (right-paired), the factor M U.
    Returns (new site tensor, zero-site factor, truncation results)."""
    mps = mps.copy()
    if l2r:
        mps.make_left_paired()
    else:
        mps.make_right_paired()
    M = mps.data
    Mt = M.transpose()
    dm = bm_gemm(M, Mt) if l2r else bm_gemm(Mt, M)
    half = left_boundary_tensor_mpo(mps, left, mpo) if l2r else right_boundary_tensor_mpo(mps, right, mpo)
    for h in half:
        ht = h.transpose()
        tdm = bm_gemm(h, ht) if l2r else bm_gemm(ht, h)
        for (lc, rc), b in zip(tdm.keys, tdm.blocks):
            if M.find_block(lc, rc) == M.n_blocks():
                continue
            p = dm.find_block(lc, rc)
            if p == dm.n_blocks():
                dm.insert_block(alpha * b, lc, rc)
            else:
                dm.blocks[p] = dm.blocks[p] + alpha * b
    U, S, trunc = heev_truncate(dm, cutoff, Mmax)
    if l2r:
        new = MPSTensor.from_block(mps.phys_i, mps.left_i, U.right_basis(), U, LEFT_PAIRED)
        zero = bm_gemm(U.transpose(), M)
    else:
        Ut = U.transpose()
        new = MPSTensor.from_block(mps.phys_i, Ut.left_basis(), mps.right_i, Ut, RIGHT_PAIRED)
        zero = bm_gemm(M, U)
    return new, zero, trunc


# --------------------------------------------------------------------------- Jacobi-Davidson
def _project(t: MPSTensor, ortho: List[MPSTensor]) -> MPSTensor:
    """``SingleSiteVS::project`` (``fw/optimize/ietl_lanczos_solver.h:90-95``)."""
    for o in ortho:
        t.axpy(-o.dot(t) / o.dot(o), o)
    return t


def jcd_solve(apply_h, init: MPSTensor, tol: float, maxiter: int, ortho: Optional[List[MPSTensor]] = None,
              completeness: float = 1e-10):
    """``solve_ietl_jcd`` -> ``jacobi_davidson::calculate_eigenvalue`` with zero GMRES
    steps (``fw/optimize/ietl_jacobi_davidson.h:16-77``, ``ietl/jacobi.h:99-138, 361-493``).

    ``basic_iteration(maxiter, tol, tol)`` stops when ||r|| < tol or
    ||r|| < tol*|theta| (``alps/src/ietl/iteration.h``), or after maxiter steps.
    ``ortho``: vectors the solution is kept orthogonal to (excited states,
    ``ietl_jacobi_davidson.h:28-49``): Gram-Schmidt among themselves (a vector
    left with norm <= ``completeness`` is dropped), projected out of the start
    vector, of every new basis vector and of A u before the residual
    (``jacobi.h:378, 393, 432``).  If the start vector has nothing left after the
    projection the solve is skipped and <init|A init> returned with ``init``.
    Returns (theta, u, iterations).
    """
    kappa = 0.25
    local: List[MPSTensor] = []
    for o in list(ortho or [])[:max(init.data.num_elements() - 1, 0)]:
        v = o.copy().make_left_paired()
        for q in local:
            v.axpy(-q.dot(v), q)
        if v.norm() > completeness:
            local.append(v.scaled(1.0 / v.norm()))
    if local:
        tmp = init.copy().make_left_paired()
        for q in local:
            tmp.axpy(-tmp.dot(q), q)
        if tmp.norm() < completeness:
            x = init.copy().make_left_paired()
            return x.dot(apply_h(x)), x, 0
    V: List[MPSTensor] = []
    VA: List[MPSTensor] = []
    M = np.zeros((maxiter, maxiter))
    t = _project(init.copy().make_left_paired(), local)
    it = 0
    while True:
        tau = t.norm()
        for i in range(it):
            t.axpy(-V[i].dot(t), V[i])
        if t.norm() < kappa * tau:
            for i in range(it):
                t.axpy(-V[i].dot(t), V[i])
        _project(t, local)
        t = t.scaled(1.0 / t.norm())
        V.append(t)
        VA.append(apply_h(t))
        for i in range(it + 1):
            M[i, it] = V[i].dot(VA[it])
        n = it + 1
        Msym = np.triu(M[:n, :n]) + np.triu(M[:n, :n], 1).T
        w, z = np.linalg.eigh(Msym)
        theta = float(w[0])
        s = z[:, 0]
        u = V[0].scaled(s[0])
        for j in range(1, n):
            u.axpy(s[j], V[j])
        uA = VA[0].scaled(s[0])
        for j in range(1, n):
            uA.axpy(s[j], VA[j])
        _project(uA, local)
        r = uA.axpy(-theta, u)
        it += 1
        rn = r.norm()
        if rn <= tol * abs(theta) or rn < tol or it >= maxiter:
            return theta, u, it
        # t = -r + (r.u)/(u.u) u
        t = r.scaled(-1.0).axpy(r.dot(u) / u.dot(u), u)
