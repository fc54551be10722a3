"""Numpy restatement of QCMaquis's abelian (TwoU1) two-site DMRG step (oracle; tests only).

The abelian contraction engine (``ct/abelian/``, paths below
dmrg/framework/dmrg/mp_tensors/contractions/) differs from the SU(2) one in
``dmrg_ref`` only where the couplings enter: there are none.  Restated here:

* ``BoundaryMPSProduct`` / ``MPSBoundaryProduct`` with the abelian GEMMs: the
  Hermitian partner of a bond enters without any phase
  (``common/boundary_times_mps.hpp:44-51``);
* ``lbtm_kernel`` (``abelian/apply_op.hpp:23-138``): per MPO column b2 and
  term, the constant charge shifts of the operator and of T[b1], one output
  block per right sector, and ``lb_tensor_mpo`` axpys
  (``bm/detail/alps_detail.hpp:191-207``);
* ``rbtm_kernel`` (``abelian/apply_op.hpp:140-240``) with ``rb_tensor_mpo``
  (``alps_detail.hpp:209-224``);
* ``site_hamil2`` (``abelian/site_hamil.hpp:23-90``, lbtm form) and the
  boundary steps ``overlap_mpo_left_step`` / ``overlap_mpo_right_step``
  (``common/move_boundary.hpp:128-229``) with the plain block GEMM;
* the abelian ``TwoSiteTensor``: theta reshaped both -> right with the plain
  product physical index (``mt/twositetensor.hpp:22-31, 125-130``) and the
  split without the SU(2) unreduce step (``:352-366``, ``:141-180``).

Block layouts, reshapes, truncation and the eigensolver are shared with
``dmrg_ref`` (they do not depend on the group).
"""
from __future__ import annotations

from typing import List

import numpy as np

from . import dmrg_ref as R
from .qn import BlockMatrix, Index, ProductBasis, adjoin, bm_gemm, common_subset, fuse, fuse_neg_first, \
    index_product, neg


def boundary_mps_product(ket_rp: BlockMatrix, left: List[BlockMatrix], mpo, ref: Index,
                         is_hermitian=True) -> List[BlockMatrix]:
    """T[b1] = L[b1]^T . ket (or L[conj b1] . ket for a Hermitian-skipped b1, scale 1)."""
    out = []
    h = mpo.herm
    for b1 in range(len(left)):
        if h.left_skip(b1) and is_hermitian:
            out.append(R.gemm_trim_left(left[h.left_conj(b1)], ket_rp, ref))
        else:
            out.append(R.gemm_trim_left(left[b1].transpose(), ket_rp, ref))
    return out


def mps_boundary_product(ket_lp: BlockMatrix, right: List[BlockMatrix], mpo, ref: Index,
                         is_hermitian=True) -> List[BlockMatrix]:
    """t[b2] = ket . R[b2] (or ket . R[conj b2]^T, scale 1)."""
    out = []
    h = mpo.herm
    for b2 in range(len(right)):
        if h.right_skip(b2) and is_hermitian:
            out.append(R.gemm_trim_right(ket_lp, right[h.right_conj(b2)].transpose(), ref))
        else:
            out.append(R.gemm_trim_right(ket_lp, right[b2], ref))
    return out


def _delta(bm_keys_first) -> tuple:
    """Charge shift right - left of the first block of a block list."""
    lc, rc = bm_keys_first
    return fuse(rc, neg(lc))


def lbtm_kernel(b2, T: List[BlockMatrix], mpo, right_i: Index, out_left_i: Index,
                in_right_pb: ProductBasis, out_left_pb: ProductBasis) -> BlockMatrix:
    """contr[b2] = sum over b1 and the terms of W(b1,b2) of the operator applied to T[b1]."""
    ret = BlockMatrix()
    for b1 in mpo.column(b2):
        Tb = T[b1]
        if Tb.n_blocks() == 0:
            continue
        for tag, scale in mpo.at(b1, b2):
            W = mpo.op(tag)
            if W.bm.n_blocks() == 0:
                continue
            op_delta = _delta(W.bm.keys[0])
            t_delta = _delta(Tb.keys[0])
            total = fuse(op_delta, neg(t_delta))
            for out_r, r_size in right_i:
                out_l = fuse(out_r, total)
                if not out_left_i.has(out_l):
                    continue
                o = ret.find_block(out_l, out_r)
                if o == ret.n_blocks():
                    o = ret.insert_block(np.zeros((out_left_i.size_of_block(out_l), r_size)), out_l, out_r)
                ob = ret.blocks[o]
                for (phys_in, phys_out), wblock in zip(W.bm.keys, W.bm.blocks):
                    in_r = fuse(out_r, neg(phys_in))
                    in_l = fuse(in_r, neg(t_delta))
                    tb = Tb.find_block(in_l, in_r)
                    if tb == Tb.n_blocks():
                        continue
                    iro = in_right_pb(phys_in, out_r)
                    olo = out_left_pb(phys_out, in_l)
                    iblock = Tb.blocks[tb]
                    ld = iblock.shape[0]
                    for ss1 in range(wblock.shape[0]):
                        for ss2 in range(wblock.shape[1]):
                            alfa = wblock[ss1, ss2] * scale
                            ob[olo + ss2 * ld: olo + (ss2 + 1) * ld, :r_size] += \
                                alfa * iblock[:, iro + ss1 * r_size: iro + (ss1 + 1) * r_size]
                            R.FLOPS.axpy(ld * r_size)
    return ret


def rbtm_kernel(b1, t: List[BlockMatrix], mpo, left_i: Index, out_right_i: Index,
                in_left_pb: ProductBasis, out_right_pb: ProductBasis) -> BlockMatrix:
    """buf[b1] = sum over b2 and the terms of W(b1,b2) of the operator applied to t[b2]."""
    ret = BlockMatrix()
    for b2 in mpo.row(b1):
        Tb = t[b2]
        if Tb.n_blocks() == 0:
            continue
        for tag, scale in mpo.at(b1, b2):
            W = mpo.op(tag)
            if W.bm.n_blocks() == 0:
                continue
            op_delta = _delta(W.bm.keys[0])
            t_delta = _delta(Tb.keys[0])
            total = fuse(op_delta, neg(t_delta))
            for out_l, l_size in left_i:
                out_r = fuse(out_l, neg(total))
                if not out_right_i.has(out_r):
                    continue
                o = ret.find_block(out_l, out_r)
                if o == ret.n_blocks():
                    o = ret.insert_block(np.zeros((l_size, out_right_i.size_of_block(out_r))), out_l, out_r)
                ob = ret.blocks[o]
                for (phys_in, phys_out), wblock in zip(W.bm.keys, W.bm.blocks):
                    in_l = fuse(out_l, phys_in)
                    in_r = fuse(in_l, t_delta)
                    tb = Tb.find_block(in_l, in_r)
                    if tb == Tb.n_blocks():
                        continue
                    ilo = in_left_pb(phys_in, out_l)
                    oro = out_right_pb(phys_out, in_r)
                    iblock = Tb.blocks[tb]
                    rd = iblock.shape[1]
                    for ss1 in range(wblock.shape[0]):
                        for ss2 in range(wblock.shape[1]):
                            alfa = wblock[ss1, ss2] * scale
                            ob[:, oro + ss2 * rd: oro + (ss2 + 1) * rd] += \
                                alfa * iblock[ilo + ss1 * l_size: ilo + (ss1 + 1) * l_size, :rd]
                            R.FLOPS.axpy(l_size * rd)
    return ret


def _gemm_into(A: BlockMatrix, B: BlockMatrix) -> BlockMatrix:
    """Plain block GEMM (every matching charge pair, no spin filter)."""
    return bm_gemm(A, B)


def site_hamil2(ket: R.MPSTensor, left, right, mpo, is_hermitian=True) -> R.MPSTensor:
    """sigma = H_eff ket (bra = ket), left-paired."""
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
            tmp = _gemm_into(contr, right[h.right_conj(b2)].transpose())
        else:
            tmp = _gemm_into(contr, right[b2])
        for k in range(tmp.n_blocks()):
            out.match_and_add_block(tmp.blocks[k], *tmp.keys[k])
    return R.MPSTensor(phys, bra.left_i, bra.right_i, out, R.LEFT_PAIRED)


def overlap_mpo_left_step(bra: R.MPSTensor, ket: R.MPSTensor, left: List[BlockMatrix], mpo,
                          is_hermitian=True) -> List[BlockMatrix]:
    """L[i+1][b2] = contr[b2]^T . bra (left-paired); Hermitian-skipped b2 are empty."""
    bra = bra.copy()
    ket = ket.copy()
    bra.make_right_paired()
    bra_basis = bra.data.left_basis()
    ket.make_right_paired()
    T = boundary_mps_product(ket.data, left, mpo, bra_basis, is_hermitian)
    left_i = bra.left_i
    right_i = ket.right_i
    out_left_i = index_product(bra.phys_i, left_i)
    common_subset(out_left_i, bra.right_i.copy())
    out_left_pb = ProductBasis(bra.phys_i, left_i)
    in_right_pb = ProductBasis(ket.phys_i, right_i, fuse_neg_first)
    bra.make_left_paired()
    ret = []
    for b2 in range(mpo.col_dim):
        if mpo.herm.right_skip(b2) and is_hermitian:
            ret.append(BlockMatrix())
            continue
        contr = lbtm_kernel(b2, T, mpo, right_i, out_left_i, in_right_pb, out_left_pb)
        ret.append(_gemm_into(contr.transpose(), bra.data))
    return ret


def overlap_mpo_right_step(bra: R.MPSTensor, ket: R.MPSTensor, right: List[BlockMatrix], mpo,
                           is_hermitian=True) -> List[BlockMatrix]:
    """R[i][b1] = buf[b1] . bra(right-paired)^T; Hermitian-skipped b1 are empty."""
    bra = bra.copy()
    ket = ket.copy()
    phys = ket.phys_i
    right_i = bra.right_i
    left_i = ket.left_i
    out_right_i = index_product(adjoin(phys), right_i)
    bra.make_left_paired()
    ref = bra.data.right_basis()
    ket.make_left_paired()
    t = mps_boundary_product(ket.data, right, mpo, ref, is_hermitian)
    common_subset(out_right_i, bra.left_i.copy())
    in_left_pb = ProductBasis(phys, left_i)
    out_right_pb = ProductBasis(phys, right_i, fuse_neg_first)
    bra.make_right_paired()
    ret = []
    for b1 in range(mpo.row_dim):
        if mpo.herm.left_skip(b1) and is_hermitian:
            ret.append(BlockMatrix())
            continue
        buf = rbtm_kernel(b1, t, mpo, left_i, out_right_i, in_left_pb, out_right_pb)
        ret.append(_gemm_into(buf, bra.data.transpose()))
    return ret


def make_two_site_mps(A: R.MPSTensor, B: R.MPSTensor) -> R.MPSTensor:
    """theta = A(lp).B(rp), both-paired -> right-paired over phys_A x phys_B."""
    theta = R.two_site_theta(A, B)
    rp = R._reshape_both_to_right(A.phys_i, B.phys_i, A.left_i, B.right_i, theta)
    phys2 = index_product(A.phys_i, B.phys_i)
    return R.MPSTensor(phys2, A.left_i, B.right_i, rp, R.RIGHT_PAIRED)


def split_mps(u_lp: BlockMatrix, p1, p2, left_i, right_i, Mmax, cutoff, l2r: bool):
    """split_mps_l2r / r2l of the (unreduced) left-paired two-site tensor."""
    return R.split_mps(u_lp, p1, p2, left_i, right_i, Mmax, cutoff, l2r)


__all__ = ["boundary_mps_product", "mps_boundary_product", "lbtm_kernel", "rbtm_kernel", "site_hamil2",
           "overlap_mpo_left_step", "overlap_mpo_right_step", "make_two_site_mps", "split_mps"]
