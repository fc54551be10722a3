"""GPU-resident MPS tensor operations around the optimisation step.

Each tensor is one flat FP64 CUDA buffer plus a block layout; blocks are
column-major views into the buffer.  These operations restate:

* ``TwoSiteTensor(mps1, mps2)`` + ``make_mps`` (theta = A.B, both->right
  reshape, SU(2) ``reduce_right``): ``mp_tensors/twositetensor.hpp:22-31, 132-139``,
  ``mp_tensors/ts_reshape.h:231-290``, ``mp_tensors/ts_reduction.h:42-141`` --
  one native plan (``qcm_plan_two_site``);
* ``operator<<`` (``unreduce_left``) and ``reshape_left_to_both``:
  ``mp_tensors/twositetensor.hpp:372-389``, ``ts_reduction.h:143-251``,
  ``ts_reshape.h:89-145`` -- one native plan (``qcm_plan_split_theta``);
* ``split_mps_l2r/r2l`` with ``svd_truncate``: ``twositetensor.hpp:141-180``,
  ``block_matrix/block_matrix_algorithms.h:163-333``;
* ``leftNormalizeAndReturn`` / ``rightNormalizeAndReturn`` / ``multiply_from_*``:
  ``mp_tensors/mpstensor.hpp:219-330`` -- the batched SVD, the factor as one
  scaling of its output, and native plans for the reshapes and the product
  (``qcm_plan_mps_reshape``, ``qcm_plan_mps_multiply``).

Dense factorisations (SVD, density-matrix eigendecomposition, the QR/LQ of the
canonicalisation) run in the library's batched FP64 Jacobi SVD (``qcm_svd_*``)
and the truncation cut in its device cut (``qcm_truncation_cut``); the block
products of the density-matrix truncation (rho with its noise term, U^T theta,
theta U) in native grouped FP64 block products (``qcm_plan_density_matrix``,
``qcm_plan_block_gemm``).  Nothing here runs on the CPU except index bookkeeping.
"""
from __future__ import annotations

from typing import Dict, List, Optional, Tuple

import numpy as np
import torch

from . import native as N
from .engine import DeviceMPSTensor, _digest
from .symmetry import Index, ProductBasis, adjoin, common_subset, fuse, fuse_neg_first, index_product, neg


class DBM:
    """Block matrix on the device: sorted keys, per-block tensors (views allowed).
    ``layout`` / ``flat``: set when the blocks are views of one flat buffer in that
    layout (what the native plans read)."""

    def __init__(self):
        self.keys: List = []
        self.blocks: List[torch.Tensor] = []
        self.layout: Optional[N.Layout] = None
        self.flat: Optional[torch.Tensor] = None

    def find(self, lc, rc) -> int:
        k = (lc, rc)
        lo, hi = 0, len(self.keys)
        while lo < hi:
            mid = (lo + hi) // 2
            if self.keys[mid] > k:
                lo = mid + 1
            else:
                hi = mid
        return lo if lo < len(self.keys) and self.keys[lo] == k else len(self.keys)

    def insert(self, t: torch.Tensor, lc, rc) -> int:
        k = (lc, rc)
        lo, hi = 0, len(self.keys)
        while lo < hi:
            mid = (lo + hi) // 2
            if self.keys[mid] > k:
                lo = mid + 1
            else:
                hi = mid
        self.keys.insert(lo, k)
        self.blocks.insert(lo, t)
        return lo

    def get_or_zeros(self, lc, rc, shape, device):
        p = self.find(lc, rc)
        if p == len(self.keys):
            p = self.insert(torch.zeros(shape, dtype=torch.float64, device=device), lc, rc)
        return self.blocks[p]

    def left_lower_bound(self, lc) -> int:
        lo, hi = 0, len(self.keys)
        while lo < hi:
            mid = (lo + hi) // 2
            if self.keys[mid][0] > lc:
                lo = mid + 1
            else:
                hi = mid
        return lo

    def left_basis(self) -> Index:
        return Index.from_sorted([(k[0], b.shape[0]) for k, b in zip(self.keys, self.blocks)])

    def right_basis(self) -> Index:
        return Index.from_sorted([(k[1], b.shape[1]) for k, b in zip(self.keys, self.blocks)])

    def to_flat(self) -> Tuple[N.Layout, torch.Tensor]:
        lay = N.Layout(self.keys, [tuple(b.shape) for b in self.blocks])
        dev = self.blocks[0].device if self.blocks else torch.device("cuda")
        flat = torch.empty(max(lay.size, 1), dtype=torch.float64, device=dev)
        for o, b in zip(lay.offsets, self.blocks):
            r, c = b.shape
            flat[o:o + r * c].view(c, r).copy_(b.t())
        return lay, flat


def block_views(layout: N.Layout, flat: torch.Tensor) -> DBM:
    d = DBM()
    for k, o, (r, c) in zip(layout.keys, layout.offsets, layout.shapes):
        d.keys.append(k)
        d.blocks.append(flat[o:o + r * c].view(c, r).t())
    return d


def gemm(A: DBM, B: DBM, ta: bool = False, tb: bool = False) -> DBM:
    """Charge-matched block product op(A) op(B), op the transpose where asked
    (``block_matrix_algorithms.h:47-80``): one native grouped FP64 block product
    (``qcm_plan_block_gemm``).  The result's blocks are views of one flat buffer."""
    Af, Bf = _flat_of(A), _flat_of(B)
    dev = Af.flat.device
    key = ("gemm", bool(ta), bool(tb), _digest(Af.layout), _digest(Bf.layout))
    p = _RUNNER.plan(key, lambda: N.plan_block_gemm(Af.layout, ta, Bf.layout, tb))
    _, _, _, lay = N.out_tensor(p)
    out = torch.empty(max(p.out_elems, 1), dtype=torch.float64, device=dev)
    _run_fp64(p, dev, ket=Af.flat, left=Bf.flat, out=out)
    return _flat_dbm(lay, out)


def density_matrix(M: DBM, l2r: bool, half=None, alpha: float = 0.0) -> DBM:
    """rho = M M^T (``l2r``) or M^T M, plus alpha sum_b h_b h_b^T (or h_b^T h_b) over the
    blocks of ``half`` (the device boundary of ``left/right_boundary_tensor_mpo``)
    whose charges M holds (``twositetensor.hpp:195-221, 255-281``,
    ``ct/common/prediction.hpp:19-125``): one native grouped FP64 block product
    (``qcm_plan_density_matrix``)."""
    Mf = _flat_of(M)
    dev = Mf.flat.device
    noisy = half is not None and alpha != 0.0
    hl = half.layout if noisy else None
    key = ("dm", bool(l2r), _digest(Mf.layout), _digest(hl) if noisy else None, float(alpha) if noisy else 0.0)
    p = _RUNNER.plan(key, lambda: N.plan_density_matrix(Mf.layout, l2r, hl, alpha if noisy else 0.0))
    _, _, _, lay = N.out_tensor(p)
    out = torch.empty(max(p.out_elems, 1), dtype=torch.float64, device=dev)
    _run_fp64(p, dev, ket=Mf.flat, right=half.data if noisy else None, out=out)
    return _flat_dbm(lay, out)


# ------------------------------------------------------------------ reshapes
def reshape_l2r(phys: Index, left_i: Index, right_i: Index, m1: DBM) -> DBM:
    m2 = DBM()
    in_left = ProductBasis(phys, left_i)
    out_right = ProductBasis(phys, right_i, fuse_neg_first)
    for k, b in zip(m1.keys, m1.blocks):
        r = right_i.position(k[1])
        if r == len(right_i):
            continue
        in_r = right_i[r][0]
        for ps, sd in phys:
            l = left_i.position(fuse(k[0], neg(ps)))
            if l == len(left_i):
                continue
            ol, orr = left_i[l][0], fuse(neg(ps), in_r)
            ld, rd = left_i[l][1], right_i[r][1]
            ob = m2.get_or_zeros(ol, orr, (ld, out_right.size(orr)), b.device)
            ilo, oro = in_left(ps, ol), out_right(ps, in_r)
            for ss in range(sd):
                ob[:ld, oro + ss * rd:oro + (ss + 1) * rd] = b[ilo + ss * ld:ilo + (ss + 1) * ld, :rd]
    return m2


def reshape_r2l(phys: Index, left_i: Index, right_i: Index, m1: DBM) -> DBM:
    m2 = DBM()
    in_right = ProductBasis(phys, right_i, fuse_neg_first)
    out_left = ProductBasis(phys, left_i)
    for k, b in zip(m1.keys, m1.blocks):
        l = left_i.position(k[0])
        if l == len(left_i):
            continue
        in_l = left_i[l][0]
        for ps, sd in phys:
            r = right_i.position(fuse(k[1], ps))
            if r == len(right_i):
                continue
            ol, orr = fuse(ps, in_l), right_i[r][0]
            ld, rd = left_i[l][1], right_i[r][1]
            ob = m2.get_or_zeros(ol, orr, (out_left.size(ol), rd), b.device)
            iro, olo = in_right(ps, orr), out_left(ps, in_l)
            for ss in range(sd):
                ob[olo + ss * ld:olo + (ss + 1) * ld, :rd] = b[:ld, iro + ss * rd:iro + (ss + 1) * rd]
    return m2


# ------------------------------------------------------------------ MPS-level operations
def from_dbm(phys: Index, left_i: Index, right_i: Index, lp: DBM, layout_like=None) -> DeviceMPSTensor:
    lay, flat = lp.to_flat()
    return DeviceMPSTensor(phys, left_i, right_i, lay, flat)


def as_dbm(t: DeviceMPSTensor) -> DBM:
    return _flat_dbm(t.layout, t.data)


class _PlanRunner:
    """Plans of the MPS-level maps, cached by layout content, and their scratch."""

    def __init__(self, size: int = 16):
        self.plans: Dict = {}
        self.size = size
        self.ws: Dict = {}

    def plan(self, key, make):
        p = self.plans.get(key)
        if p is None:
            p = make()
            p.upload()
            while len(self.plans) >= self.size:
                self.plans.pop(next(iter(self.plans)))
            self.plans[key] = p
        else:
            self.plans[key] = self.plans.pop(key)
        return p

    def scratch(self, device, sizes):
        from .engine import Workspace
        w = self.ws.get(device)
        if w is None:
            w = self.ws[device] = Workspace(device)
        return w.get(list(sizes) + [1])[:3]


_RUNNER = _PlanRunner()


def _run_fp64(plan, device, ket=None, left=None, out=None, s2=None, right=None):
    s0, s1, s2w = _RUNNER.scratch(device, plan.scratch)
    ptr = lambda t: 0 if t is None else int(t.data_ptr())
    plan.run_typed([ptr(ket), ptr(left), ptr(right), ptr(out), ptr(s0), ptr(s1),
                    ptr(s2 if s2 is not None else s2w), 0], 0, N.PREC_FP64, _stream(device))


def make_two_site_mps(A: DeviceMPSTensor, B: DeviceMPSTensor, symmetry: int = N.SYM_SU2U1) -> DeviceMPSTensor:
    """``TwoSiteTensor(mps1, mps2)`` + ``make_mps``: theta = A(lp).B(rp), reshaped
    both->right, SU(2)-reduced (6j; not for TwoU1), returned left-paired -- one native
    plan (``qcm_plan_two_site``: the grouped block product and planned gather maps)."""
    from .engine import _digest
    key = ("theta", symmetry,
           _digest(A.phys_i, A.left_i, A.right_i, A.layout, B.phys_i, B.left_i, B.right_i, B.layout))
    plan = _RUNNER.plan(key, lambda: N.plan_two_site(A.phys_i, A.left_i, A.right_i, A.layout, B.phys_i, B.left_i,
                                                     B.right_i, B.layout, symmetry))
    phys2, left, right, lay = N.out_tensor(plan)
    out = torch.empty(max(plan.out_elems, 1), dtype=torch.float64, device=A.data.device)
    _run_fp64(plan, A.data.device, ket=A.data, left=B.data, out=out)
    return DeviceMPSTensor(phys2, left, right, lay, out)


def split_theta(u: DeviceMPSTensor, A0: DeviceMPSTensor, B0: DeviceMPSTensor, symmetry: int = N.SYM_SU2U1):
    """``tst << u`` followed by ``reshape_left_to_both``: the both-paired matrix of the
    two-site tensor (native plan ``qcm_plan_split_theta``: the 6j unreduce_left, SU2U1
    only, and the reshape as planned gather maps).  Returns (plan, layout, flat device
    buffer)."""
    from .engine import _digest
    key = ("split", symmetry, _digest(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, u.layout))
    plan = _RUNNER.plan(key, lambda: N.plan_split_theta(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, u.layout,
                                                        symmetry))
    _, _, _, lay = N.out_tensor(plan)
    out = torch.empty(max(plan.out_elems, 1), dtype=torch.float64, device=u.data.device)
    _run_fp64(plan, u.data.device, ket=u.data, out=out)
    return plan, lay, out


class Trunc:
    def __init__(self, bond_dimension, truncated_weight, truncated_fraction, smallest_ev):
        self.bond_dimension = bond_dimension
        self.truncated_weight = truncated_weight
        self.truncated_fraction = truncated_fraction
        self.smallest_ev = smallest_ev


def _stream(dev) -> int:
    return int(torch.cuda.current_stream(dev).cuda_stream)


def batched_svd(M: DBM):
    """FP64 SVD of every block of M in one batch on the GPU (``qcm_svd_*``, one-sided
    Jacobi, hand-written; replaces the per-block LAPACK gesvd/heevd/geqrf of the
    reference).  Returns the ``native.BatchedSVD`` with U, S (descending), Vt."""
    lay, flat = (M.layout, M.flat) if M.flat is not None else M.to_flat()
    svd = N.BatchedSVD(lay.shapes, lay.offsets)
    svd.run(flat, _stream(flat.device))
    return svd


def svd_truncate(M: DBM, rel_tol: float, Mmax: int):
    """``svd_truncate`` + ``estimate_truncation`` (``block_matrix_algorithms.h:210-333``):
    the batched device SVD of all blocks, then the global cut on the device
    (``qcm_truncation_cut``: keep every s >= max(cutoff s0, s[Mmax]); weight and
    fraction of the discarded values without multiplicity weighting)."""
    svd = batched_svd(M)
    keep, tr = svd.cut(Mmax, rel_tol, 0, _stream(svd.S.device))
    U, V = DBM(), DBM()
    S: Dict = {}
    for k, (key, kk) in enumerate(zip(M.keys, keep)):
        kk = int(kk)
        if kk == 0:
            continue
        lc, rc = key
        U.insert(svd.u(k)[:, :kk], lc, rc)
        V.insert(svd.vt(k)[:kk, :], rc, rc)
        S[rc] = svd.s(k)[:kk]
    return U, S, V, Trunc(int(tr.bond_dimension), tr.truncated_weight, tr.truncated_fraction, tr.smallest_ev)


def heev_truncate(dm: DBM, cutoff: float, Mmax: int):
    """``heev_truncate`` + ``estimate_truncation`` (``block_matrix_algorithms.h:188-200,
    211-251, 388-440``): the eigendecomposition of every (symmetric positive
    semi-definite) density-matrix block in one batch on the GPU -- its SVD, which
    gives the eigenpairs in descending order (``algorithms.hpp:402-421``) -- and the
    global cut on the eigenvalues on the device.  The truncated fraction is
    returned in both weight fields, as the reference does."""
    svd = batched_svd(dm)
    keep, tr = svd.cut(Mmax, cutoff, 1, _stream(svd.S.device))
    keys, shapes, offs = [], [], []
    S: Dict = {}
    for k, (key, kk) in enumerate(zip(dm.keys, keep)):
        kk = int(kk)
        if kk == 0:
            continue
        keys.append(key)
        shapes.append((dm.blocks[k].shape[0], kk))   # the first kk columns of U (ld = rows)
        offs.append(int(svd.u_off[k]))
        S[key[1]] = svd.s(k)[:kk]
    U = _flat_dbm(N.Layout(keys, shapes, offs), svd.U)
    return U, S, Trunc(int(tr.bond_dimension), tr.truncated_fraction, tr.truncated_fraction, tr.smallest_ev)


def _transpose(M: DBM) -> DBM:
    T = DBM()
    for (lc, rc), b in zip(M.keys, M.blocks):
        T.insert(b.t(), rc, lc)
    return T


def split(u: DeviceMPSTensor, A0: DeviceMPSTensor, B0: DeviceMPSTensor, Mmax: int, cutoff: float, l2r: bool,
          truncation: str = "svd", alpha: float = 0.0, engine=None, boundary=None, mpo=None,
          symmetry: int = N.SYM_SU2U1):
    """``tst << u`` then the truncation of ``SweepMPSUpdater`` (``sba/SweepMPSUpdater.h:186-203``):
    ``split_mps_l2r/r2l`` (``truncation="svd"``, the reference's default) or
    ``predict_split_l2r/r2l`` (``"heev"``, ``twositetensor.hpp:184-297``), whose
    density matrix carries the perturbation alpha sum_b h_b h_b^T when ``boundary``
    (left boundary of the pair going right, right boundary going left) and ``mpo``
    (the left / right site's MPO tensor) are given and alpha != 0.  (The
    reference computes the alpha = 0 perturbation and adds zeros; skipping it
    gives the same matrix.)  ``symmetry``: ``native.SYM_*`` of the tensors.  Returns new
    (A, B, truncation results)."""
    sp, blay, bflat = split_theta(u, A0, B0, symmetry)
    p1, p2 = A0.phys_i, B0.phys_i
    dev = u.data.device
    if truncation == "svd":
        # the whole split on the device: batched SVD, device cut, planned assembly
        svd = N.BatchedSVD(blay.shapes, blay.offsets)
        svd.run(bflat, _stream(dev))
        keep, tr = svd.cut(Mmax, cutoff, 0, _stream(dev))
        S_host = svd.S.cpu().numpy()
        ap = N.plan_split_assemble(sp, svd.u_off[:len(keep)], svd.vt_off[:len(keep)], keep, S_host,
                                   svd.s_off[:len(keep)], l2r)
        ap.upload()
        a_out = torch.empty(max(ap.out_elems, 1), dtype=torch.float64, device=dev)
        b_out = torch.empty(max(ap.scratch[2], 1), dtype=torch.float64, device=dev)
        _run_fp64(ap, dev, ket=svd.U, left=svd.Vt, out=a_out, s2=b_out)
        pa, la, ra, lay_a = N.out_tensor(ap, 0)
        pb, lb, rb, lay_b = N.out_tensor(ap, 1)
        return (DeviceMPSTensor(pa, la, ra, lay_a, a_out), DeviceMPSTensor(pb, lb, rb, lay_b, b_out),
                Trunc(int(tr.bond_dimension), tr.truncated_weight, tr.truncated_fraction, tr.smallest_ev))
    both = _flat_dbm(blay, bflat)
    if truncation in ("heev", "heev_truncation"):
        half = None
        if alpha != 0.0 and boundary is not None:
            if engine is None or mpo is None:
                raise ValueError("the heev perturbation needs the engine and the site's MPO tensor")
            if l2r:
                # theta as one site: phys p1, right index adjoin(p2) x right (from its blocks)
                t_right = both.right_basis()
                t_left = A0.left_i.copy()
                common_subset(t_left, index_product(adjoin(p1), t_right))
                tmp = from_dbm(p1, t_left, t_right, both)
                half = engine.boundary_tensor_mpo(tmp, boundary, mpo, "left")
            else:
                # theta as one site: phys p2, left index p1 x left (from its blocks)
                t_left = both.left_basis()
                t_right = B0.right_i.copy()
                common_subset(t_right, index_product(p2, t_left))
                tmp = from_dbm(p2, t_left, t_right, reshape_r2l(p2, t_left, t_right, both))
                half = engine.boundary_tensor_mpo(tmp, boundary, mpo, "right")
        dm = density_matrix(both, l2r, half, alpha)
        del half
        U, _, tr = heev_truncate(dm, cutoff, Mmax)
        del dm
        if l2r:
            A_lp = U
            B_rp = gemm(U, both, ta=True)
        else:
            B_rp = _transpose(U)
            A_lp = gemm(both, U)
    else:
        raise ValueError(f"unknown twosite_truncation {truncation!r} (svd or heev)")
    # A: MPSTensor(p1, left, A_lp.right_basis(), A_lp, LeftPaired)
    a_right = A_lp.right_basis()
    a_left = A0.left_i.copy()
    common_subset(a_left, index_product(adjoin(p1), a_right))
    A = from_dbm(p1, a_left, a_right, A_lp)
    # B: MPSTensor(p2, B_rp.left_basis(), right, B_rp, RightPaired)
    b_left = B_rp.left_basis()
    b_right = B0.right_i.copy()
    common_subset(b_right, index_product(p2, b_left))
    B = from_dbm(p2, b_left, b_right, reshape_r2l(p2, b_left, b_right, B_rp))
    return A, B, tr


def predict_new_state(u: DeviceMPSTensor, mpo, left, right, alpha: float, cutoff: float, Mmax: int, l2r: bool,
                      engine):
    """``predict_new_state_l2r_sweep`` / ``_r2l_sweep`` (``ct/common/prediction.hpp:19-125``)
    of a single-site tensor and the zero-site factor of ``getZeroSiteTensorL2R/R2L``:
    rho = M M^T (l2r, M left-paired) or M^T M (r2l, M right-paired) plus the noise term
    alpha sum_b h_b h_b^T from ``left/right_boundary_tensor_mpo``, the FP64
    eigendecomposition cut, the new site U (l2r) or U^T (r2l) and the factor U^T M
    (l2r) or M U (r2l).  Returns (new site, factor, truncation results)."""
    M = as_dbm(u) if l2r else reshape_l2r(u.phys_i, u.left_i, u.right_i, as_dbm(u))
    half = None
    if alpha != 0.0:
        half = engine.boundary_tensor_mpo(u, left if l2r else right, mpo, "left" if l2r else "right")
    dm = density_matrix(M, l2r, half, alpha)
    del half
    U, _, tr = heev_truncate(dm, cutoff, Mmax)
    del dm
    phys = u.phys_i
    if l2r:
        new_right = U.right_basis()
        new_left = u.left_i.copy()
        common_subset(new_left, index_product(adjoin(phys), new_right))
        return from_dbm(phys, new_left, new_right, U), gemm(U, M, ta=True), tr
    Ut = _transpose(U)
    new_left = Ut.left_basis()
    new_right = u.right_i.copy()
    common_subset(new_right, index_product(phys, new_left))
    return from_dbm(phys, new_left, new_right, reshape_r2l(phys, new_left, new_right, Ut)), gemm(M, U), tr


def _flat_dbm(layout: N.Layout, flat: torch.Tensor) -> DBM:
    """Block views of a flat buffer that keep the buffer and its layout."""
    d = block_views(layout, flat)
    d.layout, d.flat = layout, flat
    return d


def _scale_by_s(buf: torch.Tensor, S: torch.Tensor, shapes, offs, s_off, rows: bool) -> torch.Tensor:
    """The packed column-major blocks of ``buf`` with row t (``rows``: S Vt) or column t
    (U S) of block i scaled by S[s_off[i] + t], as one device operation."""
    idx = np.zeros(max(buf.numel(), 1), dtype=np.int64)
    for (r, c), o, so in zip(shapes, offs, s_off):
        idx[o:o + r * c] = so + (np.tile(np.arange(r), c) if rows else np.repeat(np.arange(c), r))
    return buf * S[torch.from_numpy(idx[:buf.numel()]).to(buf.device)]


def _run_mps_plan(key, make, device, ket, left=None) -> DeviceMPSTensor:
    p = _RUNNER.plan(key, make)
    phys, li, ri, lay = N.out_tensor(p)
    out = torch.empty(max(p.out_elems, 1), dtype=torch.float64, device=device)
    _run_fp64(p, device, ket=ket, left=left, out=out)
    return DeviceMPSTensor(phys, li, ri, lay, out[:lay.size])


def left_normalize_and_return(t: DeviceMPSTensor) -> Tuple[DeviceMPSTensor, DBM]:
    """``leftNormalizeAndReturn`` (``mp_tensors/mpstensor.hpp:219-236``): every left-paired
    block M = Q R with Q having orthonormal columns.  The factorisation is the batched
    device SVD, Q = U and R = S Vt: the same bond dimensions and the same product Q R
    as the reference's QR, in a different (orthogonal) gauge of the new bond, which no
    energy, overlap or truncation weight depends on.  Q is the SVD's U buffer itself
    (packed block after block in the tensor's block order) and R one scaling of Vt.
    The SVD runs single column pairs: the tall blocks of a site tensor measured slower
    in panels (a sweep at L=24, m=1024: 0.6 s)."""
    svd = N.BatchedSVD(t.layout.shapes, t.layout.offsets, panel_width=0)
    svd.run(t.data, _stream(t.data.device))
    n = len(t.layout.keys)
    ks = [min(r, c) for r, c in t.layout.shapes]
    q_lay = N.Layout(t.layout.keys, [(r, k) for (r, _), k in zip(t.layout.shapes, ks)])
    r_shapes = [(k, c) for (_, c), k in zip(t.layout.shapes, ks)]
    r_lay = N.Layout([(rc, rc) for _, rc in t.layout.keys], r_shapes)
    assert q_lay.offsets == [int(x) for x in svd.u_off[:n]] and r_lay.offsets == [int(x) for x in svd.vt_off[:n]]
    Rf = _scale_by_s(svd.Vt[:r_lay.size], svd.S, r_shapes, r_lay.offsets, svd.s_off[:n], rows=True)
    new_right = Index.from_sorted([(rc, k) for (_, rc), k in zip(t.layout.keys, ks)])
    return DeviceMPSTensor(t.phys_i, t.left_i, new_right, q_lay, svd.U[:q_lay.size]), _flat_dbm(r_lay, Rf)


def right_normalize_and_return(t: DeviceMPSTensor) -> Tuple[DeviceMPSTensor, DBM]:
    """``rightNormalizeAndReturn`` (``mp_tensors/mpstensor.hpp:239-258``): every
    right-paired block M = L Q with Q having orthonormal rows, from the batched device
    SVD (L = U S, Q = Vt; the gauge remark of ``left_normalize_and_return`` applies).
    The reshapes are native gather plans; L is one scaling of U."""
    dev = t.data.device
    rp = _run_mps_plan(("rs", 1, _digest(t.phys_i, t.left_i, t.right_i, t.layout)),
                       lambda: N.plan_mps_reshape(t.phys_i, t.left_i, t.right_i, t.layout, True), dev, t.data)
    svd = N.BatchedSVD(rp.layout.shapes, rp.layout.offsets, panel_width=0)
    svd.run(rp.data, _stream(dev))
    n = len(rp.layout.keys)
    ks = [min(r, c) for r, c in rp.layout.shapes]
    l_shapes = [(r, k) for (r, _), k in zip(rp.layout.shapes, ks)]
    l_lay = N.Layout([(lc, lc) for lc, _ in rp.layout.keys], l_shapes)
    q_lay = N.Layout(rp.layout.keys, [(k, c) for (_, c), k in zip(rp.layout.shapes, ks)])
    assert l_lay.offsets == [int(x) for x in svd.u_off[:n]] and q_lay.offsets == [int(x) for x in svd.vt_off[:n]]
    Lf = _scale_by_s(svd.U[:l_lay.size], svd.S, l_shapes, l_lay.offsets, svd.s_off[:n], rows=False)
    new_left = Index.from_sorted([(lc, k) for (lc, _), k in zip(rp.layout.keys, ks)])
    Q = _run_mps_plan(("rs", 0, _digest(t.phys_i, new_left, t.right_i, q_lay)),
                      lambda: N.plan_mps_reshape(t.phys_i, new_left, t.right_i, q_lay, False), dev,
                      svd.Vt[:q_lay.size])
    return Q, _flat_dbm(l_lay, Lf)


def _flat_of(Nm: DBM) -> DBM:
    """Nm itself when its blocks are still exactly the views of its flat buffer,
    else a packed copy."""
    if Nm.flat is not None and Nm.layout is not None and list(Nm.keys) == Nm.layout.keys:
        return Nm
    lay, flat = Nm.to_flat()
    return _flat_dbm(lay, flat)


def multiply_from_left(t: DeviceMPSTensor, Nm: DBM) -> DeviceMPSTensor:
    """``MPSTensor::multiply_from_left`` (``mp_tensors/mpstensor.hpp:314-321``): N . T
    over the left bond, one native plan (reshape, grouped block product, reshape)."""
    Nf = _flat_of(Nm)
    return _run_mps_plan(("mul", 1, _digest(t.phys_i, t.left_i, t.right_i, t.layout, Nf.layout)),
                         lambda: N.plan_mps_multiply(t.phys_i, t.left_i, t.right_i, t.layout, Nf.layout, True),
                         t.data.device, t.data, Nf.flat)


def multiply_from_right(t: DeviceMPSTensor, Nm: DBM) -> DeviceMPSTensor:
    """``MPSTensor::multiply_from_right`` (``mp_tensors/mpstensor.hpp:302-309``): T . N
    over the right bond, one grouped block product."""
    Nf = _flat_of(Nm)
    return _run_mps_plan(("mul", 0, _digest(t.phys_i, t.left_i, t.right_i, t.layout, Nf.layout)),
                         lambda: N.plan_mps_multiply(t.phys_i, t.left_i, t.right_i, t.layout, Nf.layout, False),
                         t.data.device, t.data, Nf.flat)


__all__ = ["DBM", "block_views", "make_two_site_mps", "split", "svd_truncate", "heev_truncate", "density_matrix", "gemm",
           "predict_new_state",
           "left_normalize_and_return", "right_normalize_and_return", "multiply_from_left", "multiply_from_right", "reshape_l2r", "reshape_r2l"]
