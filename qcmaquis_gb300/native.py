"""ctypes binding of ``libqcm_gb300.so`` (the C ABI declared in ``include/qcm_gb300.h``).

Loading fails loudly when the library is missing: the GPU path has no
fallback.  The flatteners turn host-side layouts (``Index``, block lists,
boundaries, ``MPOTensor``) into the plain arrays the ABI takes; the arrays
are kept alive on the returned objects.
"""
from __future__ import annotations

import ctypes as C
import os
from typing import List, Sequence

import numpy as np

from .symmetry import Index

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libqcm_gb300.so")

QCM_BUF_KET, QCM_BUF_LEFT, QCM_BUF_RIGHT, QCM_BUF_OUT, QCM_BUF_S0, QCM_BUF_S1, QCM_BUF_S2, QCM_BUF_IMG = range(8)
QCM_NBUF = 8
PREC_FP64, PREC_TF32, PREC_BF16X3, PREC_BF16X2 = 0, 1, 2, 3

i32p = C.POINTER(C.c_int32)
i64p = C.POINTER(C.c_int64)
f64p = C.POINTER(C.c_double)


class CIndex(C.Structure):
    _fields_ = [("n", C.c_int32), ("q", i32p), ("size", i64p)]


class CBlocks(C.Structure):
    _fields_ = [("n", C.c_int32), ("q", i32p), ("rows", i64p), ("cols", i64p), ("off", i64p)]


class CBoundary(C.Structure):
    _fields_ = [("aux", C.c_int32), ("blk_ptr", i32p), ("q", i32p), ("rows", i64p), ("cols", i64p), ("off", i64p)]


class CMpo(C.Structure):
    _fields_ = [("row_dim", C.c_int32), ("col_dim", C.c_int32),
                ("left_spin", i32p), ("right_spin", i32p), ("left_herm", i32p), ("right_herm", i32p),
                ("left_phase", i32p), ("right_phase", i32p),
                ("col_ptr", i32p), ("row_of", i32p), ("term_ptr", i32p), ("term_op", i32p), ("term_scale", f64p),
                ("n_ops", C.c_int32), ("op_spin", i32p), ("op_blk_ptr", i32p), ("blk_q", i32p),
                ("blk_ent_ptr", i32p), ("ent", i32p), ("ent_coeff", f64p), ("symmetry", C.c_int32)]


class CTagTable(C.Structure):
    _fields_ = [("n_tags", C.c_int32), ("fermionic", i32p), ("spin", i32p), ("herm_conj", i32p), ("pdiff", i32p),
                ("identity", C.c_int32), ("identity_full", C.c_int32), ("fill", C.c_int32), ("symmetry", C.c_int32)]


class CMpoSite(C.Structure):
    _fields_ = [("row_dim", C.c_int32), ("col_dim", C.c_int32), ("bond_dim", C.c_int32), ("n_elem", C.c_int32),
                ("elem_b1", i32p), ("elem_b2", i32p), ("elem_ptr", i32p), ("term_tag", i32p),
                ("term_scale", f64p), ("term_label", i32p), ("right_spin", i32p), ("right_herm", i32p),
                ("right_phase", i32p)]


class CChemTags(C.Structure):
    _fields_ = [("ident", C.c_int32), ("count", C.c_int32), ("docc", C.c_int32), ("bundles", (C.c_int32 * 6) * 9)]


class CTermView(C.Structure):
    _fields_ = [("n_terms", C.c_int64), ("term_ptr", i32p), ("pos", i32p), ("tag", i32p), ("coeff", f64p),
                ("fermionic", i32p), ("src_ptr", i64p), ("src_idx", i64p), ("src_val", f64p)]


# symmetry groups of qcm_mpo_t.symmetry and the MPS-level plans
SYM_SU2U1, SYM_TWOU1, SYM_U1 = 0, 1, 2


def symmetry_code(name: str) -> int:
    """QCM_SYM_* of a symmetry name ("su2u1", "2u1", "u1")."""
    codes = {"su2u1": SYM_SU2U1, "2u1": SYM_TWOU1, "u1": SYM_U1}
    if name not in codes:
        raise ValueError(f"unsupported symmetry {name!r}")
    return codes[name]


_lib = None


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"native library {LIB_PATH} is missing: run __graft_entry__.build() (no CPU fallback)")
    L = C.CDLL(LIB_PATH)
    L.qcm_last_error.restype = C.c_char_p
    L.qcm_version.restype = C.c_int
    for name in ("qcm_plan_sigma",):
        getattr(L, name).argtypes = [C.POINTER(CIndex)] * 3 + [C.POINTER(CBlocks), C.POINTER(CBoundary),
                                                               C.POINTER(CBoundary), C.POINTER(CMpo), C.c_int32,
                                                               C.POINTER(C.c_void_p)]
    for name in ("qcm_plan_boundary_left", "qcm_plan_boundary_right"):
        getattr(L, name).argtypes = [C.POINTER(CIndex)] * 3 + [C.POINTER(CBlocks), C.POINTER(CBoundary),
                                                               C.POINTER(CMpo), C.c_int32, C.POINTER(C.c_void_p)]
    L.qcm_plan_boundary_tensor_mpo.argtypes = [C.POINTER(CIndex)] * 3 + [C.POINTER(CBlocks), C.POINTER(CBoundary),
                                                                      C.POINTER(CMpo), C.c_int32, C.c_int32,
                                                                      C.POINTER(C.c_void_p)]
    L.qcm_plan_sigma_opts.argtypes = [C.POINTER(CIndex)] * 3 + [C.POINTER(CBlocks), C.POINTER(CBoundary),
                                                              C.POINTER(CBoundary), C.POINTER(CMpo), C.c_int32,
                                                              C.c_void_p, C.POINTER(C.c_void_p)]
    L.qcm_plan_diagonal.argtypes = [C.POINTER(CIndex)] * 3 + [C.POINTER(CBlocks), C.POINTER(CBoundary),
                                                            C.POINTER(CBoundary), C.POINTER(CMpo),
                                                            C.POINTER(C.c_void_p)]
    L.qcm_plan_zerosite.argtypes = [C.POINTER(CBlocks), C.POINTER(CBoundary), C.POINTER(CBoundary),
                                    C.POINTER(CMpo), C.POINTER(CMpo), C.c_int32, C.POINTER(C.c_void_p)]
    L.qcm_mpo_twosite_begin.argtypes = [C.POINTER(CMpo), C.POINTER(CMpo), C.POINTER(C.c_void_p), i32p]
    L.qcm_mpo_twosite_keys.argtypes = [C.c_void_p, i32p]
    L.qcm_mpo_twosite_finish.argtypes = [C.c_void_p, C.POINTER(CMpo)]
    L.qcm_mpo_buf_view.argtypes = [C.c_void_p, C.POINTER(CMpo), i64p]
    L.qcm_mpo_buf_term_pos.argtypes = [C.c_void_p, i32p]
    L.qcm_mpo_twosite.argtypes = [C.POINTER(CMpo), C.POINTER(CMpo), C.POINTER(CIndex), C.POINTER(CIndex),
                                  C.POINTER(C.c_void_p)]
    L.qcm_mpo_buf_destroy.argtypes = [C.c_void_p]
    L.qcm_mpo_buf_destroy.restype = None
    L.qcm_plan_block_gemm.argtypes = [C.POINTER(CBlocks), C.c_int32, C.POINTER(CBlocks), C.c_int32,
                                      C.POINTER(C.c_void_p)]
    L.qcm_plan_density_matrix.argtypes = [C.POINTER(CBlocks), C.c_int32, C.POINTER(CBoundary), C.c_double,
                                          C.POINTER(C.c_void_p)]
    L.qcm_chem_terms.argtypes = [C.c_int32, C.c_int32, C.c_int64, i32p, f64p, C.c_double, C.POINTER(CChemTags),
                                 C.POINTER(C.c_void_p)]
    L.qcm_term_buf_view.argtypes = [C.c_void_p, C.POINTER(CTermView)]
    L.qcm_term_buf_destroy.argtypes = [C.c_void_p]
    L.qcm_term_buf_destroy.restype = None
    L.qcm_mpo_maker_create.argtypes = [C.c_int32, C.POINTER(CTagTable), C.POINTER(C.c_void_p)]
    L.qcm_mpo_maker_add_terms.argtypes = [C.c_void_p, C.c_int32, i32p, i32p, i32p, f64p, i32p]
    L.qcm_mpo_maker_site_terms.argtypes = [C.c_void_p, C.c_int32, C.c_int32, i32p, f64p, i32p]
    L.qcm_mpo_maker_finish.argtypes = [C.c_void_p, C.POINTER(CTagTable), C.c_int32, C.c_int32]
    L.qcm_mpo_maker_site.argtypes = [C.c_void_p, C.c_int32, C.POINTER(CMpoSite)]
    L.qcm_mpo_maker_destroy.argtypes = [C.c_void_p]
    L.qcm_mpo_maker_destroy.restype = None
    L.qcm_plan_merge.argtypes = [C.POINTER(C.c_void_p), C.c_int32, i64p, C.POINTER(C.c_void_p)]
    L.qcm_plan_sizes.argtypes = [C.c_void_p, i64p, i64p]
    L.qcm_plan_image_bytes.argtypes = [C.c_void_p, i64p]
    L.qcm_plan_last_kernels.argtypes = [C.c_void_p, i32p]
    L.qcm_plan_stage_images.argtypes = [C.c_void_p, C.c_int32, i64p, i64p, i64p, i64p, f64p, i64p]
    L.qcm_plan_stage_image_aux.argtypes = [C.c_void_p, C.c_int32, i64p, i64p, i64p, C.POINTER(C.c_uint8)]
    L.qcm_plan_work.argtypes = [C.c_void_p, f64p, f64p, f64p, i32p]
    L.qcm_plan_out_layout.argtypes = [C.c_void_p, i32p, i32p, i32p, i32p, i64p, i64p, i64p]
    L.qcm_plan_num_stages.argtypes = [C.c_void_p, i32p]
    L.qcm_plan_stage_info.argtypes = [C.c_void_p, C.c_int32, i32p, i64p, i64p]
    L.qcm_plan_stage_axpy.argtypes = [C.c_void_p, C.c_int32, i64p, i64p, f64p]
    L.qcm_plan_stage_gemm.argtypes = [C.c_void_p, C.c_int32, i64p, i64p, f64p]
    L.qcm_plan_stage_dot.argtypes = [C.c_void_p, C.c_int32, i64p, i64p, f64p, i32p, i32p]
    L.qcm_plan_energy_gradient.argtypes = [C.POINTER(CIndex)] * 3 + [C.POINTER(CBlocks), C.POINTER(CBoundary),
                                                                  C.POINTER(CBoundary), C.POINTER(CMpo), C.c_int32,
                                                                  C.POINTER(C.c_void_p)]
    L.qcm_plan_upload.argtypes = [C.c_void_p]
    L.qcm_plan_run.argtypes = [C.c_void_p, C.POINTER(C.c_void_p), C.c_int32, C.c_void_p]
    L.qcm_plan_run_stages.argtypes = [C.c_void_p, C.POINTER(C.c_void_p), C.c_int32, C.c_void_p, C.c_int32,
                                      C.c_int32]
    L.qcm_plan_run_typed.argtypes = [C.c_void_p, C.POINTER(C.c_void_p), C.c_uint32, C.c_int32, C.c_void_p,
                                     C.c_int32, C.c_int32]
    L.qcm_plan_destroy.argtypes = [C.c_void_p]
    L.qcm_plan_destroy.restype = None
    L.qcm_dot.argtypes = [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    L.qcm_nrm2.argtypes = [C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    L.qcm_axpby.argtypes = [C.c_double, C.c_void_p, C.c_double, C.c_void_p, C.c_int64, C.c_void_p]
    L.qcm_lincomb.argtypes = [C.POINTER(C.c_void_p), f64p, C.c_int32, C.c_void_p, C.c_int64, C.c_void_p]
    L.qcm_multi_dot.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.c_void_p, C.c_int64, C.c_void_p, C.c_void_p]
    L.qcm_device_status.argtypes = [C.POINTER(C.c_int32)]
    L.qcm_multi_dot_noalloc.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.c_void_p, C.c_int64, C.c_void_p,
                                        C.c_void_p]
    L.qcm_seg_multi_dot.argtypes = [C.POINTER(C.c_void_p), C.c_int32, C.c_void_p, C.c_void_p, C.c_int32,
                                    C.c_void_p, C.c_void_p]
    L.qcm_plan_two_site.argtypes = [C.POINTER(CIndex)] * 3 + [C.POINTER(CBlocks)] + [C.POINTER(CIndex)] * 3 + \
        [C.POINTER(CBlocks), C.c_int32, C.POINTER(C.c_void_p)]
    L.qcm_plan_split_theta.argtypes = [C.POINTER(CIndex)] * 4 + [C.POINTER(CBlocks), C.c_int32,
                                                                  C.POINTER(C.c_void_p)]
    L.qcm_plan_split_assemble.argtypes = [C.c_void_p, i64p, i64p, i64p, f64p, i64p, C.c_int32,
                                          C.POINTER(C.c_void_p)]
    L.qcm_plan_out_tensor.argtypes = [C.c_void_p, C.c_int32, i32p, i32p, i64p, i64p, i64p, i32p, i32p, i64p]
    L.qcm_plan_mps_multiply.argtypes = [C.POINTER(CIndex)] * 3 + [C.POINTER(CBlocks)] * 2 + \
        [C.c_int32, C.POINTER(C.c_void_p)]
    L.qcm_plan_mps_reshape.argtypes = [C.POINTER(CIndex)] * 3 + [C.POINTER(CBlocks), C.c_int32,
                                                                  C.POINTER(C.c_void_p)]
    L.qcm_ctx_create.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
    L.qcm_ctx_set_stream.argtypes = [C.c_void_p, C.c_void_p]
    L.qcm_ctx_destroy.argtypes = [C.c_void_p]
    L.qcm_ctx_destroy.restype = None
    L.qcm_ctx_run.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64,
                              C.c_void_p, C.c_int32]
    L.qcm_boundary_step.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p,
                                    C.c_int32]
    L.qcm_jcd_solve.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p, C.c_int64, C.c_int32,
                                C.c_void_p, C.c_int64, C.c_double, C.c_int32, C.POINTER(C.c_void_p), C.c_int32,
                                C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_int32)]
    L.qcm_svd_create.argtypes = [C.c_int32, i64p, i64p, i64p, C.POINTER(C.c_void_p)]
    L.qcm_svd_sizes.argtypes = [C.c_void_p, i64p, i64p, i64p, i64p]
    L.qcm_svd_block_offsets.argtypes = [C.c_void_p, i64p, i64p, i64p]
    L.qcm_svd_run.argtypes = [C.c_void_p] + [C.c_void_p] * 6
    L.qcm_svd_last_sweeps.argtypes = [C.c_void_p, i32p]
    L.qcm_svd_set_panel_width.argtypes = [C.c_void_p, C.c_int32]
    L.qcm_svd_panel_width.argtypes = [C.c_void_p, i32p]
    L.qcm_svd_destroy.argtypes = [C.c_void_p]
    L.qcm_svd_destroy.restype = None
    L.qcm_truncation_cut.argtypes = [C.c_void_p, C.c_int32, i64p, C.c_int64, C.c_double, C.c_int32, i64p,
                                     C.POINTER(CTrunc), C.c_void_p]
    _lib = L
    return L


class Context:
    """Owner of a ``qcm_ctx`` (scratch, image buffer, FP32 boundary shadows and the
    eigensolver's vectors on one device and stream)."""

    def __init__(self, stream: int = 0):
        h = C.c_void_p()
        check(lib().qcm_ctx_create(C.c_void_p(stream) if stream else None, C.byref(h)), "qcm_ctx_create")
        self.h = h

    def set_stream(self, stream: int):
        check(lib().qcm_ctx_set_stream(self.h, C.c_void_p(stream) if stream else None), "qcm_ctx_set_stream")

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.qcm_ctx_destroy(self.h)
            self.h = None


class CTrunc(C.Structure):
    _fields_ = [("bond_dimension", C.c_int64), ("truncated_weight", C.c_double),
                ("truncated_fraction", C.c_double), ("smallest_ev", C.c_double), ("evalscut", C.c_double)]


class BatchedSVD:
    """FP64 SVD of a batch of independent blocks on the GPU (``qcm_svd_*``: one-sided
    Jacobi).  ``shapes`` = [(rows, cols)], ``offsets`` = element offsets of the
    column-major blocks in the source buffer.  ``run`` returns flat device arrays
    U, S, Vt packed block after block; ``u(k)``, ``s(k)``, ``vt(k)`` are views of block
    k (U: rows x k_k, S: k_k descending, Vt: k_k x cols)."""

    def __init__(self, shapes, offsets, panel_width=None):
        self.shapes = [(int(r), int(c)) for r, c in shapes]
        n = len(self.shapes)
        rows = np.array([r for r, _ in self.shapes] or [0], dtype=np.int64)
        cols = np.array([c for _, c in self.shapes] or [0], dtype=np.int64)
        offs = np.array(list(offsets) or [0], dtype=np.int64)
        h = C.c_void_p()
        check(lib().qcm_svd_create(n, _p(rows, i64p), _p(cols, i64p), _p(offs, i64p), C.byref(h)), "qcm_svd_create")
        self.h = h
        if panel_width is not None:
            check(lib().qcm_svd_set_panel_width(h, int(panel_width)), "qcm_svd_set_panel_width")
        w, u, sv, vt = C.c_int64(), C.c_int64(), C.c_int64(), C.c_int64()
        check(lib().qcm_svd_sizes(h, C.byref(w), C.byref(u), C.byref(sv), C.byref(vt)), "qcm_svd_sizes")
        self.sizes = (w.value, u.value, sv.value, vt.value)
        self.s_off = np.zeros(max(n, 1), dtype=np.int64)
        self.u_off = np.zeros(max(n, 1), dtype=np.int64)
        self.vt_off = np.zeros(max(n, 1), dtype=np.int64)
        check(lib().qcm_svd_block_offsets(h, _p(self.s_off, i64p), _p(self.u_off, i64p), _p(self.vt_off, i64p)),
              "qcm_svd_block_offsets")
        self.U = self.S = self.Vt = None

    def run(self, src, stream, work=None):
        import torch
        dev = src.device
        w, u, sv, vt = self.sizes
        work = torch.empty(max(w, 1), dtype=torch.float64, device=dev) if work is None else work
        self.U = torch.empty(max(u, 1), dtype=torch.float64, device=dev)
        self.S = torch.empty(max(sv, 1), dtype=torch.float64, device=dev)
        self.Vt = torch.empty(max(vt, 1), dtype=torch.float64, device=dev)
        check(lib().qcm_svd_run(self.h, C.c_void_p(src.data_ptr()), C.c_void_p(work.data_ptr()),
                                C.c_void_p(self.U.data_ptr()), C.c_void_p(self.S.data_ptr()),
                                C.c_void_p(self.Vt.data_ptr()), C.c_void_p(stream)), "qcm_svd_run")
        return self.U, self.S, self.Vt

    def k(self, i):
        r, c = self.shapes[i]
        return min(r, c)

    def u(self, i):
        r, c = self.shapes[i]
        k = min(r, c)
        o = int(self.u_off[i])
        return self.U[o:o + r * k].view(k, r).t()

    def s(self, i):
        o = int(self.s_off[i])
        return self.S[o:o + self.k(i)]

    def vt(self, i):
        r, c = self.shapes[i]
        k = min(r, c)
        o = int(self.vt_off[i])
        return self.Vt[o:o + k * c].view(c, k).t()

    def panel_width(self) -> int:
        """Columns per panel of the tournament rounds (0: single column pairs)."""
        bw = C.c_int32()
        check(lib().qcm_svd_panel_width(self.h, C.byref(bw)), "qcm_svd_panel_width")
        return bw.value

    def sweeps(self) -> int:
        n = C.c_int32()
        check(lib().qcm_svd_last_sweeps(self.h, C.byref(n)), "qcm_svd_last_sweeps")
        return n.value

    def cut(self, Mmax: int, cutoff: float, mode: int, stream):
        """The device truncation cut over this batch's values (see ``qcm_truncation_cut``);
        returns (keep per block, qcm_trunc_t)."""
        n = len(self.shapes)
        blk = np.zeros(n + 1, dtype=np.int64)
        for i in range(n):
            blk[i + 1] = blk[i] + self.k(i)
        keep = np.zeros(max(n, 1), dtype=np.int64)
        tr = CTrunc()
        check(lib().qcm_truncation_cut(C.c_void_p(self.S.data_ptr()), n, _p(blk, i64p), int(Mmax), float(cutoff),
                                       int(mode), _p(keep, i64p), C.byref(tr), C.c_void_p(stream)),
              "qcm_truncation_cut")
        return keep[:n], tr

    def __del__(self):
        try:
            if getattr(self, "h", None):
                lib().qcm_svd_destroy(self.h)
                self.h = None
        except Exception:
            pass


def check(rc: int, what: str = ""):
    if rc != 0:
        msg = lib().qcm_last_error().decode()
        raise RuntimeError(f"{what} failed ({rc}): {msg}")


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t)


# ------------------------------------------------------------------ flatteners
class FIndex:
    def __init__(self, idx: Index):
        n = len(idx)
        self.q = np.array([x for c, _ in idx for x in c], dtype=np.int32).reshape(-1)
        if self.q.size == 0:
            self.q = np.zeros(2, dtype=np.int32)
        self.size = np.array([s for _, s in idx] or [0], dtype=np.int64)
        self.c = CIndex(n, _p(self.q, i32p), _p(self.size, i64p))


class Layout:
    """Block list of one block-sparse tensor with sequential offsets."""

    def __init__(self, keys: Sequence, shapes: Sequence, offsets=None):
        self.keys = [tuple(k) for k in keys]
        self.shapes = [tuple(int(x) for x in s) for s in shapes]
        if offsets is None:
            offsets = []
            o = 0
            for r, c in self.shapes:
                offsets.append(o)
                o += r * c
        self.offsets = [int(o) for o in offsets]
        self.size = max([o + r * c for o, (r, c) in zip(self.offsets, self.shapes)] or [0])
        self._make_c()

    def _make_c(self):
        n = len(self.keys)
        self.q = np.array([[k[0][0], k[0][1], k[1][0], k[1][1]] for k in self.keys] or [[0, 0, 0, 0]],
                          dtype=np.int32).reshape(-1)
        self.rows = np.array([s[0] for s in self.shapes] or [0], dtype=np.int64)
        self.cols = np.array([s[1] for s in self.shapes] or [0], dtype=np.int64)
        self.off = np.array(self.offsets or [0], dtype=np.int64)
        self.c = CBlocks(n, _p(self.q, i32p), _p(self.rows, i64p), _p(self.cols, i64p), _p(self.off, i64p))

    @classmethod
    def of(cls, bm):
        return cls(bm.keys, [b.shape for b in bm.blocks])

    def pack(self, bm) -> np.ndarray:
        out = np.zeros(self.size)
        for k, o, (r, c) in zip(self.keys, self.offsets, self.shapes):
            p = bm.find_block(*k)
            if p < bm.n_blocks():
                out[o:o + r * c] = np.asarray(bm.blocks[p]).ravel(order="F")
        return out

    def unpack(self, flat: np.ndarray):
        from .block_matrix import BlockMatrix
        bm = BlockMatrix()
        for k, o, (r, c) in zip(self.keys, self.offsets, self.shapes):
            bm.keys.append(k)
            bm.blocks.append(np.asarray(flat[o:o + r * c]).reshape((r, c), order="F").copy())
        return bm


class BoundaryLayout:
    """One block list per MPO bond index, all in one arena."""

    def __init__(self, per_b: List[Layout] = None, *, blk_ptr=None, keys=None, shapes=None, offsets=None):
        if per_b is not None:
            keys, shapes, offsets, blk_ptr = [], [], [], [0]
            base = 0
            for lay in per_b:
                for k, s in zip(lay.keys, lay.shapes):
                    keys.append(k)
                    shapes.append(s)
                    offsets.append(base)
                    base += s[0] * s[1]
                blk_ptr.append(len(keys))
        self.keys = [tuple(k) for k in keys]
        self.shapes = [tuple(s) for s in shapes]
        self.offsets = list(offsets)
        self.blk_ptr = list(blk_ptr)
        self.aux = len(self.blk_ptr) - 1
        self.size = max([o + r * c for o, (r, c) in zip(self.offsets, self.shapes)] or [0])
        n = len(self.keys)
        self.q = np.array([[k[0][0], k[0][1], k[1][0], k[1][1]] for k in self.keys] or [[0, 0, 0, 0]],
                          dtype=np.int32).reshape(-1)
        self.rows = np.array([s[0] for s in self.shapes] or [0], dtype=np.int64)
        self.cols = np.array([s[1] for s in self.shapes] or [0], dtype=np.int64)
        self.off = np.array(self.offsets or [0], dtype=np.int64)
        self.ptr = np.array(self.blk_ptr, dtype=np.int32)
        self.c = CBoundary(self.aux, _p(self.ptr, i32p), _p(self.q, i32p), _p(self.rows, i64p),
                           _p(self.cols, i64p), _p(self.off, i64p))

    @classmethod
    def of(cls, boundary):
        return cls([Layout.of(bm) for bm in boundary])

    def pack(self, boundary) -> np.ndarray:
        out = np.zeros(self.size)
        for b in range(self.aux):
            bm = boundary[b]
            for k in range(self.blk_ptr[b], self.blk_ptr[b + 1]):
                key = self.keys[k]
                p = bm.find_block(*key)
                r, c = self.shapes[k]
                if p < bm.n_blocks():
                    out[self.offsets[k]:self.offsets[k] + r * c] = np.asarray(bm.blocks[p]).ravel(order="F")
        return out

    def unpack(self, flat: np.ndarray):
        from .block_matrix import BlockMatrix
        out = []
        for b in range(self.aux):
            bm = BlockMatrix()
            for k in range(self.blk_ptr[b], self.blk_ptr[b + 1]):
                r, c = self.shapes[k]
                o = self.offsets[k]
                bm.keys.append(self.keys[k])
                bm.blocks.append(np.asarray(flat[o:o + r * c]).reshape((r, c), order="F").copy())
            out.append(bm)
        return out


class FMpo:
    """Flattened MPOTensor (see ``qcm_mpo_t``)."""

    def __init__(self, mpo):
        self.mpo = mpo
        self.symmetry = symmetry_code(getattr(mpo, "symmetry", "su2u1"))
        self.left_spin = np.array([s.get() for s in mpo.left_spins], dtype=np.int32)
        self.right_spin = np.array([s.get() for s in mpo.right_spins], dtype=np.int32)
        self.left_herm = np.array(mpo.herm.LeftHerm, dtype=np.int32)
        self.right_herm = np.array(mpo.herm.RightHerm, dtype=np.int32)
        self.left_phase = np.array(mpo.herm.LeftPhase, dtype=np.int32)
        self.right_phase = np.array(mpo.herm.RightPhase, dtype=np.int32)
        col_ptr, row_of, term_ptr, term_op, term_scale = [0], [], [0], [], []
        # per flattened term: (b1, b2, position in the element list) and the model-term label
        self.term_key, self.term_label = [], []
        used_ops = {}
        labels_at = getattr(mpo, "labels_at", None)
        for b2 in range(mpo.col_dim):
            for b1 in mpo.column(b2):
                row_of.append(b1)
                labs = labels_at(b1, b2) if labels_at else [None] * len(mpo.at(b1, b2))
                for pos, ((tag, scale), lab) in enumerate(zip(mpo.at(b1, b2), labs)):
                    if tag not in used_ops:
                        used_ops[tag] = len(used_ops)
                    term_op.append(used_ops[tag])
                    term_scale.append(scale)
                    self.term_key.append((b1, b2, pos))
                    self.term_label.append(lab)
                term_ptr.append(len(term_op))
            col_ptr.append(len(row_of))
        op_spin, op_blk_ptr, blk_q, blk_ent_ptr, ent, ent_coeff = [], [0], [], [0], [], []
        self.op_tags = [tag for tag, _ in sorted(used_ops.items(), key=lambda kv: kv[1])]
        for tag, oid in sorted(used_ops.items(), key=lambda kv: kv[1]):
            op = mpo.op(tag)
            sp = mpo.sparse(tag)
            op_spin.append(op.spin.get())
            for (pin, pout), ents in zip(op.bm.keys, sp):
                blk_q += [pin[0], pin[1], pout[0], pout[1]]
                for (r, c, rs, cs, v) in ents:
                    ent += [r, c, rs, cs]
                    ent_coeff.append(v)
                blk_ent_ptr.append(len(ent_coeff))
            op_blk_ptr.append(len(blk_ent_ptr) - 1)
        a32 = lambda x: np.array(x or [0], dtype=np.int32)
        self.col_ptr = a32(col_ptr)
        self.row_of = a32(row_of)
        self.term_ptr = a32(term_ptr)
        self.term_op = a32(term_op)
        self.term_scale = np.array(term_scale or [0.0], dtype=np.float64)
        self.op_spin = a32(op_spin)
        self.op_blk_ptr = a32(op_blk_ptr)
        self.blk_q = a32(blk_q)
        self.blk_ent_ptr = a32(blk_ent_ptr)
        self.ent = a32(ent)
        self.ent_coeff = np.array(ent_coeff or [0.0], dtype=np.float64)
        self.n_ops = len(op_spin)
        self._make_c()

    def _make_c(self):
        mpo = self.mpo
        self.c = CMpo(mpo.row_dim, mpo.col_dim, _p(self.left_spin, i32p), _p(self.right_spin, i32p),
                      _p(self.left_herm, i32p), _p(self.right_herm, i32p), _p(self.left_phase, i32p),
                      _p(self.right_phase, i32p), _p(self.col_ptr, i32p), _p(self.row_of, i32p),
                      _p(self.term_ptr, i32p), _p(self.term_op, i32p), _p(self.term_scale, f64p),
                      self.n_ops, _p(self.op_spin, i32p), _p(self.op_blk_ptr, i32p), _p(self.blk_q, i32p),
                      _p(self.blk_ent_ptr, i32p), _p(self.ent, i32p), _p(self.ent_coeff, f64p), self.symmetry)

    @property
    def n_terms(self) -> int:
        return len(self.term_key)

    def with_scales(self, scales) -> "FMpo":
        """The same tensor with its term scales replaced (flattened term order)."""
        import copy
        f = copy.copy(self)
        f.term_scale = np.array(scales, dtype=np.float64).reshape(-1)
        if f.term_scale.size != max(self.n_terms, 1):
            raise ValueError("one scale per flattened term")
        f._make_c()
        return f


class _FlatTensor:
    """Shape of a tensor that exists only in flattened form."""

    def __init__(self, row_dim: int, col_dim: int):
        self.row_dim = row_dim
        self.col_dim = col_dim


def _copy(ptr, n, dtype):
    if n <= 0:
        return np.zeros(1, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


class FTagTable:
    """The operator table a term list names, as the native MPO maker reads it
    (``qcm_tag_table_t``): per tag fermionic, spin (2S, action), Hermitian
    conjugate and the particle-number change of its first block."""

    def __init__(self, th, identity: int, identity_full: int, fill: int, symmetry: str):
        from .symmetry import particle_number
        n = len(th.ops)
        self.ferm = np.array([1 if th.is_fermionic(t) else 0 for t in range(n)], dtype=np.int32)
        self.spin = np.array([(op.spin.get(), op.spin.action()) for op in th.ops], dtype=np.int32).reshape(-1)
        self.herm = np.array([th.herm_conj(t) for t in range(n)], dtype=np.int32)
        pd = []
        for op in th.ops:
            keys = op.bm.keys
            pd.append(particle_number(keys[0][0]) - particle_number(keys[0][1]) if keys else 0)
        self.pdiff = np.array(pd, dtype=np.int32)
        self.c = CTagTable(n, _p(self.ferm, i32p), _p(self.spin, i32p), _p(self.herm, i32p), _p(self.pdiff, i32p),
                           identity, identity_full, fill, symmetry_code(symmetry))


CHEM_BUNDLES = ("create", "destroy", "count", "flip", "e2d", "d2e", "docc", "create_count", "destroy_count")
CHEM_FIELDS = ("couple_up", "couple_down", "fill_couple_up", "fill_couple_down", "no_couple", "fill_no_couple")


class TermArrays:
    """Model terms as flat arrays (``qcm_chem_terms``): term t has operators
    (pos, tag)[term_ptr[t]:term_ptr[t+1]], coefficient coeff[t], fermionic[t], and
    per unit of integral keys[src_idx[s]] the coefficient src_val[s],
    s in [src_ptr[t], src_ptr[t+1])."""

    def __init__(self, term_ptr, pos, tag, coeff, fermionic, src_ptr, src_idx, src_val, keys):
        self.term_ptr, self.pos, self.tag, self.coeff = term_ptr, pos, tag, coeff
        self.fermionic, self.src_ptr, self.src_idx, self.src_val, self.keys = fermionic, src_ptr, src_idx, src_val, keys

    def __len__(self):
        return len(self.coeff)


def chem_terms(L_sites: int, nelec: int, integrals: dict, cutoff: float, ops, col) -> TermArrays:
    """The SU2U1 chemistry model's terms from its integral map (``qcm_chem_terms``):
    the same terms, coefficients and per-integral provenance as ``model.QCModel``'s
    Python generator, in the same order."""
    keys = list(integrals.keys())
    idx = np.array([list(k) for k in keys] or [[0, 0, 0, 0]], dtype=np.int32).reshape(-1)
    val = np.array([float(integrals[k]) for k in keys] or [0.0], dtype=np.float64)
    tags = CChemTags()
    tags.ident, tags.count, tags.docc = ops.ident, ops.count, ops.docc
    for b, name in enumerate(CHEM_BUNDLES):
        bundle = getattr(col, name)
        for f, field in enumerate(CHEM_FIELDS):
            x = getattr(bundle, field)
            tags.bundles[b][f] = -1 if x is None else int(x)
    L = lib()
    h = C.c_void_p()
    check(L.qcm_chem_terms(L_sites, nelec, len(keys), _p(idx, i32p), _p(val, f64p), float(cutoff), C.byref(tags),
                           C.byref(h)), "qcm_chem_terms")
    try:
        v = CTermView()
        check(L.qcm_term_buf_view(h, C.byref(v)), "qcm_term_buf_view")
        n = int(v.n_terms)
        ptr = _copy(v.term_ptr, n + 1, np.int32)[:n + 1]
        nops = int(ptr[-1])
        sptr = _copy(v.src_ptr, n + 1, np.int64)[:n + 1]
        ns = int(sptr[-1])
        return TermArrays(ptr, _copy(v.pos, nops, np.int32)[:nops], _copy(v.tag, nops, np.int32)[:nops],
                          _copy(v.coeff, n, np.float64)[:n], _copy(v.fermionic, n, np.int32)[:n], sptr,
                          _copy(v.src_idx, ns, np.int64)[:ns], _copy(v.src_val, ns, np.float64)[:ns], keys)
    finally:
        L.qcm_term_buf_destroy(h)


def mpo_maker_sites(L_sites: int, tags: FTagTable, terms, site_terms, leftmost_right: int, rightmost_left: int):
    """Single-site MPO tensors from the native maker (``qcm_mpo_maker_*``).

    ``terms`` = (term_ptr, pos, tag, coeff, label) arrays of the terms of two or
    more operators; ``site_terms`` = {site: [(tag, scale, label or None), ...]}.
    Returns per site (row_dim, col_dim, elem_b1, elem_b2, elem_ptr, term_tag,
    term_scale, term_label, right_spin (bond_dim x 2), right_herm, right_phase),
    the arrays as Python lists."""
    L = lib()
    h = C.c_void_p()
    check(L.qcm_mpo_maker_create(L_sites, C.byref(tags.c), C.byref(h)), "qcm_mpo_maker_create")
    try:
        ptr = np.ascontiguousarray(terms[0], dtype=np.int32)
        pos = np.ascontiguousarray(terms[1], dtype=np.int32)
        tag = np.ascontiguousarray(terms[2], dtype=np.int32)
        coeff = np.ascontiguousarray(terms[3], dtype=np.float64)
        label = np.ascontiguousarray(terms[4], dtype=np.int32)
        if len(coeff):
            check(L.qcm_mpo_maker_add_terms(h, len(coeff), _p(ptr, i32p), _p(pos, i32p), _p(tag, i32p),
                                            _p(coeff, f64p), _p(label, i32p)), "qcm_mpo_maker_add_terms")
        for site in sorted(site_terms):
            ents = site_terms[site]
            st = np.array([e[0] for e in ents], dtype=np.int32)
            ss = np.array([e[1] for e in ents], dtype=np.float64)
            sl = np.array([-1 if e[2] is None else e[2] for e in ents], dtype=np.int32)
            check(L.qcm_mpo_maker_site_terms(h, site, len(ents), _p(st, i32p), _p(ss, f64p), _p(sl, i32p)),
                  "qcm_mpo_maker_site_terms")
        check(L.qcm_mpo_maker_finish(h, C.byref(tags.c), leftmost_right, rightmost_left), "qcm_mpo_maker_finish")
        out = []
        for p in range(L_sites):
            v = CMpoSite()
            check(L.qcm_mpo_maker_site(h, p, C.byref(v)), "qcm_mpo_maker_site")
            ne, nb = v.n_elem, v.bond_dim
            eptr = _copy(v.elem_ptr, ne + 1, np.int32)
            nt = int(eptr[-1])
            out.append((v.row_dim, v.col_dim, _copy(v.elem_b1, ne, np.int32)[:ne].tolist(),
                        _copy(v.elem_b2, ne, np.int32)[:ne].tolist(), eptr.tolist(),
                        _copy(v.term_tag, nt, np.int32)[:nt].tolist(), _copy(v.term_scale, nt, np.float64)[:nt].tolist(),
                        _copy(v.term_label, nt, np.int32)[:nt].tolist(),
                        _copy(v.right_spin, 2 * nb, np.int32)[:2 * nb].reshape(-1, 2).tolist(),
                        _copy(v.right_herm, nb, np.int32)[:nb].tolist(), _copy(v.right_phase, nb, np.int32)[:nb].tolist()))
        return out
    finally:
        L.qcm_mpo_maker_destroy(h)


def make_twosite_fmpo(w1: FMpo, w2: FMpo, phys1: Index, phys2: Index = None, native_kron: bool = False) -> FMpo:
    """The flattened two-site MPO tensor of W1 (x) W2 (``make_twosite_mpo``,
    ``mp_tensors/ts_ops.h:78-152``) from the native builder.  The chain walk and
    the sums run in ``qcm_mpo_twosite_*``; the distinct spin-coupled Kronecker
    products are formed here by ``op_kron_su2`` (term for term the result then
    equals ``FMpo(make_twosite_mpo(...))``), or with ``native_kron`` in native
    code too (``qcm_mpo_twosite``: its Wigner symbols are long-double sums, so
    coefficients can differ from the exact-rational ones in the last bits)."""
    phys2 = phys1 if phys2 is None else phys2
    L = lib()
    h = C.c_void_p()
    if native_kron:
        f1, f2 = FIndex(phys1), FIndex(phys2)
        check(L.qcm_mpo_twosite(C.byref(w1.c), C.byref(w2.c), C.byref(f1.c), C.byref(f2.c), C.byref(h)),
              "qcm_mpo_twosite")
    else:
        _twosite_products(L, w1, w2, phys1, phys2, h)
    try:
        return _fmpo_from_buf(L, h)
    finally:
        L.qcm_mpo_buf_destroy(h)


def _twosite_products(L, w1: FMpo, w2: FMpo, phys1: Index, phys2: Index, h):
    """qcm_mpo_twosite_begin / _keys / _finish with the products formed by op_kron_su2."""
    from .site_operator import SpinDescriptor, op_kron_abelian, op_kron_su2
    nk = C.c_int32()
    check(L.qcm_mpo_twosite_begin(C.byref(w1.c), C.byref(w2.c), C.byref(h), C.byref(nk)), "qcm_mpo_twosite_begin")
    try:
        keys = np.zeros(max(6 * nk.value, 1), dtype=np.int32)
        check(L.qcm_mpo_twosite_keys(h, _p(keys, i32p)), "qcm_mpo_twosite_keys")
        op_spin, op_blk_ptr, blk_q, blk_ent_ptr, ent, ent_coeff = [], [0], [], [0], [], []
        for o1, o2, j, jpp, jp, sp in keys[:6 * nk.value].reshape(-1, 6).tolist():
            op1 = w1.mpo.op(w1.op_tags[o1])
            op2 = w2.mpo.op(w2.op_tags[o2])
            if w1.symmetry != SYM_SU2U1:
                prod = op_kron_abelian(phys1, phys2, op1, op2)
            else:
                prod = op_kron_su2(phys1, phys2, op1, op2, SpinDescriptor(j), SpinDescriptor(jpp),
                                   SpinDescriptor(jp), SpinDescriptor(sp, j, jp))
            prod.remove_empty_blocks()
            op_spin.append(sp)
            for (pin, pout), ents in zip(prod.bm.keys, prod.sparse()):
                blk_q += [pin[0], pin[1], pout[0], pout[1]]
                for (r, c, rs, cs, v) in ents:
                    ent += [r, c, rs, cs]
                    ent_coeff.append(v)
                blk_ent_ptr.append(len(ent_coeff))
            op_blk_ptr.append(len(blk_ent_ptr) - 1)
        a32 = lambda x: np.array(x or [0], dtype=np.int32)
        arrs = dict(op_spin=a32(op_spin), op_blk_ptr=a32(op_blk_ptr), blk_q=a32(blk_q),
                    blk_ent_ptr=a32(blk_ent_ptr), ent=a32(ent),
                    ent_coeff=np.array(ent_coeff or [0.0], dtype=np.float64))
        prods = CMpo()
        prods.n_ops = len(op_spin)
        for k in ("op_spin", "op_blk_ptr", "blk_q", "blk_ent_ptr", "ent"):
            setattr(prods, k, _p(arrs[k], i32p))
        prods.ent_coeff = _p(arrs["ent_coeff"], f64p)
        check(L.qcm_mpo_twosite_finish(h, C.byref(prods)), "qcm_mpo_twosite_finish")
    except Exception:
        L.qcm_mpo_buf_destroy(h)
        h.value = None
        raise


def _fmpo_from_buf(L, h) -> FMpo:
    """Copy a built two-site tensor out of its native buffer into an FMpo."""
    v = CMpo()
    sz = (C.c_int64 * 4)()
    check(L.qcm_mpo_buf_view(h, C.byref(v), sz), "qcm_mpo_buf_view")
    ne, nt, nb, nent = sz[0], sz[1], sz[2], sz[3]
    f = FMpo.__new__(FMpo)
    f.mpo = _FlatTensor(v.row_dim, v.col_dim)
    f.symmetry = int(v.symmetry)
    f.left_spin = _copy(v.left_spin, v.row_dim, np.int32)
    f.right_spin = _copy(v.right_spin, v.col_dim, np.int32)
    f.left_herm = _copy(v.left_herm, v.row_dim, np.int32)
    f.right_herm = _copy(v.right_herm, v.col_dim, np.int32)
    f.left_phase = _copy(v.left_phase, v.row_dim, np.int32)
    f.right_phase = _copy(v.right_phase, v.col_dim, np.int32)
    f.col_ptr = _copy(v.col_ptr, v.col_dim + 1, np.int32)
    f.row_of = _copy(v.row_of, ne, np.int32)
    f.term_ptr = _copy(v.term_ptr, ne + 1, np.int32)
    f.term_op = _copy(v.term_op, nt, np.int32)
    f.term_scale = _copy(v.term_scale, nt, np.float64)
    f.n_ops = v.n_ops
    f.op_spin = _copy(v.op_spin, nt, np.int32)
    f.op_blk_ptr = _copy(v.op_blk_ptr, nt + 1, np.int32)
    f.blk_q = _copy(v.blk_q, 4 * nb, np.int32)
    f.blk_ent_ptr = _copy(v.blk_ent_ptr, nb + 1, np.int32)
    f.ent = _copy(v.ent, 4 * nent, np.int32)
    f.ent_coeff = _copy(v.ent_coeff, nent, np.float64)
    pos = np.zeros(max(nt, 1), dtype=np.int32)
    check(L.qcm_mpo_buf_term_pos(h, _p(pos, i32p)), "qcm_mpo_buf_term_pos")
    b2 = np.repeat(np.arange(f.mpo.col_dim), np.diff(f.col_ptr[:f.mpo.col_dim + 1]))
    tb1 = np.repeat(f.row_of[:ne], np.diff(f.term_ptr[:ne + 1])) if ne else np.zeros(0, dtype=np.int32)
    tb2 = np.repeat(b2, np.diff(f.term_ptr[:ne + 1])) if ne else np.zeros(0, dtype=np.int64)
    f.term_key = list(zip(tb1.tolist(), tb2.tolist(), pos[:nt].tolist()))
    f.term_label = [None] * nt
    f.op_tags = list(range(nt))
    f._make_c()
    return f


def make_ts_cache_fmpo(mpo, phys: Index) -> List[FMpo]:
    """Flattened two-site MPO tensors of every site pair (``make_ts_cache_mpo``,
    ``mp_tensors/ts_ops.h:154-170``) from the native builder."""
    flat = [FMpo(w) for w in mpo]
    return [make_twosite_fmpo(flat[p], flat[p + 1], phys) for p in range(len(mpo) - 1)]


# ------------------------------------------------------------------ plans
class Plan:
    """Owner of a native plan handle."""

    def __init__(self, handle, kind: str):
        self.h = handle
        self.kind = kind
        out = C.c_int64()
        sc = (C.c_int64 * 3)()
        check(lib().qcm_plan_sizes(self.h, C.byref(out), sc), "qcm_plan_sizes")
        self.out_elems = out.value
        self.scratch = [sc[0], sc[1], sc[2]]
        ib = C.c_int64()
        check(lib().qcm_plan_image_bytes(self.h, C.byref(ib)), "qcm_plan_image_bytes")
        self.image_bytes = ib.value
        gf, af, ab, nl = C.c_double(), C.c_double(), C.c_double(), C.c_int32()
        check(lib().qcm_plan_work(self.h, C.byref(gf), C.byref(af), C.byref(ab), C.byref(nl)), "qcm_plan_work")
        self.gemm_flops, self.axpy_flops, self.axpy_bytes, self.launches = gf.value, af.value, ab.value, nl.value
        self.uploaded = False

    def __del__(self):
        if getattr(self, "h", None) and _lib is not None:
            _lib.qcm_plan_destroy(self.h)
            self.h = None

    def out_layout(self) -> BoundaryLayout:
        aux, nb = C.c_int32(), C.c_int32()
        check(lib().qcm_plan_out_layout(self.h, C.byref(aux), C.byref(nb), None, None, None, None, None),
              "qcm_plan_out_layout")
        n = max(nb.value, 1)
        ptr = np.zeros(aux.value + 1, dtype=np.int32)
        q = np.zeros(4 * n, dtype=np.int32)
        rows = np.zeros(n, dtype=np.int64)
        cols = np.zeros(n, dtype=np.int64)
        off = np.zeros(n, dtype=np.int64)
        check(lib().qcm_plan_out_layout(self.h, C.byref(aux), C.byref(nb), _p(ptr, i32p), _p(q, i32p),
                                        _p(rows, i64p), _p(cols, i64p), _p(off, i64p)), "qcm_plan_out_layout")
        nb = nb.value
        keys = [((int(q[4 * k]), int(q[4 * k + 1])), (int(q[4 * k + 2]), int(q[4 * k + 3]))) for k in range(nb)]
        shapes = [(int(rows[k]), int(cols[k])) for k in range(nb)]
        return BoundaryLayout(blk_ptr=list(ptr), keys=keys, shapes=shapes, offsets=[int(x) for x in off[:nb]])

    def stages(self):
        """Export the task tables (for host-side inspection and tests)."""
        n = C.c_int32()
        check(lib().qcm_plan_num_stages(self.h, C.byref(n)), "qcm_plan_num_stages")
        out = []
        for s in range(n.value):
            kind, no, nt = C.c_int32(), C.c_int64(), C.c_int64()
            check(lib().qcm_plan_stage_info(self.h, s, C.byref(kind), C.byref(no), C.byref(nt)), "stage_info")
            if kind.value == 0:
                od = np.zeros((max(no.value, 1), 7), dtype=np.int64)
                td = np.zeros((max(nt.value, 1), 3), dtype=np.int64)
                ta = np.zeros(max(nt.value, 1))
                check(lib().qcm_plan_stage_axpy(self.h, s, _p(od, i64p), _p(td, i64p), _p(ta, f64p)), "stage_axpy")
                out.append(("axpy", od[:no.value], td[:nt.value], ta[:nt.value]))
            elif kind.value == 1:
                od = np.zeros((max(no.value, 1), 7), dtype=np.int64)
                sd = np.zeros((max(nt.value, 1), 9), dtype=np.int64)
                sa = np.zeros(max(nt.value, 1))
                check(lib().qcm_plan_stage_gemm(self.h, s, _p(od, i64p), _p(sd, i64p), _p(sa, f64p)), "stage_gemm")
                out.append(("gemm", od[:no.value], sd[:nt.value], sa[:nt.value]))
            elif kind.value == 3:
                od = np.zeros((max(no.value, 1), 7), dtype=np.int64)
                td = np.zeros((max(nt.value, 1), 3), dtype=np.int64)
                w = np.zeros(max(nt.value, 1))
                tt = np.zeros(max(nt.value, 1), dtype=np.int32)
                meta = np.zeros(2, dtype=np.int32)
                check(lib().qcm_plan_stage_dot(self.h, s, _p(od, i64p), _p(td, i64p), _p(w, f64p), _p(tt, i32p),
                                               _p(meta, i32p)), "stage_dot")
                out.append(("dot", od[:no.value], td[:nt.value], w[:nt.value], tt[:nt.value], int(meta[0]),
                            int(meta[1])))
            else:
                out.append(("zero", int(no.value), int(nt.value)))
        return out

    def last_kernels(self) -> int:
        """Kernels the last run of this plan launched."""
        n = C.c_int32()
        check(lib().qcm_plan_last_kernels(self.h, C.byref(n)), "qcm_plan_last_kernels")
        return n.value

    def stage_images(self, stage: int):
        """Export the BF16x3 image-executor tables of a GEMM stage (host-side inspection and tests)."""
        cnt = np.zeros(4, dtype=np.int64)
        check(lib().qcm_plan_stage_images(self.h, stage, _p(cnt, i64p), None, None, None, None, None),
              "qcm_plan_stage_images")
        npn, no, ns, nu = [int(x) for x in cnt]
        pd = np.zeros((max(npn, 1), 8), dtype=np.int64)
        od = np.zeros((max(no, 1), 10), dtype=np.int64)
        sd = np.zeros((max(ns, 1), 8), dtype=np.int64)
        sa = np.zeros(max(ns, 1))
        td = np.zeros((max(nu, 1), 6), dtype=np.int64)
        check(lib().qcm_plan_stage_images(self.h, stage, _p(cnt, i64p), _p(pd, i64p), _p(od, i64p), _p(sd, i64p),
                                          _p(sa, f64p), _p(td, i64p)), "qcm_plan_stage_images")
        ac = np.zeros(3, dtype=np.int64)
        check(lib().qcm_plan_stage_image_aux(self.h, stage, _p(ac, i64p), None, None, None), "qcm_plan_stage_image_aux")
        gat = np.zeros(max(int(ac[0]), 1), dtype=np.int64)
        col = np.zeros(max(int(ac[1]), 1), dtype=np.int64)
        cim = np.zeros(max(int(ac[2]), 1), dtype=np.uint8)
        check(lib().qcm_plan_stage_image_aux(self.h, stage, _p(ac, i64p), _p(gat, i64p), _p(col, i64p),
                                             cim.ctypes.data_as(C.POINTER(C.c_uint8))), "qcm_plan_stage_image_aux")
        return {"panels": pd[:npn], "outs": od[:no], "segs": sd[:ns], "alpha": sa[:ns], "tiles": td[:nu],
                "gather": gat[:int(ac[0])], "coltab": col[:int(ac[1])], "cimg": cim[:int(ac[2])]}

    def upload(self):
        if not self.uploaded:
            check(lib().qcm_plan_upload(self.h), "qcm_plan_upload")
            self.uploaded = True

    def run(self, ptrs: Sequence[int], precision: int = PREC_FP64, stream: int = 0, first: int = 0,
            last: int = -1):
        arr = (C.c_void_p * QCM_NBUF)(*[C.c_void_p(int(p)) if p else None for p in ptrs])
        check(lib().qcm_plan_run_stages(self.h, arr, precision, C.c_void_p(stream) if stream else None, first, last),
              "qcm_plan_run_stages")

    def run_typed(self, ptrs: Sequence[int], f32mask: int, precision: int, stream: int = 0, first: int = 0,
                  last: int = -1):
        arr = (C.c_void_p * QCM_NBUF)(*[C.c_void_p(int(p)) if p else None for p in ptrs])
        check(lib().qcm_plan_run_typed(self.h, arr, f32mask, precision, C.c_void_p(stream) if stream else None,
                                       first, last), "qcm_plan_run_typed")

    def stage_kinds(self):
        n = C.c_int32()
        check(lib().qcm_plan_num_stages(self.h, C.byref(n)), "qcm_plan_num_stages")
        kinds = []
        for s in range(n.value):
            k, a, b = C.c_int32(), C.c_int64(), C.c_int64()
            check(lib().qcm_plan_stage_info(self.h, s, C.byref(k), C.byref(a), C.byref(b)), "stage_info")
            kinds.append(("axpy", "gemm", "zero")[k.value])
        return kinds


def out_tensor(plan: "Plan", which: int = 0):
    """Output tensor of an MPS-level plan (``qcm_plan_out_tensor``): (phys, left, right,
    Layout with the plan's offsets)."""
    nb = C.c_int32()
    n3 = (C.c_int32 * 3)()
    check(lib().qcm_plan_out_tensor(plan.h, which, C.byref(nb), None, None, None, None, n3, None, None),
          "qcm_plan_out_tensor")
    n = max(nb.value, 1)
    ni = max(n3[0] + n3[1] + n3[2], 1)
    q = np.zeros(4 * n, dtype=np.int32)
    rows, cols, off = (np.zeros(n, dtype=np.int64) for _ in range(3))
    iq = np.zeros(2 * ni, dtype=np.int32)
    isz = np.zeros(ni, dtype=np.int64)
    check(lib().qcm_plan_out_tensor(plan.h, which, C.byref(nb), _p(q, i32p), _p(rows, i64p), _p(cols, i64p),
                                    _p(off, i64p), n3, _p(iq, i32p), _p(isz, i64p)), "qcm_plan_out_tensor")
    nb = nb.value
    keys = [((int(q[4 * k]), int(q[4 * k + 1])), (int(q[4 * k + 2]), int(q[4 * k + 3]))) for k in range(nb)]
    shapes = [(int(rows[k]), int(cols[k])) for k in range(nb)]
    idx, base = [], 0
    for i in range(3):
        idx.append(Index.from_sorted([((int(iq[2 * (base + k)]), int(iq[2 * (base + k) + 1])), int(isz[base + k]))
                                      for k in range(n3[i])]))
        base += n3[i]
    return idx[0], idx[1], idx[2], Layout(keys, shapes, [int(x) for x in off[:nb]])


def plan_two_site(a_phys, a_left, a_right, a_lay: "Layout", b_phys, b_left, b_right, b_lay: "Layout",
                  symmetry: int = SYM_SU2U1) -> "Plan":
    """``qcm_plan_two_site``: the two-site tensor of sites (i, i+1) (SU(2)-reduced for
    SU2U1) from their left-paired tensors (slots KET = A, LEFT = B, OUT = the two-site
    tensor)."""
    f = [FIndex(x) for x in (a_phys, a_left, a_right, b_phys, b_left, b_right)]
    h = C.c_void_p()
    check(lib().qcm_plan_two_site(C.byref(f[0].c), C.byref(f[1].c), C.byref(f[2].c), C.byref(a_lay.c),
                                  C.byref(f[3].c), C.byref(f[4].c), C.byref(f[5].c), C.byref(b_lay.c),
                                  int(symmetry), C.byref(h)), "qcm_plan_two_site")
    return Plan(h, "theta")


def plan_split_theta(p1, p2, left_i, right_i, u_lay: "Layout", symmetry: int = SYM_SU2U1) -> "Plan":
    """``qcm_plan_split_theta``: the both-paired two-site tensor (slot OUT) from the
    left-paired one (slot KET)."""
    f = [FIndex(x) for x in (p1, p2, left_i, right_i)]
    h = C.c_void_p()
    check(lib().qcm_plan_split_theta(C.byref(f[0].c), C.byref(f[1].c), C.byref(f[2].c), C.byref(f[3].c),
                                     C.byref(u_lay.c), int(symmetry), C.byref(h)), "qcm_plan_split_theta")
    return Plan(h, "split")


def plan_split_assemble(split: "Plan", u_off, vt_off, keep, S_host, s_off, l2r: bool) -> "Plan":
    """``qcm_plan_split_assemble``: the two new site tensors of a truncated SVD split
    (slots KET = U, LEFT = Vt; OUT = site i left-paired, S2 = site i+1 left-paired)."""
    a = [np.ascontiguousarray(x, dtype=np.int64) for x in (u_off, vt_off, keep, s_off)]
    sv = np.ascontiguousarray(S_host, dtype=np.float64)
    h = C.c_void_p()
    check(lib().qcm_plan_split_assemble(split.h, _p(a[0], i64p), _p(a[1], i64p), _p(a[2], i64p), _p(sv, f64p),
                                        _p(a[3], i64p), 1 if l2r else 0, C.byref(h)), "qcm_plan_split_assemble")
    return Plan(h, "assemble")


def plan_mps_multiply(phys, left_i, right_i, t_lay: "Layout", n_lay: "Layout", from_left: bool) -> "Plan":
    """``qcm_plan_mps_multiply``: N . T (``from_left``, ``multiply_from_left``) or T . N
    (``multiply_from_right``) for the left-paired site tensor T (slot KET) and the
    block-diagonal bond factor N (slot LEFT); OUT = the new tensor, left-paired."""
    f = [FIndex(x) for x in (phys, left_i, right_i)]
    h = C.c_void_p()
    check(lib().qcm_plan_mps_multiply(C.byref(f[0].c), C.byref(f[1].c), C.byref(f[2].c), C.byref(t_lay.c),
                                      C.byref(n_lay.c), 1 if from_left else 0, C.byref(h)), "qcm_plan_mps_multiply")
    return Plan(h, "mps")


def plan_mps_reshape(phys, left_i, right_i, lay: "Layout", to_right: bool) -> "Plan":
    """``qcm_plan_mps_reshape``: a site tensor (slot KET) from left- to right-paired
    (``to_right``) or back (slot OUT)."""
    f = [FIndex(x) for x in (phys, left_i, right_i)]
    h = C.c_void_p()
    check(lib().qcm_plan_mps_reshape(C.byref(f[0].c), C.byref(f[1].c), C.byref(f[2].c), C.byref(lay.c),
                                     1 if to_right else 0, C.byref(h)), "qcm_plan_mps_reshape")
    return Plan(h, "mps")


def plan_block_gemm(a_lay: "Layout", ta: bool, b_lay: "Layout", tb: bool) -> "Plan":
    """``qcm_plan_block_gemm``: OUT = op(A) op(B), charge-matched (A in slot KET, B in
    slot LEFT); the output layout through ``out_tensor``."""
    h = C.c_void_p()
    check(lib().qcm_plan_block_gemm(C.byref(a_lay.c), 1 if ta else 0, C.byref(b_lay.c), 1 if tb else 0,
                                    C.byref(h)), "qcm_plan_block_gemm")
    return Plan(h, "mps")


def plan_density_matrix(theta: "Layout", l2r: bool, half: "BoundaryLayout" = None, alpha: float = 0.0) -> "Plan":
    """``qcm_plan_density_matrix``: rho = theta theta^T (``l2r``) or theta^T theta (theta
    in slot KET), plus alpha sum_b h_b h_b^T (h in slot RIGHT) when ``half`` is given."""
    h = C.c_void_p()
    hp = C.byref(half.c) if (half is not None and alpha != 0.0) else None
    check(lib().qcm_plan_density_matrix(C.byref(theta.c), 1 if l2r else 0, hp, float(alpha), C.byref(h)),
          "qcm_plan_density_matrix")
    return Plan(h, "mps")


class CPlanOpts(C.Structure):
    _fields_ = [("split_k_segs", C.c_int32), ("dense_min_terms", C.c_int32), ("n_tile_max", C.c_int32),
                ("k1_schedule", C.c_int32), ("reserved", C.c_int32 * 4)]


def plan_sigma(phys: Index, left_i: Index, right_i: Index, psi: Layout, L: BoundaryLayout, R: BoundaryLayout,
               mpo: FMpo, hermitian: bool = True, split_k_segs: int = 0, dense_min_terms: int = 0,
               n_tile_max: int = 0, k1_schedule: int = 0) -> Plan:
    """``qcm_plan_sigma`` (``qcm_plan_sigma_opts`` when a plan-shape option is given)."""
    fp, fl, fr = FIndex(phys), FIndex(left_i), FIndex(right_i)
    h = C.c_void_p()
    if split_k_segs or dense_min_terms or n_tile_max or k1_schedule:
        o = CPlanOpts(int(split_k_segs), int(dense_min_terms), int(n_tile_max), int(k1_schedule))
        check(lib().qcm_plan_sigma_opts(C.byref(fp.c), C.byref(fl.c), C.byref(fr.c), C.byref(psi.c), C.byref(L.c),
                                        C.byref(R.c), C.byref(mpo.c), 1 if hermitian else 0, C.byref(o),
                                        C.byref(h)), "qcm_plan_sigma_opts")
    else:
        check(lib().qcm_plan_sigma(C.byref(fp.c), C.byref(fl.c), C.byref(fr.c), C.byref(psi.c), C.byref(L.c),
                                   C.byref(R.c), C.byref(mpo.c), 1 if hermitian else 0, C.byref(h)),
              "qcm_plan_sigma")
    return Plan(h, "sigma")


def plan_boundary_left(phys, left_i, right_i, mps: Layout, L: BoundaryLayout, mpo: FMpo, hermitian=True) -> Plan:
    fp, fl, fr = FIndex(phys), FIndex(left_i), FIndex(right_i)
    h = C.c_void_p()
    check(lib().qcm_plan_boundary_left(C.byref(fp.c), C.byref(fl.c), C.byref(fr.c), C.byref(mps.c), C.byref(L.c),
                                       C.byref(mpo.c), 1 if hermitian else 0, C.byref(h)), "qcm_plan_boundary_left")
    return Plan(h, "bleft")


def plan_boundary_right(phys, left_i, right_i, mps: Layout, R: BoundaryLayout, mpo: FMpo, hermitian=True) -> Plan:
    fp, fl, fr = FIndex(phys), FIndex(left_i), FIndex(right_i)
    h = C.c_void_p()
    check(lib().qcm_plan_boundary_right(C.byref(fp.c), C.byref(fl.c), C.byref(fr.c), C.byref(mps.c), C.byref(R.c),
                                        C.byref(mpo.c), 1 if hermitian else 0, C.byref(h)), "qcm_plan_boundary_right")
    return Plan(h, "bright")


def plan_energy_gradient(phys: Index, left_i: Index, right_i: Index, psi: Layout, L: BoundaryLayout,
                         R: BoundaryLayout, mpo: FMpo, hermitian: bool = True) -> Plan:
    """Gradient of <psi|H_eff psi> with respect to every term scale of ``mpo`` (flattened
    term order of ``FMpo``); run in the FP64 form, output length = number of terms."""
    fp, fl, fr = FIndex(phys), FIndex(left_i), FIndex(right_i)
    h = C.c_void_p()
    check(lib().qcm_plan_energy_gradient(C.byref(fp.c), C.byref(fl.c), C.byref(fr.c), C.byref(psi.c), C.byref(L.c),
                                         C.byref(R.c), C.byref(mpo.c), 1 if hermitian else 0, C.byref(h)),
          "qcm_plan_energy_gradient")
    return Plan(h, "grad")


def plan_merge(plans, caller_offsets) -> Plan:
    """One plan for several sigma problems (``qcm_plan_merge``); ``caller_offsets`` is a
    sequence of (KET, LEFT, RIGHT, OUT) element offsets, one per plan."""
    n = len(plans)
    arr = (C.c_void_p * n)(*[p.h for p in plans])
    off = np.ascontiguousarray(np.array(caller_offsets, dtype=np.int64).reshape(n, 4))
    h = C.c_void_p()
    check(lib().qcm_plan_merge(arr, n, _p(off, i64p), C.byref(h)), "qcm_plan_merge")
    p = Plan(h, "sigma")
    p._parts = list(plans)
    return p


def plan_boundary_tensor_mpo(phys, left_i, right_i, mps: Layout, B: BoundaryLayout, mpo: FMpo, side: str,
                             hermitian=True) -> Plan:
    """``left_boundary_tensor_mpo`` (side "left") / ``right_boundary_tensor_mpo`` (side "right"):
    the plan's output is the bra-free boundary, layout through ``out_layout``."""
    if side not in ("left", "right"):
        raise ValueError("side must be 'left' or 'right'")
    fp, fl, fr = FIndex(phys), FIndex(left_i), FIndex(right_i)
    h = C.c_void_p()
    check(lib().qcm_plan_boundary_tensor_mpo(C.byref(fp.c), C.byref(fl.c), C.byref(fr.c), C.byref(mps.c),
                                             C.byref(B.c), C.byref(mpo.c), 0 if side == "left" else 1,
                                             1 if hermitian else 0, C.byref(h)), "qcm_plan_boundary_tensor_mpo")
    return Plan(h, "btm_" + side)


def plan_diagonal(phys: Index, left_i: Index, right_i: Index, psi: Layout, L: BoundaryLayout, R: BoundaryLayout,
                  mpo: FMpo) -> Plan:
    """``diagonal_hamiltonian``: the diagonal of H_eff in psi's layout (FP64; the
    boundaries must hold every bond index)."""
    fp, fl, fr = FIndex(phys), FIndex(left_i), FIndex(right_i)
    h = C.c_void_p()
    check(lib().qcm_plan_diagonal(C.byref(fp.c), C.byref(fl.c), C.byref(fr.c), C.byref(psi.c), C.byref(L.c),
                                  C.byref(R.c), C.byref(mpo.c), C.byref(h)), "qcm_plan_diagonal")
    return Plan(h, "diag")


def plan_zerosite(bond: Layout, L: BoundaryLayout, R: BoundaryLayout, mpo_left: FMpo, mpo_right: FMpo,
                  hermitian=True) -> Plan:
    """``zerosite_hamil2``: sigma = H_eff C for the bond matrix C (layout ``bond``), the
    boundaries L = L[i+1], R = R[i+1] of that bond and the MPO tensors W[i], W[i+1]."""
    h = C.c_void_p()
    check(lib().qcm_plan_zerosite(C.byref(bond.c), C.byref(L.c), C.byref(R.c), C.byref(mpo_left.c),
                                  C.byref(mpo_right.c), 1 if hermitian else 0, C.byref(h)), "qcm_plan_zerosite")
    return Plan(h, "sigma")


__all__ = ["lib", "check", "Layout", "BoundaryLayout", "FMpo", "FIndex", "Plan", "plan_sigma",
           "plan_boundary_left", "plan_boundary_right", "plan_boundary_tensor_mpo", "plan_energy_gradient",
           "plan_merge", "plan_zerosite", "plan_diagonal", "make_twosite_fmpo", "make_ts_cache_fmpo", "PREC_BF16X2", "PREC_FP64", "PREC_TF32", "PREC_BF16X3"]
