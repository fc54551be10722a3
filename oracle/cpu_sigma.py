"""The C++/OpenMP oracle sigma (``oracle/sigma_ref.cpp``) from Python (test
infrastructure and the timed CPU baseline; never used by the library).

``build()`` compiles ``oracle/_build/libsigma_ref.so`` with g++ -O3 -fopenmp.
Block products go to the host's OpenBLAS when one is found -- the copy numpy
ships (``numpy.libs/libscipy_openblas64_*``, ILP64 CBLAS, set to one thread so
that the oracle's own OpenMP loop over the MPO bonds owns the cores) -- and to
the oracle's own loop nest otherwise.

Inputs are plain arrays in the library's C-ABI layout structs; nothing here
loads the library itself.
"""
from __future__ import annotations

import ctypes as C
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "sigma_ref.cpp")
LIB = os.path.join(HERE, "_build", "libsigma_ref.so")

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
                ("blk_ent_ptr", i32p), ("ent", i32p), ("ent_coeff", f64p)]


MPO_ARRAYS = ("left_spin", "right_spin", "left_herm", "right_herm", "left_phase", "right_phase", "col_ptr", "row_of",
              "term_ptr", "term_op", "term_scale", "op_spin", "op_blk_ptr", "blk_q", "blk_ent_ptr", "ent",
              "ent_coeff")


def build(force: bool = False) -> str:
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        cmd = ["g++", "-std=c++17", "-O3", "-fopenmp", "-fPIC", "-shared", "-I" + os.path.join(ROOT, "include"), SRC,
               "-o", LIB]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("building the C++ oracle failed:\n" + r.stderr)
    return LIB


_lib = None
_blas = None


def lib():
    global _lib
    if _lib is None:
        L = C.CDLL(build())
        L.oracle_sigma.restype = C.c_int
        L.oracle_sigma.argtypes = [C.POINTER(CIndex)] * 3 + [C.POINTER(CBlocks), f64p, C.POINTER(CBoundary), f64p,
                                                             C.POINTER(CBoundary), f64p, C.POINTER(CMpo), C.c_int32,
                                                             f64p, f64p, C.c_void_p, C.c_int32, C.c_char_p,
                                                             C.c_int32]
        _lib = L
    return _lib


def host_blas():
    """(address of an ILP64 cblas_dgemm, description) of numpy's bundled OpenBLAS, set
    to one thread; (None, reason) when there is none."""
    global _blas
    if _blas is not None:
        return _blas
    import numpy
    libs = os.path.join(os.path.dirname(os.path.dirname(numpy.__file__)), "numpy.libs")
    for path in sorted(glob.glob(os.path.join(libs, "*openblas*.so*"))):
        try:
            h = C.CDLL(path)
        except OSError:
            continue
        for gemm, thr in (("scipy_cblas_dgemm64_", "scipy_openblas_set_num_threads64_"),
                          ("cblas_dgemm64_", "openblas_set_num_threads64_")):
            f = getattr(h, gemm, None)
            if f is None:
                continue
            t = getattr(h, thr, None)
            if t is not None:
                t.argtypes = [C.c_int]
                t(1)
            _blas = (C.cast(f, C.c_void_p).value, f"{os.path.basename(path)} {gemm} (one thread per OpenMP worker)")
            return _blas
    _blas = (None, "no host BLAS found: the oracle's own loop nest")
    return _blas


def _idx(index):
    q = np.array([x for c, _ in index for x in c] or [0], dtype=np.int32)
    s = np.array([sz for _, sz in index] or [0], dtype=np.int64)
    return CIndex(len(index), q.ctypes.data_as(i32p), s.ctypes.data_as(i64p)), (q, s)


class SigmaInputs:
    """Flat arrays of one sigma problem: indices, ket layout, boundary layouts, MPO."""

    def __init__(self, arrays: dict):
        self.a = {k: np.ascontiguousarray(v) for k, v in arrays.items()}
        a = self.a
        keep = []
        self.phys, k1 = self._index("phys")
        self.left, k2 = self._index("left")
        self.right, k3 = self._index("right")
        keep += [k1, k2, k3]
        self.psi = CBlocks(len(a["psi.rows"]), a["psi.q"].ctypes.data_as(i32p), a["psi.rows"].ctypes.data_as(i64p),
                           a["psi.cols"].ctypes.data_as(i64p), a["psi.off"].ctypes.data_as(i64p))
        self.L = self._boundary("L")
        self.R = self._boundary("R")
        d = a["W.dims"]
        self.W = CMpo(int(d[0]), int(d[1]), *[a["W." + k].ctypes.data_as(f64p if k in ("term_scale", "ent_coeff")
                                                                            else i32p) for k in MPO_ARRAYS[:11]],
                      int(d[2]), *[a["W." + k].ctypes.data_as(f64p if k == "ent_coeff" else i32p)
                                   for k in MPO_ARRAYS[11:]])
        self._keep = keep
        self.psi_size = int(max((o + r * c for o, r, c in zip(a["psi.off"], a["psi.rows"], a["psi.cols"])),
                                default=0))
        self.L_size = self._size("L")
        self.R_size = self._size("R")

    def _index(self, k):
        q, s = self.a[k + ".q"].astype(np.int32), self.a[k + ".size"].astype(np.int64)
        self.a[k + ".q"], self.a[k + ".size"] = q, s
        return CIndex(len(s), q.ctypes.data_as(i32p), s.ctypes.data_as(i64p)), (q, s)

    def _boundary(self, k):
        a = self.a
        return CBoundary(len(a[k + ".blk_ptr"]) - 1, a[k + ".blk_ptr"].ctypes.data_as(i32p),
                         a[k + ".q"].ctypes.data_as(i32p), a[k + ".rows"].ctypes.data_as(i64p),
                         a[k + ".cols"].ctypes.data_as(i64p), a[k + ".off"].ctypes.data_as(i64p))

    def _size(self, k):
        a = self.a
        return int(max((o + r * c for o, r, c in zip(a[k + ".off"], a[k + ".rows"], a[k + ".cols"])), default=0))


def sigma(inp: SigmaInputs, psi: np.ndarray, Ldata: np.ndarray, Rdata: np.ndarray, hermitian: bool = True,
          threads: int = 0, use_blas: bool = True):
    """sigma in the ket's layout and the work counters (gemm FLOPs, axpy FLOPs, threads)."""
    out = np.zeros(max(inp.psi_size, 1))
    work = np.zeros(3)
    err = C.create_string_buffer(512)
    gemm = host_blas()[0] if use_blas else None
    psi = np.ascontiguousarray(psi, dtype=np.float64)
    Ldata = np.ascontiguousarray(Ldata, dtype=np.float64)
    Rdata = np.ascontiguousarray(Rdata, dtype=np.float64)
    rc = lib().oracle_sigma(C.byref(inp.phys), C.byref(inp.left), C.byref(inp.right), C.byref(inp.psi),
                            psi.ctypes.data_as(f64p), C.byref(inp.L), Ldata.ctypes.data_as(f64p), C.byref(inp.R),
                            Rdata.ctypes.data_as(f64p), C.byref(inp.W), 1 if hermitian else 0,
                            out.ctypes.data_as(f64p), work.ctypes.data_as(f64p), C.c_void_p(gemm) if gemm else None,
                            int(threads), err, 512)
    if rc != 0:
        raise RuntimeError("oracle_sigma: " + err.value.decode())
    return out[:inp.psi_size], work


def flatten_mpo(mpo, prefix: str = "W.") -> dict:
    """An MPO tensor (any object with the reference's MPOTensor members: row/col_dim,
    column, at, op, left/right_spin, herm) as the C-ABI arrays: elements column by
    column, their (operator, scale) terms, each used operator's SU(2) rank and its
    sparse blocks (``bm/sparse_operator.h:105-168``)."""
    from .ts_mpo import sparse_of
    col_ptr, row_of, term_ptr, term_op, term_scale = [0], [], [0], [], []
    used = {}
    for b2 in range(mpo.col_dim):
        for b1 in mpo.column(b2):
            row_of.append(b1)
            for tag, scale in mpo.at(b1, b2):
                term_op.append(used.setdefault(tag, len(used)))
                term_scale.append(scale)
            term_ptr.append(len(term_op))
        col_ptr.append(len(row_of))
    op_spin, op_blk_ptr, blk_q, blk_ent_ptr, ent, ent_coeff = [], [0], [], [0], [], []
    for tag, _ in sorted(used.items(), key=lambda kv: kv[1]):
        op = mpo.op(tag)
        op_spin.append(op.spin.get())
        for (pin, pout), ents in zip(op.bm.keys, sparse_of(op)):
            blk_q += [pin[0], pin[1], pout[0], pout[1]]
            for (r, c, rs, cs, v) in ents:
                ent += [r, c, rs, cs]
                ent_coeff.append(v)
            blk_ent_ptr.append(len(ent_coeff))
        op_blk_ptr.append(len(blk_ent_ptr) - 1)
    h = mpo.herm
    i32 = lambda x: np.array(x or [0], dtype=np.int32)
    out = {"dims": np.array([mpo.row_dim, mpo.col_dim, len(op_spin)], dtype=np.int32),
           "left_spin": i32([s.get() for s in mpo.left_spins]), "right_spin": i32([s.get() for s in mpo.right_spins]),
           "left_herm": i32(h.LeftHerm), "right_herm": i32(h.RightHerm), "left_phase": i32(h.LeftPhase),
           "right_phase": i32(h.RightPhase), "col_ptr": i32(col_ptr), "row_of": i32(row_of),
           "term_ptr": i32(term_ptr), "term_op": i32(term_op),
           "term_scale": np.array(term_scale or [0.0], dtype=np.float64), "op_spin": i32(op_spin),
           "op_blk_ptr": i32(op_blk_ptr), "blk_q": i32(blk_q), "blk_ent_ptr": i32(blk_ent_ptr), "ent": i32(ent),
           "ent_coeff": np.array(ent_coeff or [0.0], dtype=np.float64)}
    return {prefix + k: v for k, v in out.items()}


def index_arrays(index, prefix: str) -> dict:
    return {prefix + ".q": np.array([x for c, _ in index for x in c] or [0], dtype=np.int32),
            prefix + ".size": np.array([s for _, s in index], dtype=np.int64)}


def block_arrays(keys, shapes, offsets, prefix: str) -> dict:
    return {prefix + ".q": np.array([[a[0], a[1], b[0], b[1]] for a, b in keys] or [[0, 0, 0, 0]],
                                    dtype=np.int32).reshape(-1),
            prefix + ".rows": np.array([s[0] for s in shapes], dtype=np.int64),
            prefix + ".cols": np.array([s[1] for s in shapes], dtype=np.int64),
            prefix + ".off": np.array(list(offsets), dtype=np.int64)}


def boundary_arrays(per_b, prefix: str):
    """Layout arrays of a boundary given as a list of block lists [(keys, shapes)], b-major
    arena; returns (arrays, total elements)."""
    keys, shapes, offs, ptr, base = [], [], [], [0], 0
    for ks, ss in per_b:
        for k, s in zip(ks, ss):
            keys.append(k)
            shapes.append(s)
            offs.append(base)
            base += s[0] * s[1]
        ptr.append(len(keys))
    out = block_arrays(keys, shapes, offs, prefix)
    out[prefix + ".blk_ptr"] = np.array(ptr, dtype=np.int32)
    return out, base


__all__ = ["build", "lib", "host_blas", "SigmaInputs", "sigma", "MPO_ARRAYS", "flatten_mpo", "index_arrays",
           "block_arrays", "boundary_arrays"]
