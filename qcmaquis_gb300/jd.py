"""Jacobi-Davidson eigensolver on the GPU (``solve_ietl_jcd``).

Restates ``jacobi_davidson::calculate_eigenvalue`` with zero GMRES steps, as
the live path runs it (``dmrg/framework/ietl/jacobi.h:99-138, 361-493``,
``dmrg/framework/dmrg/optimize/ietl_jacobi_davidson.h:16-77``):
modified Gram-Schmidt with one refinement when the norm drops below
kappa = 0.25 of its start, normalisation, sigma vector, projected matrix
column, smallest Ritz pair, u = V s, uA = VA s, residual r = uA - theta u,
stop when ||r|| <= tol*|theta| or ||r|| < tol or after maxiter steps, else
t = -r + (r.u / u.u) u.

Vectors are flat FP64 CUDA buffers in the two-site tensor's left-paired
layout; the iteration runs in native code (``qcm_jcd_solve``) with the
library's deterministic reductions.  The k x k (k <= maxiter) projected
eigenproblem is solved on the host in FP64 (the reference uses LAPACK dsyevx
there too).  ``VecOps`` exposes the vector kernels to the batched solver.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import native as N
from .engine import DeviceMPSTensor, SiteProblem


class VecOps:
    def __init__(self, device):
        self.lib = N.lib()
        self.res = torch.zeros(64, dtype=torch.float64, device=device)
        self.stream = lambda: C.c_void_p(int(torch.cuda.current_stream(device).cuda_stream))

    def dot(self, x: torch.Tensor, y: torch.Tensor) -> float:
        N.check(self.lib.qcm_dot(x.data_ptr(), y.data_ptr(), x.numel(), self.res.data_ptr(), self.stream()), "dot")
        return float(self.res[0].item())

    def nrm2(self, x: torch.Tensor) -> float:
        N.check(self.lib.qcm_nrm2(x.data_ptr(), x.numel(), self.res.data_ptr(), self.stream()), "nrm2")
        return float(self.res[0].item())

    def multi_dot(self, vs: List[torch.Tensor], y: torch.Tensor) -> np.ndarray:
        arr = (C.c_void_p * len(vs))(*[C.c_void_p(v.data_ptr()) for v in vs])
        N.check(self.lib.qcm_multi_dot(arr, len(vs), y.data_ptr(), y.numel(), self.res.data_ptr(), self.stream()),
                "multi_dot")
        return self.res[:len(vs)].cpu().numpy().copy()

    def axpby(self, a: float, x: torch.Tensor, b: float, y: torch.Tensor):
        N.check(self.lib.qcm_axpby(a, x.data_ptr(), b, y.data_ptr(), x.numel(), self.stream()), "axpby")

    def lincomb(self, vs: List[torch.Tensor], coef, out: torch.Tensor):
        arr = (C.c_void_p * len(vs))(*[C.c_void_p(v.data_ptr()) for v in vs])
        c = np.ascontiguousarray(coef, dtype=np.float64)
        N.check(self.lib.qcm_lincomb(arr, c.ctypes.data_as(N.f64p), len(vs), out.data_ptr(), out.numel(),
                                     self.stream()), "lincomb")


def solve_ietl_jcd(sp: SiteProblem, init: DeviceMPSTensor, tol: float = 1e-8, maxiter: int = 10,
                   ortho: Optional[Sequence[torch.Tensor]] = None, completeness: float = 1e-10):
    """Smallest eigenpair of H_eff; returns (theta, eigenvector tensor, iterations).

    Runs the library's native Jacobi-Davidson (``qcm_jcd_solve``: the iteration of
    ``jacobi.h:361-451`` with zero GMRES steps, every Gram-Schmidt and projection
    coefficient kept on the device) on the engine's context, with the site
    problem's sigma plan in the engine's precision.

    ``ortho``: flat vectors in ``init``'s layout the solution is kept orthogonal
    to (excited states, ``ietl_jacobi_davidson.h:28-49``): Gram-Schmidt among
    themselves (dropped at norm <= 1e-10), projected out of the start vector, of
    every new basis vector and of A u before the residual
    (``SingleSiteVS::project``, ``jacobi.h:378, 393, 432``).  With nothing left of
    the start vector after the projection the solve is skipped: (<init|A init>,
    init, 0)."""
    if completeness != 1e-10:
        raise ValueError("the native solver drops constraint vectors below a norm of 1e-10")
    eng = sp.engine
    plan = eng.sigma_plan(init, sp.left, sp.right, sp.mpo)
    ctx = eng.context()
    out = torch.empty_like(init.data)
    e, it = C.c_double(), C.c_int32()
    ov = list(ortho or [])
    arr = (C.c_void_p * max(len(ov), 1))(*[C.c_void_p(v.data_ptr()) for v in ov]) if ov else None
    lt, rt = sp.left.data, sp.right.data
    N.check(N.lib().qcm_jcd_solve(ctx.h, plan.h, C.c_void_p(lt.data_ptr()), lt.numel(), C.c_void_p(rt.data_ptr()),
                                  rt.numel(), eng.precision, C.c_void_p(init.data.data_ptr()), init.n, float(tol),
                                  int(maxiter), arr, len(ov), C.c_void_p(out.data_ptr()), C.byref(e), C.byref(it)),
            "qcm_jcd_solve")
    eng.launches += it.value * plan.last_kernels()
    return e.value, init.like(out), it.value


__all__ = ["solve_ietl_jcd", "VecOps"]
