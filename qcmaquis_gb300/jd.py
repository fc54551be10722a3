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
layout; dot products, norms and updates use the library's deterministic
reductions.  The k x k (k <= maxiter) projected eigenproblem is solved on the
host in FP64 (the reference uses LAPACK dsyevx there too).
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

    ``ortho``: flat vectors in ``init``'s layout the solution is kept orthogonal
    to (excited states, ``ietl_jacobi_davidson.h:28-49``): Gram-Schmidt among
    themselves (dropped at norm <= ``completeness``), projected out of the start
    vector, of every new basis vector and of A u before the residual
    (``SingleSiteVS::project``, ``jacobi.h:378, 393, 432``).  With nothing left of
    the start vector after the projection the solve is skipped: (<init|A init>,
    init, 0)."""
    dev = init.data.device
    ops = VecOps(dev)
    n = init.n
    local: List[torch.Tensor] = []
    for o in list(ortho or [])[:max(n - 1, 0)]:
        v = o.clone()
        for q in local:
            ops.axpby(-ops.dot(q, v), q, 1.0, v)
        nv = ops.nrm2(v)
        if nv > completeness:
            ops.axpby(1.0 / nv, v, 0.0, v)
            local.append(v)

    def project(x: torch.Tensor):
        for q in local:
            ops.axpby(-ops.dot(q, x) / ops.dot(q, q), q, 1.0, x)

    if local:
        tmp = init.data.clone()
        for q in local:
            ops.axpby(-ops.dot(tmp, q), q, 1.0, tmp)
        if ops.nrm2(tmp) < completeness:
            return ops.dot(init.data, sp.apply(init).data), init, 0
    V: List[torch.Tensor] = []
    VA: List[torch.Tensor] = []
    M = np.zeros((maxiter, maxiter))
    kappa = 0.25
    t = init.data.clone()
    project(t)
    it = 0
    while True:
        tau = ops.nrm2(t)
        for i in range(it):
            ops.axpby(-ops.dot(V[i], t), V[i], 1.0, t)
        if ops.nrm2(t) < kappa * tau:
            for i in range(it):
                ops.axpby(-ops.dot(V[i], t), V[i], 1.0, t)
        project(t)
        nt = ops.nrm2(t)
        ops.axpby(1.0 / nt, t, 0.0, t)
        V.append(t)
        va = sp.apply(init.like(t)).data
        VA.append(va)
        col = ops.multi_dot(V, va)
        M[:it + 1, it] = col
        k = it + 1
        Ms = np.triu(M[:k, :k]) + np.triu(M[:k, :k], 1).T
        w, z = np.linalg.eigh(Ms)
        theta = float(w[0])
        s = z[:, 0]
        u = torch.empty(n, dtype=torch.float64, device=dev)
        uA = torch.empty(n, dtype=torch.float64, device=dev)
        ops.lincomb(V, s, u)
        ops.lincomb(VA, s, uA)
        project(uA)
        ops.axpby(-theta, u, 1.0, uA)  # r = uA - theta u  (in uA)
        it += 1
        rn = ops.nrm2(uA)
        if rn <= tol * abs(theta) or rn < tol or it >= maxiter:
            return theta, init.like(u), it
        ru = ops.dot(uA, u)
        uu = ops.dot(u, u)
        t = torch.empty(n, dtype=torch.float64, device=dev)
        ops.axpby(-1.0, uA, 0.0, t)
        ops.axpby(ru / uu, u, 1.0, t)


__all__ = ["solve_ietl_jcd", "VecOps"]
