"""Many independent site problems solved together on one GPU.

The sigma plans of all problems are merged into one plan (``qcm_plan_merge``):
their vectors, boundaries and results live back to back in shared arenas and
every stage of a sigma vector runs all problems' work in one launch -- one
persistent grouped block-product launch per stage for the whole batch.  The
merged sigma can be captured once in a CUDA graph and replayed for every
Davidson step.  ``solve_jcd_batched`` runs the reference's Jacobi-Davidson
iteration (``dmrg/framework/ietl/jacobi.h:361-493`` with zero GMRES steps, as
``jd.solve_ietl_jcd``) for all problems in lockstep on the concatenated
vectors: per-problem dot products through one segmented reduction
(``qcm_seg_multi_dot``), per-problem coefficients broadcast over each problem's
segment, a problem that has converged keeps its result and stops updating.
The reference solves its excited states and independent problems one after
the other; batching is this implementation's own.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Optional, Sequence, Tuple

import numpy as np
import torch

from . import native as N
from .engine import DeviceBoundary, DeviceMPSTensor, Engine


class BatchedSigma:
    """sigma = H_eff psi for a batch of problems (psi_k, L_k, R_k, W_k) in one merged plan."""

    def __init__(self, engine: Engine, problems: Sequence[Tuple[DeviceMPSTensor, DeviceBoundary, DeviceBoundary,
                                                                 object]]):
        self.engine = engine
        dev = engine.device
        self.kets = [p[0] for p in problems]
        plans, offs = [], []
        ko = lo = ro = 0
        for ket, L, R, mpo in problems:
            p = N.plan_sigma(ket.phys_i, ket.left_i, ket.right_i, ket.layout, L.layout, R.layout, engine.fmpo(mpo),
                             engine.hermitian)
            plans.append(p)
            # sigma has the ket's layout: the result slice is the ket slice
            offs.append((ko, lo, ro, ko))
            ko += max(ket.n, 1)
            lo += L.data.numel()
            ro += R.data.numel()
        self.plan = N.plan_merge(plans, offs)
        self.plan.upload()
        self.n = ko
        self.offsets = [o[0] for o in offs] + [ko]
        self.lengths = [max(k.n, 1) for k in self.kets]
        self.left = DeviceBoundary(None, torch.cat([p[1].data for p in problems]))
        self.right = DeviceBoundary(None, torch.cat([p[2].data for p in problems]))
        self.seg = torch.tensor(self.offsets, dtype=torch.int64, device=dev)
        self._graph = None
        self._gin = self._gout = None

    def pack(self, vectors: Sequence[torch.Tensor]) -> torch.Tensor:
        """Concatenate one flat vector per problem into the batch layout."""
        out = torch.zeros(self.n, dtype=torch.float64, device=self.engine.device)
        for o, v in zip(self.offsets, vectors):
            out[o:o + v.numel()].copy_(v)
        return out

    def unpack(self, x: torch.Tensor) -> List[torch.Tensor]:
        return [x[o:o + k.n] for o, k in zip(self.offsets, self.kets)]

    def apply(self, x: torch.Tensor, out: Optional[torch.Tensor] = None, precision=None) -> torch.Tensor:
        """All problems' sigma vectors, one launch per stage."""
        if out is None:
            out = torch.empty(self.n, dtype=torch.float64, device=self.engine.device)
        self.engine.run(self.plan, ket=x, left=self.left, right=self.right, out=out, precision=precision)
        return out

    def capture(self, precision=None):
        """Capture the merged sigma in a CUDA graph on static input/output buffers."""
        dev = self.engine.device
        self._gin = torch.zeros(self.n, dtype=torch.float64, device=dev)
        self._gout = torch.empty(self.n, dtype=torch.float64, device=dev)
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            for _ in range(2):   # scratch and FP32 shadows allocated before the capture
                self.apply(self._gin, self._gout, precision)
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.apply(self._gin, self._gout, precision)
        self._graph = g
        return self

    def apply_graph(self, x: torch.Tensor) -> torch.Tensor:
        """Replay the captured sigma: copy in, replay, copy out."""
        self._gin.copy_(x)
        self._graph.replay()
        return self._gout.clone()


class _SegOps:
    """Per-problem reductions and coefficient broadcasts on concatenated vectors."""

    def __init__(self, bs: BatchedSigma):
        self.lib = N.lib()
        self.P = len(bs.kets)
        self.seg = bs.seg
        self.lengths = torch.tensor(bs.lengths, dtype=torch.int64, device=bs.seg.device)
        self.out = torch.zeros(32 * self.P, dtype=torch.float64, device=bs.seg.device)
        self.dev = bs.seg.device

    def dots(self, vs: Sequence[torch.Tensor], y: torch.Tensor) -> np.ndarray:
        """(len(vs), P) array of segment dots, one launch per 32 vectors."""
        res = []
        stream = C.c_void_p(int(torch.cuda.current_stream(self.dev).cuda_stream))
        for c0 in range(0, len(vs), 32):
            part = vs[c0:c0 + 32]
            arr = (C.c_void_p * len(part))(*[C.c_void_p(v.data_ptr()) for v in part])
            N.check(self.lib.qcm_seg_multi_dot(arr, len(part), y.data_ptr(), self.seg.data_ptr(), self.P,
                                               self.out.data_ptr(), stream), "qcm_seg_multi_dot")
            res.append(self.out[:len(part) * self.P].view(len(part), self.P).cpu().numpy().copy())
        return np.concatenate(res, axis=0)

    def spread(self, coef) -> torch.Tensor:
        """One coefficient per problem broadcast over the problem's segment."""
        c = torch.as_tensor(np.asarray(coef, dtype=np.float64), device=self.dev)
        return torch.repeat_interleave(c, self.lengths)


def solve_jcd_batched(bs: BatchedSigma, inits: torch.Tensor, tol: float = 1e-8, maxiter: int = 10,
                      use_graph: bool = False):
    """Smallest eigenpair of every problem's H_eff, all problems in lockstep.
    Returns (theta per problem, eigenvectors in the batch layout, iterations per
    problem)."""
    ops = _SegOps(bs)
    P = ops.P
    kappa = 0.25
    apply = bs.apply_graph if (use_graph and bs._graph is not None) else bs.apply
    M = np.zeros((P, maxiter, maxiter))
    V: List[torch.Tensor] = []
    VA: List[torch.Tensor] = []
    active = np.ones(P, dtype=bool)
    theta = np.zeros(P)
    iters = np.zeros(P, dtype=np.int64)
    result = torch.zeros_like(inits)
    t = inits.clone()
    it = 0
    while True:
        tau = np.sqrt(np.maximum(ops.dots([t], t)[0], 0.0))
        for i in range(it):
            t -= ops.spread(ops.dots([V[i]], t)[0]) * V[i]
        nrm = np.sqrt(np.maximum(ops.dots([t], t)[0], 0.0))
        refine = nrm < kappa * tau
        if refine.any():
            for i in range(it):
                t -= ops.spread(ops.dots([V[i]], t)[0] * refine) * V[i]
        nt = np.sqrt(np.maximum(ops.dots([t], t)[0], 0.0))
        t *= ops.spread(np.where(nt > 0, 1.0 / np.where(nt > 0, nt, 1.0), 0.0))
        V.append(t)
        va = apply(t)
        VA.append(va)
        col = ops.dots(V, va)                       # (it + 1, P)
        S = np.zeros((it + 1, P))
        for k in np.nonzero(active)[0]:
            M[k, :it + 1, it] = col[:, k]
            Mk = M[k, :it + 1, :it + 1]
            Ms = np.triu(Mk) + np.triu(Mk, 1).T
            w, z = np.linalg.eigh(Ms)
            theta[k] = float(w[0])
            S[:, k] = z[:, 0]
        u = torch.zeros_like(t)
        uA = torch.zeros_like(t)
        for j in range(it + 1):
            c = ops.spread(S[j])
            u += c * V[j]
            uA += c * VA[j]
        r = uA - ops.spread(theta) * u
        it += 1
        rn = np.sqrt(np.maximum(ops.dots([r], r)[0], 0.0))
        done = active & ((rn <= tol * np.abs(theta)) | (rn < tol) | (it >= maxiter))
        if done.any():
            mask = ops.spread(done.astype(np.float64)) > 0
            result = torch.where(mask, u, result)
            iters[done] = it
            active &= ~done
        if not active.any():
            return theta, result, iters
        ru = ops.dots([r], u)[0]
        uu = ops.dots([u], u)[0]
        # t = -r + (r.u / u.u) u for the active problems, 0 for the finished ones
        f = np.where(active, ru / np.where(uu != 0, uu, 1.0), 0.0)
        t = (ops.spread(f) * u) - ops.spread(active.astype(np.float64)) * r


__all__ = ["BatchedSigma", "solve_jcd_batched"]
