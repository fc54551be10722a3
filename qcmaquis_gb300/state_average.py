"""State-averaged two-site DMRG: k roots of one Hamiltonian in one MPS.

The roots share every site tensor except the one at the orthogonality centre,
which carries the root index; the boundaries, and so the site Hamiltonian,
are shared too.  A microiteration at sites (i, i+1):

* forms the k two-site tensors theta_r (the centre tensor of root r times the
  shared neighbour) with the native two-site plan;
* applies H_eff to all k vectors at once: the site problem's sigma plan merged
  k times with shared boundary slots (``qcm_plan_merge``), so every stage of
  the k sigma vectors is one launch -- one persistent grouped block-product
  launch per stage per Davidson step, optionally replayed from a CUDA graph;
* finds the k lowest eigenpairs with a block Davidson iteration (FP64 vector
  algebra on the device: the library's multi-dot and linear-combination
  kernels; the Rayleigh-Ritz problem on the host);
* truncates with the state-averaged density matrix rho = sum_r w_r theta_r
  theta_r^T, through the SVD of the weighted concatenation
  M = [sqrt(w_1) theta_1, ..., sqrt(w_k) theta_k] (its left singular vectors and
  squared singular values are rho's eigenpairs; the batched Jacobi SVD and the
  device cut of the single-root path), keeping the new shared site tensor
  U and the k new centre tensors U^T theta_r (r2l: theta_r V).

The reference optimises excited states one after another, each orthogonal to
the lower ones (``sba/SweepBasedEnergyMinimization.h:52-67``, built in
``excited.py``); the state-averaged form is this implementation's own.  The
block Davidson uses the reference's zero-GMRES Jacobi-Davidson correction
t = -r + (r.u / u.u) u per unconverged root and its stopping rule
(|r| <= tol |theta|).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import List, Optional, Sequence

import numpy as np
import torch

from . import mps_ops as O
from . import native as N
from .engine import DeviceBoundary, DeviceMPSTensor, Engine
from .jd import VecOps
from .symmetry import adjoin, common_subset, index_product


class SharedSigma:
    """sigma of k vectors of one site problem: its plan merged k times, the vectors
    (and results) back to back, the boundaries shared by every copy."""

    def __init__(self, engine: Engine, ket: DeviceMPSTensor, L: DeviceBoundary, R: DeviceBoundary, mpo, k: int):
        self.engine = engine
        self.k = k
        self.n = max(ket.n, 1)
        base = N.plan_sigma(ket.phys_i, ket.left_i, ket.right_i, ket.layout, L.layout, R.layout, engine.fmpo(mpo),
                            engine.hermitian)
        self.plan = N.plan_merge([base] * k, [(r * self.n, 0, 0, r * self.n) for r in range(k)])
        self.plan.upload()
        self.L, self.R = L, R
        self.calls = 0
        self._graph = None

    def apply(self, X: torch.Tensor, out: Optional[torch.Tensor] = None) -> torch.Tensor:
        """X: (k, n) contiguous; returns H_eff applied to every row, one launch per stage."""
        if out is None:
            out = torch.empty_like(X)
        self.engine.run(self.plan, ket=X, left=self.L, right=self.R, out=out)
        self.calls += 1
        return out

    def capture(self):
        """Capture the merged sigma in a CUDA graph on static buffers."""
        dev = self.engine.device
        self._gin = torch.zeros((self.k, self.n), dtype=torch.float64, device=dev)
        self._gout = torch.empty_like(self._gin)
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            for _ in range(2):
                self.engine.run(self.plan, ket=self._gin, left=self.L, right=self.R, out=self._gout)
        torch.cuda.current_stream(dev).wait_stream(side)
        torch.cuda.synchronize(dev)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.engine.run(self.plan, ket=self._gin, left=self.L, right=self.R, out=self._gout)
        self._graph = g
        return self

    def apply_graph(self, X: torch.Tensor) -> torch.Tensor:
        self._gin.copy_(X)
        self._graph.replay()
        self.calls += 1
        return self._gout.clone()


def block_davidson(sig: SharedSigma, X0: torch.Tensor, tol: float = 1e-8, maxiter: int = 20, max_sub: int = 0,
                   use_graph: bool = False):
    """The k lowest eigenpairs of the shared H_eff from the k start vectors X0 (k, n).
    Returns (eigenvalues (k,), eigenvectors (k, n), iterations)."""
    k, n = X0.shape
    dev = X0.device
    ops = VecOps(dev)
    max_sub = max_sub or max(4 * k, k + 8)
    apply = sig.apply_graph if (use_graph and sig._graph is not None) else sig.apply
    V: List[torch.Tensor] = []
    AV: List[torch.Tensor] = []

    def dots(vs, y):
        out = []
        for c in range(0, len(vs), 32):
            out.append(ops.multi_dot(vs[c:c + 32], y))
        return np.concatenate(out) if out else np.zeros(0)

    def lin(vs, coef, out):
        """out = sum_i coef_i vs_i (chunks of 32 vectors per launch)."""
        ops.lincomb(vs[:32], coef[:32], out)
        tmp = None
        for c in range(32, len(vs), 32):
            tmp = torch.empty_like(out) if tmp is None else tmp
            ops.lincomb(vs[c:c + 32], coef[c:c + 32], tmp)
            ops.axpby(1.0, tmp, 1.0, out)

    def orthonormalize_into(cands: Sequence[torch.Tensor]) -> List[torch.Tensor]:
        """Modified Gram-Schmidt (two passes) of the candidates against V and each other."""
        added = []
        tmp = torch.empty(n, dtype=torch.float64, device=dev)
        for t in cands:
            t = t.clone()
            tau = math.sqrt(max(ops.dot(t, t), 0.0))
            for _ in range(2):
                basis = V + added
                if basis:
                    lin(basis, dots(basis, t), tmp)
                    ops.axpby(-1.0, tmp, 1.0, t)
            nt = math.sqrt(max(ops.dot(t, t), 0.0))
            if tau == 0.0 or nt <= 1e-10 * tau:
                continue
            ops.axpby(0.0, t, 1.0 / nt, t)
            added.append(t)
        return added

    def extend(cands):
        new = orthonormalize_into(cands)
        if not new:
            return 0
        X = torch.stack(new + [torch.zeros(n, dtype=torch.float64, device=dev)] * (k - len(new))) \
            if len(new) < k else torch.stack(new)
        AX = apply(X.contiguous())
        for j, v in enumerate(new):
            V.append(v)
            AV.append(AX[j].clone())
        return len(new)

    extend([X0[r] for r in range(k)])
    # start vectors that span fewer than k directions (the roots' centre tensors at a
    # chain end have few parameters) are completed with seeded random directions
    gen = torch.Generator(device=dev).manual_seed(1234)
    for _ in range(4 * k):
        if len(V) >= k:
            break
        extend([torch.randn(n, dtype=torch.float64, device=dev, generator=gen) for _ in range(k - len(V))])
    if len(V) < k:
        raise ValueError(f"the site problem has fewer than {k} dimensions")
    theta = np.zeros(k)
    U = torch.zeros((k, n), dtype=torch.float64, device=dev)
    it = 0
    while True:
        m = len(V)
        Mh = np.zeros((m, m))
        for j in range(m):
            Mh[:, j] = dots(V, AV[j])
        Mh = 0.5 * (Mh + Mh.T)
        w, Z = np.linalg.eigh(Mh)
        theta = w[:k].copy()
        AU = torch.zeros((k, n), dtype=torch.float64, device=dev)
        for r in range(k):
            lin(V, np.ascontiguousarray(Z[:, r]), U[r])
            lin(AV, np.ascontiguousarray(Z[:, r]), AU[r])
        it += 1
        res = []
        conv = np.zeros(k, dtype=bool)
        for r in range(k):
            rv = AU[r].clone()
            ops.axpby(-float(theta[r]), U[r], 1.0, rv)
            rn = math.sqrt(max(ops.dot(rv, rv), 0.0))
            conv[r] = rn <= tol * abs(theta[r]) or rn < tol
            res.append(rv)
        if conv.all() or it >= maxiter:
            return theta, U, it
        cands = []
        for r in np.nonzero(~conv)[0]:
            u, rv = U[r], res[r]
            f = ops.dot(rv, u) / max(ops.dot(u, u), 1e-300)
            t = -rv
            ops.axpby(f, u, 1.0, t)
            cands.append(t)
        if len(V) + len(cands) > max_sub:
            # restart from the current Ritz vectors
            V.clear()
            AV.clear()
            for r in range(k):
                V.append(U[r].clone())
                AV.append(AU[r].clone())
        if extend(cands) == 0:
            return theta, U, it


def _concat(blocks_by_root: List[O.DBM], w: Sequence[float], l2r: bool) -> O.DBM:
    """M = [sqrt(w_r) theta_r] concatenated along columns (l2r) or rows (r2l), block by block."""
    M = O.DBM()
    base = blocks_by_root[0]
    for j, key in enumerate(base.keys):
        parts = [math.sqrt(w[r]) * blocks_by_root[r].blocks[j] for r in range(len(blocks_by_root))]
        M.keys.append(key)
        M.blocks.append(torch.cat(parts, dim=1 if l2r else 0).contiguous())
    return M


def sa_split(thetas: Sequence[DeviceMPSTensor], A0: DeviceMPSTensor, B0: DeviceMPSTensor, w: Sequence[float],
             Mmax: int, cutoff: float, l2r: bool, symmetry: int = N.SYM_SU2U1):
    """The state-averaged truncation of the k two-site tensors: returns (shared site
    tensor, k centre tensors, truncation results).  l2r: the shared tensor is the new
    site i (left-normalised) and the centres sit at i+1; r2l: the shared one is site
    i+1 (right-normalised) and the centres sit at site i."""
    p1, p2 = A0.phys_i, B0.phys_i
    both = []
    for t in thetas:
        _, blay, bflat = O.split_theta(t, A0, B0, symmetry)
        both.append(O.block_views(blay, bflat.clone()))
    M = _concat(both, w, l2r)
    U, S, V, tr = O.svd_truncate(M, cutoff, Mmax)
    k = len(thetas)
    if l2r:
        A_lp = U
        a_right = A_lp.right_basis()
        a_left = A0.left_i.copy()
        common_subset(a_left, index_product(adjoin(p1), a_right))
        shared = O.from_dbm(p1, a_left, a_right, A_lp)
        centres = []
        for r in range(k):
            Brp = O.DBM()
            for (lc, rc), vb in zip(V.keys, V.blocks):
                cols = vb.shape[1] // k
                Brp.insert((S[rc][:, None] * vb[:, r * cols:(r + 1) * cols]) / math.sqrt(w[r]), lc, rc)
            b_left = Brp.left_basis()
            b_right = B0.right_i.copy()
            common_subset(b_right, index_product(p2, b_left))
            centres.append(O.from_dbm(p2, b_left, b_right, O.reshape_r2l(p2, b_left, b_right, Brp)))
        return shared, centres, tr
    Brp = V
    b_left = Brp.left_basis()
    b_right = B0.right_i.copy()
    common_subset(b_right, index_product(p2, b_left))
    shared = O.from_dbm(p2, b_left, b_right, O.reshape_r2l(p2, b_left, b_right, Brp))
    centres = []
    for r in range(k):
        Alp = O.DBM()
        for (lc, rc), ub in zip(U.keys, U.blocks):
            rows = ub.shape[0] // k
            Alp.insert((ub[r * rows:(r + 1) * rows, :] * S[rc][None, :]) / math.sqrt(w[r]), lc, rc)
        a_right = Alp.right_basis()
        a_left = A0.left_i.copy()
        common_subset(a_left, index_product(adjoin(p1), a_right))
        centres.append(O.from_dbm(p1, a_left, a_right, Alp))
    return shared, centres, tr


@dataclass
class SARecord:
    energies: List[np.ndarray] = field(default_factory=list)       # Ritz values per microiteration
    sweep_energies: List[np.ndarray] = field(default_factory=list)  # FP64 <H>_r per sweep
    truncated_weight: List[float] = field(default_factory=list)
    bond_dimension: List[int] = field(default_factory=list)
    iterations: List[int] = field(default_factory=list)
    sigma_launches: List[int] = field(default_factory=list)          # merged sigma calls per microiteration
    sweep_seconds: List[float] = field(default_factory=list)


def _root_chain(mps: List[DeviceMPSTensor], center: int, c: DeviceMPSTensor) -> List[DeviceMPSTensor]:
    out = list(mps)
    out[center] = c
    return out


def run_sa_dmrg(model, mpo, p, nelec: int, twoS: int = 0, nroots: int = 2, weights: Optional[Sequence[float]] = None,
                mps: Optional[List[DeviceMPSTensor]] = None, engine: Optional[Engine] = None, device="cuda",
                precision: int = 0, ts_mpo=None, use_graph: bool = False, seed: int = 7):
    """State-averaged two-site sweeps for the ``nroots`` lowest states (equal weights
    by default).  ``p`` is a ``sweep.SweepParams`` (Mmax, cutoff, Davidson tolerance
    and iteration limit, sweep count).  Returns (SARecord, shared MPS, centre site,
    centre tensors)."""
    import time
    from .sweep import (JD_RESIDUAL_FLOOR, _ones_boundary, default_mps_init, expval, get_cutoff, get_Mmax,
                        normalize_right, overlap)
    L = model.L
    k = int(nroots)
    w = [1.0 / k] * k if weights is None else [float(x) / sum(weights) for x in weights]
    sym = N.symmetry_code(getattr(model, "symmetry", "su2u1"))
    right_end = model.right_end if sym != N.SYM_SU2U1 else (nelec, twoS)
    engine = engine or Engine(device, precision=precision)
    engine_full = Engine(device, hermitian=False)
    # a mixed-precision sigma cannot resolve residuals below its own error
    jd_tol = max(p.ietl_jcd_tol, JD_RESIDUAL_FLOOR.get(engine.precision, 0.0))
    if mps is None:
        mps = default_mps_init(L, model.phys, right_end, p.init_bond_dimension, p.seed, device,
                               abelian=sym != N.SYM_SU2U1)
        normalize_right(mps)
    if ts_mpo is None:
        ts_mpo = N.make_ts_cache_fmpo(mpo, model.phys)
    gen = torch.Generator(device=engine.device).manual_seed(seed)
    centre = 0
    roots = [mps[0]]
    for _ in range(1, k):
        d = torch.rand(mps[0].data.shape, dtype=torch.float64, device=engine.device, generator=gen)
        roots.append(DeviceMPSTensor(mps[0].phys_i, mps[0].left_i, mps[0].right_i, mps[0].layout, d))
    left: List = [None] * (L + 1)
    right: List = [None] * (L + 1)
    left[0] = _ones_boundary((0, 0), engine.device)
    right[L] = _ones_boundary(right_end, engine.device)
    for i in range(L - 1, 0, -1):
        right[i] = engine.overlap_mpo_right_step(mps[i], right[i + 1], mpo[i])
    rec = SARecord()
    nmicro = 2 * (L - 2) if L > 2 else 1
    for sweep in range(p.nsweeps):
        t0 = time.time()
        Mmax = get_Mmax(p, sweep)
        cutoff = get_cutoff(p, sweep)
        for mi in range(nmicro):
            site = mi if mi < L - 1 else 2 * L - 4 - mi
            forward = mi < L - 1
            change = (mi == L - 2) or (mi == nmicro - 1)
            l2r = forward and not change
            if centre == site:
                thetas = [O.make_two_site_mps(c, mps[site + 1], sym) for c in roots]
            elif centre == site + 1:
                thetas = [O.make_two_site_mps(mps[site], c, sym) for c in roots]
            else:
                raise RuntimeError("the centre is not on the site pair")
            sig = SharedSigma(engine, thetas[0], left[site], right[site + 2], ts_mpo[site], k)
            if use_graph:
                sig.capture()
            X0 = torch.stack([t.data for t in thetas]).contiguous()
            theta, Uv, iters = block_davidson(sig, X0, jd_tol, p.ietl_jcd_maxiter, use_graph=use_graph)
            rec.energies.append(theta + mpo.core_energy)
            rec.iterations.append(iters)
            rec.sigma_launches.append(sig.calls)
            A0, B0 = (roots[0], mps[site + 1]) if centre == site else (mps[site], roots[0])
            us = [DeviceMPSTensor(thetas[0].phys_i, thetas[0].left_i, thetas[0].right_i, thetas[0].layout,
                                  Uv[r].clone()) for r in range(k)]
            shared, centres, tr = sa_split(us, A0, B0, w, Mmax, cutoff, l2r, sym)
            rec.truncated_weight.append(tr.truncated_weight)
            rec.bond_dimension.append(tr.bond_dimension)
            if l2r:
                mps[site] = shared
                mps[site + 1] = centres[0]
                centre = site + 1
                left[site + 1] = engine.overlap_mpo_left_step(mps[site], left[site], mpo[site])
            else:
                mps[site + 1] = shared
                mps[site] = centres[0]
                centre = site
                right[site + 1] = engine.overlap_mpo_right_step(mps[site + 1], right[site + 2], mpo[site + 1])
            roots = centres
        torch.cuda.synchronize()
        rec.sweep_seconds.append(time.time() - t0)
        e = []
        for c in roots:
            chain = _root_chain(mps, centre, c)
            e.append(expval(chain, mpo, engine_full, right_end) / overlap(chain) + mpo.core_energy)
        rec.sweep_energies.append(np.array(e))
    return rec, mps, centre, roots


__all__ = ["SharedSigma", "block_davidson", "sa_split", "run_sa_dmrg", "SARecord"]
