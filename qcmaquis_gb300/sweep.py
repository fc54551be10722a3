"""Two-site ground-state sweeps on the GPU.

Mirrors the live driver of the reference -- ``SweepBasedEnergyMinimization`` on
``GenericSweepSimulation::runSingleSweep`` (``sba/GenericSweepSimulation.h:73-152,
212-268``), the two-site microiteration schedule
(``sba/SweepOptimizationTypeTrait.h:85-142``), ``BoundaryPropagator``
(``sba/BoundaryPropagator.h:36-150``) and ``SweepMPSUpdater<TwoSite>``
(``sba/SweepMPSUpdater.h:180-258``) -- with every tensor on the GPU: sigma
vectors and boundary updates through the native plans, the eigensolver on
the native vector kernels, factorisations through cuSOLVER.  Per-sweep
energies follow ``get_energy`` (``fw/sim/interface_sim.h:355-360``).
"""
from __future__ import annotations

import math
import time
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np
import torch

from . import mps_ops as O
from .block_matrix import BlockMatrix
from .engine import DeviceBoundary, DeviceMPSTensor, Engine, SiteProblem
from .excited import OverlapBoundaries
from .jd import solve_ietl_jcd
from . import native as N
from .mps import allowed_sectors
from .symmetry import Index, adjoin, common_subset, index_product


@dataclass
class SweepParams:
    """The sweep keys of ``DmrgParameters`` (``fw/utils/DmrgParameters.h:37-68``)."""
    nsweeps: int = 2
    max_bond_dimension: int = 64
    sweep_bond_dimensions: Optional[List[int]] = None
    init_bond_dimension: int = 5
    truncation_initial: float = 1e-16
    truncation_final: float = 1e-16
    ngrowsweeps: int = 2
    ietl_jcd_tol: float = 1e-8
    ietl_jcd_maxiter: int = 10
    seed: int = 42
    # "svd" (default) or "heev" with the noise schedule below (DmrgParameters.h:45-59)
    twosite_truncation: str = "svd"
    alpha_initial: float = 1e-2
    alpha_main: float = 1e-4
    alpha_final: float = 1e-8
    nmainsweeps: int = 5


def get_alpha(p: SweepParams, sweep: int) -> float:
    """``getAlpha`` (``sba/GenericSweepSimulation.h:242-253``)."""
    if sweep < p.ngrowsweeps:
        return p.alpha_initial
    if sweep < p.ngrowsweeps + p.nmainsweeps:
        return p.alpha_main
    return p.alpha_final


def _log_interpolate(y0, y1, N, i):
    if N < 2:
        return y1
    if y0 == 0:
        return 0.0
    return y0 * math.exp(math.log(y1 / y0) / (N - 1) * i)


def get_cutoff(p: SweepParams, sweep: int) -> float:
    if sweep >= p.ngrowsweeps:
        return p.truncation_final
    return _log_interpolate(p.truncation_initial, p.truncation_final, p.ngrowsweeps, sweep)


def get_Mmax(p: SweepParams, sweep: int) -> int:
    if p.sweep_bond_dimensions:
        return p.sweep_bond_dimensions[min(sweep, len(p.sweep_bond_dimensions) - 1)]
    return p.max_bond_dimension


@dataclass
class SweepRecord:
    energies: List[float] = field(default_factory=list)
    truncated_weight: List[float] = field(default_factory=list)
    bond_dimension: List[int] = field(default_factory=list)
    jd_iterations: List[int] = field(default_factory=list)
    sweep_energy: List[float] = field(default_factory=list)
    sweep_truncated_weight: List[float] = field(default_factory=list)
    sweep_seconds: List[float] = field(default_factory=list)
    sigma_calls: int = 0
    plan_hits: int = 0
    boundary_plan_hits: int = 0
    # per microiteration: a digest of the sigma problem's layouts (psi, L, R) -- equal
    # digests at the same site in different sweeps could share one plan
    layout_digests: List[int] = field(default_factory=list)
    # measurement runs with a shadow FP64 engine: per microiteration (Ritz value, FP64
    # Rayleigh quotient of the eigenvector, FP64 eigenvalue from the same start)
    shadow: List = field(default_factory=list)
    # wall time per part of the sweeps (host clock, device synchronised at each part's end)
    seconds: Dict[str, float] = field(default_factory=lambda: {"eigensolver": 0.0, "truncation": 0.0,
                                                               "boundary": 0.0, "plans": 0.0})


# Relative residual a mixed-precision sigma can resolve: below it the residual of the
# eigensolver is rounding of the sigma itself (measured relative sigma errors at
# m=1024: BF16x3 1.1e-6 to 2.1e-6, BF16x2 3.8e-6, TF32 2.6e-4), so the solver stops
# there instead of running to its iteration limit.  FP64 keeps the reference's test.
JD_RESIDUAL_FLOOR = {N.PREC_FP64: 0.0, N.PREC_TF32: 5e-4, N.PREC_BF16X3: 2e-6, N.PREC_BF16X2: 1e-5}


def default_mps_init(L, phys, right_end, init_bond_dimension, seed, device="cuda",
                     abelian: bool = False) -> List[DeviceMPSTensor]:
    """``default_mps_init`` (``mp_tensors/mps_initializers.h:34-81``): allowed sectors capped at
    ``init_bond_dimension``, uniform [0,1) entries (numpy PCG64 stream seeded with ``seed``,
    filled block by block in column-major order), each site divided by its norm.
    ``abelian``: TwoU1 charges."""
    rng = np.random.default_rng(seed)
    allowed = allowed_sectors(L, phys, right_end, init_bond_dimension, abelian=abelian)
    out = []
    for i in range(L):
        lb = index_product(phys, allowed[i])
        rb = allowed[i + 1].copy()
        common_subset(lb, rb)
        left = allowed[i].copy()
        common_subset(left, index_product(adjoin(phys), rb))
        bm = BlockMatrix.from_indices(lb, rb)
        for k in range(bm.n_blocks()):
            b = bm.blocks[k]
            bm.blocks[k] = rng.random(b.size).reshape(b.shape, order="F")
        bm.scale(1.0 / bm.norm())

        class _T:
            pass
        t = _T()
        t.phys_i, t.left_i, t.right_i, t.data = phys, left, rb, bm
        out.append(DeviceMPSTensor.from_host(t, device=device))
    return out


def normalize_right(mps: List[DeviceMPSTensor]):
    """``MPS::normalize_right`` (``mp_tensors/mps.hpp:117-128``)."""
    L = len(mps)
    for i in range(L - 1, 0, -1):
        mps[i], t = O.right_normalize_and_return(mps[i])
        mps[i - 1] = O.multiply_from_right(mps[i - 1], t)
    mps[0], nf = O.right_normalize_and_return(mps[0])
    tr = sum(float(torch.trace(b).item()) for b in nf.blocks)
    if tr < 0:
        mps[0].data.mul_(-1.0)


def _ones_boundary(c, device):
    return DeviceBoundary.from_host([BlockMatrix.from_indices(Index([(c, 1)]), Index([(c, 1)]), fill=1.0)], device)


def overlap(mps: List[DeviceMPSTensor]) -> float:
    """<psi|psi> by transfer matrices (``overlap``, ``mp_tensors/mps_mpo_ops.h``)."""
    Lb = O.DBM()
    Lb.insert(torch.ones((1, 1), dtype=torch.float64, device=mps[0].data.device), (0, 0), (0, 0))
    for t in mps:
        rp = O.reshape_l2r(t.phys_i, t.left_i, t.right_i, O.as_dbm(t))
        t1 = O.gemm(Lb, rp)
        t3 = O.reshape_r2l(t.phys_i, t.left_i, t.right_i, t1)
        Lb = O.gemm(O.as_dbm(t), t3, ta=True)
    return float(sum(torch.trace(b).item() for b in Lb.blocks))


def expval(mps: List[DeviceMPSTensor], mpo, engine_full: Engine, right_end) -> float:
    """<psi|H|psi> without the core energy (``mp_tensors/mps_mpo_ops.h:57-68``)."""
    left = _ones_boundary((0, 0), engine_full.device)
    for i, t in enumerate(mps):
        left = engine_full.overlap_mpo_left_step(t, left, mpo[i])
    host = left.to_host()
    return float(sum(np.trace(b) for b in host[0].blocks))


def run_dmrg(model, mpo, p: SweepParams, nelec: int, twoS: int = 0, mps: Optional[List[DeviceMPSTensor]] = None,
             engine: Optional[Engine] = None, device="cuda", callback=None, precision: int = 0, ts_mpo=None,
             boundary_precision: Optional[int] = None, time_parts: bool = True, checkpoint: Optional[str] = None,
             start_sweep: int = 0, plan_cache: int = 0, ortho_states: Optional[List[List[DeviceMPSTensor]]] = None,
             jd_residual_floor: Optional[float] = None, shadow: Optional[Engine] = None):
    """Two-site sweeps.  ``precision`` selects the sigma-vector form (0 = FP64,
    1 = TF32, 2 = BF16x3 tensor cores); boundary updates, the eigensolver's
    vector algebra, the subspace problem, the truncation (SVD, or the
    density-matrix eigendecomposition with ``twosite_truncation="heev"``) and the
    per-sweep energy stay FP64.  ``boundary_precision`` (default: FP64) selects the form
    of the boundary updates' block products (the boundaries are stored in FP64
    either way).  ``mps`` (right-normalised) replaces the default initial
    state; ``ts_mpo`` is a prebuilt two-site MPO cache (``native.make_ts_cache_fmpo``, or
    ``mpo.make_ts_cache_mpo``); by default the native builder makes it.
    ``time_parts`` synchronises the device after each part of a microiteration to
    time it (``SweepRecord.seconds``); without it the device finishes one
    microiteration's boundary update while the host builds the next sigma plan.
    ``checkpoint`` (a directory) saves the MPS and the sweep status after every
    sweep (``sim.hpp:197-211``); ``start_sweep`` resumes a run at that sweep of
    its schedule (``mps`` from ``checkpoint.load``, sweeps start_sweep..nsweeps-1).
    ``plan_cache`` > 0 keeps that many sigma plans and that many boundary-step plans,
    keyed by their layouts, so a site problem or boundary step whose layouts recur
    in a later sweep reuses its plan.
    ``ortho_states``: device MPSs the state is optimised orthogonal to (excited
    states, ``n_ortho_states`` / ``ortho_states``,
    ``sba/SweepBasedEnergyMinimization.h:52-67``; ``excited.OverlapBoundaries``).
    ``jd_residual_floor``: the eigensolver stops once |r| <= max(tol, floor) |theta|;
    default ``JD_RESIDUAL_FLOOR`` of the sigma precision (0 for FP64: the
    reference's stopping rule unchanged).
    ``shadow`` (an FP64 engine; measurement runs only): at every microiteration also
    evaluate the eigenvector's Rayleigh quotient with FP64 sigma vectors and solve the
    same site problem, from the same start, with the FP64 eigensolver; the three
    energies go to ``SweepRecord.shadow`` as (Ritz value, FP64 Rayleigh quotient of
    the eigenvector, FP64 eigenvalue), without changing the sweep."""
    L = model.L
    phys = model.phys
    engine = engine or Engine(device, precision=precision)
    floor = JD_RESIDUAL_FLOOR.get(engine.precision, 0.0) if jd_residual_floor is None else jd_residual_floor
    jd_tol = max(p.ietl_jcd_tol, floor)
    if plan_cache > 0:
        engine.plan_cache_size = plan_cache
        engine.boundary_plan_cache_size = plan_cache
    engine_full = Engine(device, hermitian=False)
    bprec = 0 if boundary_precision is None else boundary_precision
    # SU2U1: the target (N, 2S); abelian models carry theirs ((N_up, N_down) or (N, 0))
    sym = N.symmetry_code(getattr(model, "symmetry", "su2u1"))
    right_end = model.right_end if sym != N.SYM_SU2U1 else (nelec, twoS)
    if mps is None:
        mps = default_mps_init(L, phys, right_end, p.init_bond_dimension, p.seed, device,
                               abelian=sym != N.SYM_SU2U1)
        normalize_right(mps)
    if ts_mpo is None:
        ts_mpo = N.make_ts_cache_fmpo(mpo, phys)
    left: List = [None] * (L + 1)
    right: List = [None] * (L + 1)
    left[0] = _ones_boundary((0, 0), engine.device)
    right[L] = _ones_boundary(right_end, engine.device)
    for i in range(L - 1, 0, -1):
        right[i] = engine.overlap_mpo_right_step(mps[i], right[i + 1], mpo[i], precision=bprec)
    ovl = OverlapBoundaries(mps, ortho_states, right_end) if ortho_states else None
    rec = SweepRecord()
    nmicro = 2 * (L - 2) if L > 2 else 1
    for sweep in range(start_sweep, p.nsweeps):
        t0 = time.time()
        Mmax = get_Mmax(p, sweep)
        cutoff = get_cutoff(p, sweep)
        for mi in range(nmicro):
            site = mi if mi < L - 1 else 2 * L - 4 - mi
            forward = mi < L - 1
            change = (mi == L - 2) or (mi == nmicro - 1)
            l2r = forward and not change
            tp0 = engine.plan_seconds
            t_a = time.time()
            psi = O.make_two_site_mps(mps[site], mps[site + 1], sym)
            rec.layout_digests.append(hash((site, tuple(psi.layout.keys), tuple(psi.layout.shapes),
                                            tuple(left[site].layout.keys), tuple(left[site].layout.shapes),
                                            tuple(right[site + 2].layout.keys), tuple(right[site + 2].layout.shapes))))
            sp = SiteProblem(engine, left[site], right[site + 2], ts_mpo[site])
            ortho = ovl.vectors(site, psi) if ovl else None
            theta, u, iters = solve_ietl_jcd(sp, psi, jd_tol, p.ietl_jcd_maxiter, ortho)
            if time_parts:
                torch.cuda.synchronize()
            t_b = time.time()
            rec.energies.append(theta + mpo.core_energy)
            rec.jd_iterations.append(iters)
            rec.sigma_calls += iters
            if shadow is not None:
                sp64 = SiteProblem(shadow, left[site], right[site + 2], ts_mpo[site])
                hu = sp64.apply(u).data
                e_var = float(torch.dot(u.data, hu) / torch.dot(u.data, u.data))
                e64, _, _ = solve_ietl_jcd(sp64, psi, p.ietl_jcd_tol, p.ietl_jcd_maxiter, ortho)
                rec.shadow.append((theta + mpo.core_energy, e_var + mpo.core_energy, e64 + mpo.core_energy))
            if p.twosite_truncation == "svd":
                A, B, tr = O.split(u, mps[site], mps[site + 1], Mmax, cutoff, l2r, symmetry=sym)
            else:
                # SweepMPSUpdater.h:192-203: the pair's left boundary and left site's MPO
                # tensor going right, the right boundary and right site's tensor going left
                bnd, w = (left[site], mpo[site]) if l2r else (right[site + 2], mpo[site + 1])
                A, B, tr = O.split(u, mps[site], mps[site + 1], Mmax, cutoff, l2r, truncation=p.twosite_truncation,
                                   alpha=get_alpha(p, sweep), engine=engine, boundary=bnd, mpo=w, symmetry=sym)
            mps[site], mps[site + 1] = A, B
            if time_parts:
                torch.cuda.synchronize()
            t_c = time.time()
            rec.truncated_weight.append(tr.truncated_weight)
            rec.bond_dimension.append(tr.bond_dimension)
            # mergeUnitaryFactor first (its factorisation waits for the device), then the
            # boundary update, which is launched and left running: without part timing the
            # host goes on to plan the next site problem while the device works
            if l2r:
                if site + 2 < L:
                    mps[site + 1], t = O.left_normalize_and_return(mps[site + 1])
                    mps[site + 2] = O.multiply_from_left(mps[site + 2], t)
                else:
                    mps[site + 1], _ = O.left_normalize_and_return(mps[site + 1])
                left[site + 1] = engine.overlap_mpo_left_step(mps[site], left[site], mpo[site], precision=bprec)
            else:
                if site > 0:
                    mps[site], t = O.right_normalize_and_return(mps[site])
                    mps[site - 1] = O.multiply_from_right(mps[site - 1], t)
                else:
                    mps[site], _ = O.right_normalize_and_return(mps[site])
                right[site + 1] = engine.overlap_mpo_right_step(mps[site + 1], right[site + 2], mpo[site + 1],
                                                                precision=bprec)
            if ovl:
                # SweepBasedEnergyMinimization::propagateOtherTensors
                if l2r:
                    ovl.update_left(site + 1)
                else:
                    ovl.update_right(site + 1)
            if time_parts:
                torch.cuda.synchronize()
            t_d = time.time()
            rec.seconds["eigensolver"] += t_b - t_a
            rec.seconds["truncation"] += t_c - t_b
            rec.seconds["boundary"] += t_d - t_c
            rec.seconds["plans"] += engine.plan_seconds - tp0
            if callback:
                callback(sweep, mi, rec)
        torch.cuda.synchronize()
        rec.sweep_seconds.append(time.time() - t0)
        rec.plan_hits = engine.plan_hits
        rec.boundary_plan_hits = engine.boundary_plan_hits
        e = expval(mps, mpo, engine_full, right_end) / overlap(mps) + mpo.core_energy
        rec.sweep_energy.append(e)
        rec.sweep_truncated_weight.append(max(rec.truncated_weight[-nmicro:]))
        if checkpoint:
            from .checkpoint import save
            save(checkpoint, mps, status={"sweep": sweep + 1, "energy": e,
                                          "truncated_weight": rec.sweep_truncated_weight[-1]},
                 parameters={k: v for k, v in vars(p).items()})
    return rec, mps


def run_dmrg_single_site(model, mpo, p: SweepParams, nelec: int, twoS: int = 0,
                         mps: Optional[List[DeviceMPSTensor]] = None, engine: Optional[Engine] = None, device="cuda",
                         precision: int = 0, callback=None):
    """Single-site sweeps on the GPU: ``SweepOptimizationTypeTrait<SingleSite>``
    (``sba/SweepOptimizationTypeTrait.h:23-84``) with ``SweepMPSUpdater<SingleSite>``
    (``sba/SweepMPSUpdater.h:32-155``): 2(L-1) microiterations, the local problem on
    one site with L[i], R[i+1] and the single-site MPO tensor (a sigma plan of its
    own), the density-matrix prediction with the sweep's noise alpha
    (``mps_ops.predict_new_state``), the boundary update and the zero-site factor
    merged into the neighbour.  ``precision`` as for ``run_dmrg``."""
    L = model.L
    phys = model.phys
    engine = engine or Engine(device, precision=precision)
    engine_full = Engine(device, hermitian=False)
    # SU2U1: the target (N, 2S); abelian models carry theirs ((N_up, N_down) or (N, 0))
    sym = N.symmetry_code(getattr(model, "symmetry", "su2u1"))
    right_end = model.right_end if sym != N.SYM_SU2U1 else (nelec, twoS)
    if mps is None:
        mps = default_mps_init(L, phys, right_end, p.init_bond_dimension, p.seed, device,
                               abelian=sym != N.SYM_SU2U1)
        normalize_right(mps)
    left: List = [None] * (L + 1)
    right: List = [None] * (L + 1)
    left[0] = _ones_boundary((0, 0), engine.device)
    right[L] = _ones_boundary(right_end, engine.device)
    for i in range(L - 1, 0, -1):
        right[i] = engine.overlap_mpo_right_step(mps[i], right[i + 1], mpo[i])
    rec = SweepRecord()
    nmicro = 1 if L == 1 else (2 if L == 2 else 2 * (L - 1))
    for sweep in range(p.nsweeps):
        t0 = time.time()
        Mmax = get_Mmax(p, sweep)
        cutoff = get_cutoff(p, sweep)
        alpha = get_alpha(p, sweep)
        for mi in range(nmicro):
            site = mi if mi < L else 2 * L - 2 - mi
            forward = mi < L
            change = (mi == L - 1) or (mi == nmicro - 1)
            l2r = forward and not change
            sp = SiteProblem(engine, left[site], right[site + 1], mpo[site])
            theta, u, iters = solve_ietl_jcd(sp, mps[site], p.ietl_jcd_tol, p.ietl_jcd_maxiter)
            rec.energies.append(theta + mpo.core_energy)
            rec.jd_iterations.append(iters)
            rec.sigma_calls += iters
            mps[site] = u
            tr = None
            if l2r and site < L - 1:
                mps[site], zero, tr = O.predict_new_state(u, mpo[site], left[site], right[site + 1], alpha, cutoff,
                                                          Mmax, True, engine)
                left[site + 1] = engine.overlap_mpo_left_step(mps[site], left[site], mpo[site])
                mps[site + 1] = O.multiply_from_left(mps[site + 1], zero)
            elif not l2r and site > 0:
                mps[site], zero, tr = O.predict_new_state(u, mpo[site], left[site], right[site + 1], alpha, cutoff,
                                                          Mmax, False, engine)
                right[site] = engine.overlap_mpo_right_step(mps[site], right[site + 1], mpo[site])
                mps[site - 1] = O.multiply_from_right(mps[site - 1], zero)
            if tr is not None:
                rec.truncated_weight.append(tr.truncated_weight)
                rec.bond_dimension.append(tr.bond_dimension)
            if callback:
                callback(sweep, mi, rec)
        torch.cuda.synchronize()
        rec.sweep_seconds.append(time.time() - t0)
        e = expval(mps, mpo, engine_full, right_end) / overlap(mps) + mpo.core_energy
        rec.sweep_energy.append(e)
        rec.sweep_truncated_weight.append(max(rec.truncated_weight[-(nmicro - 1):] or [0.0]))
    return rec, mps


__all__ = ["SweepParams", "SweepRecord", "run_dmrg", "run_dmrg_single_site", "get_alpha", "default_mps_init", "normalize_right", "expval", "overlap"]
