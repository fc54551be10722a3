"""Two-site ground-state sweep of the oracle (tests only).

Restates the live sweep driver: ``SweepBasedEnergyMinimization`` over
``GenericSweepSimulation::runSingleSweep``
(``sba/GenericSweepSimulation.h:73-152, 212-268``), the microiteration
schedule of ``SweepOptimizationTypeTrait<TwoSite>``
(``sba/SweepOptimizationTypeTrait.h:85-142``), the boundary bookkeeping of
``BoundaryPropagator`` (``sba/BoundaryPropagator.h:36-150``) and the
truncate/merge steps of ``SweepMPSUpdater<TwoSite>``
(``sba/SweepMPSUpdater.h:180-258``).  Energies follow ``get_energy``
(``fw/sim/interface_sim.h:355-360``): <psi|H|psi>/<psi|psi> + core energy.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field
from typing import Dict, List, Optional

import numpy as np

from .ts_mpo import make_ts_cache_mpo

from . import abelian as A
from . import dmrg_ref as R


def _abelian(model_or_mpo) -> bool:
    """TwoU1 and U1 models and their MPO tensors carry symmetry "2u1" / "u1"."""
    return getattr(model_or_mpo, "symmetry", "su2u1") != "su2u1"


def _engine(abelian: bool):
    """The contraction functions of the group: the abelian engine or the SU(2) one."""
    return A if abelian else R


@dataclass
class SweepParams:
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
    # truncation mode and noise schedule (``fw/utils/DmrgParameters.h:45-59``)
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


def log_interpolate(y0, y1, N, i):
    if N < 2:
        return y1
    if y0 == 0:
        return 0.0
    x = math.log(y1 / y0) / (N - 1)
    return y0 * math.exp(x * i)


def get_cutoff(p: SweepParams, sweep: int) -> float:
    if sweep >= p.ngrowsweeps:
        return p.truncation_final
    return log_interpolate(p.truncation_initial, p.truncation_final, p.ngrowsweeps, sweep)


def get_Mmax(p: SweepParams, sweep: int) -> int:
    if p.sweep_bond_dimensions:
        return p.sweep_bond_dimensions[min(sweep, len(p.sweep_bond_dimensions) - 1)]
    return p.max_bond_dimension


@dataclass
class SweepRecord:
    energies: List[float] = field(default_factory=list)
    truncated_weight: List[float] = field(default_factory=list)
    bond_dimension: List[int] = field(default_factory=list)
    sweep_energy: List[float] = field(default_factory=list)
    sweep_truncated_weight: List[float] = field(default_factory=list)


def expval(mps: List[R.MPSTensor], mpo) -> float:
    """``expval`` (``mp_tensors/mps_mpo_ops.h:57-68``) without the core energy."""
    E = _engine(_abelian(mpo[0]))
    left = R.left_boundary(mps[0])
    for i in range(len(mps)):
        left = E.overlap_mpo_left_step(mps[i], mps[i], left, mpo[i], is_hermitian=False)
    return sum(b.trace() for b in left[:1])


def overlap(mps: List[R.MPSTensor]) -> float:
    """<psi|psi> through the plain overlap steps."""
    left = R.left_boundary(mps[0])[0]
    for t in mps:
        a = t.copy().make_left_paired()
        # left^T-contracted transfer: L' = A^T (L (x) 1) A for a real MPS
        rp = t.copy().make_right_paired()
        t1 = R.bm_gemm(left, rp.data)
        t3 = R.reshape_right_to_left(t.phys_i, t.left_i, t.right_i, t1)
        left = R.bm_gemm(a.data.transpose(), t3)
    return left.trace()


def initial_state(model, mpo, p: SweepParams, nelec: int, twoS: int):
    """The random right-normalised start; SU2U1 targets (nelec, twoS), a TwoU1 model
    its own (N_up, N_down)."""
    phys = model.phys
    ab = _abelian(model)
    right_end = model.right_end if ab else (nelec, twoS)
    mps = R.default_mps_init(model.L, phys, right_end, p.init_bond_dimension, p.seed, abelian=ab)
    R.normalize_right(mps)
    return mps


class OverlapBoundaries:
    """``OverlapPropagator`` (``sba/OverlapPropagator.h``): per orthogonal state n the
    MPO-free left and right overlap boundaries <psi|phi_n> of the current state
    ``mps`` (bra) with phi_n (ket), started at site 0 (the right ones all built)."""

    def __init__(self, mps: List[R.MPSTensor], others: List[List[R.MPSTensor]]):
        L = len(mps)
        self.mps, self.others = mps, others
        self.left = [[None] * (L + 1) for _ in others]
        self.right = [[None] * (L + 1) for _ in others]
        for n in range(len(others)):
            self.left[n][0] = R.left_boundary(mps[0])[0]
            self.right[n][L] = R.right_boundary(mps[L - 1])[0]
            for i in range(L - 1, 0, -1):
                self.update_right(i, n)

    def update_left(self, i: int, only=None):
        for n in (range(len(self.others)) if only is None else [only]):
            self.left[n][i] = R.overlap_left_step(self.mps[i - 1], self.others[n][i - 1], self.left[n][i - 1])

    def update_right(self, i: int, only=None):
        for n in (range(len(self.others)) if only is None else [only]):
            self.right[n][i] = R.overlap_right_step(self.mps[i], self.others[n][i], self.right[n][i + 1])

    def vectors(self, site: int, psi: R.MPSTensor) -> List[R.MPSTensor]:
        """``getOrthogonalVector`` of every state for the two-site problem at (site, site + 1)."""
        out = []
        for n, phi in enumerate(self.others):
            theta = R.make_two_site_mps(phi[site], phi[site + 1])
            out.append(R.site_ortho_boundaries(psi, theta, self.left[n][site], self.right[n][site + 2]))
        return out


def run_dmrg(model, mpo, p: SweepParams, nelec: int, twoS: int = 0, mps=None,
             callback=None, ortho_states=None) -> (SweepRecord, List[R.MPSTensor]):
    """Two-site sweeps; ``ortho_states``: MPSs the state is optimised orthogonal to
    (``n_ortho_states`` / ``ortho_states``, ``sba/SweepBasedEnergyMinimization.h:52-67``)."""
    L = model.L
    phys = model.phys
    ab = _abelian(model)
    E = _engine(ab)
    if ab and ortho_states:
        raise ValueError("orthogonal states are implemented for SU2U1 only")
    if mps is None:
        mps = initial_state(model, mpo, p, nelec, twoS)
    ts_mpo = make_ts_cache_mpo(mpo, phys)
    ovl = OverlapBoundaries(mps, list(ortho_states)) if ortho_states else None
    left: List = [None] * (L + 1)
    right: List = [None] * (L + 1)
    left[0] = R.left_boundary(mps[0])
    right[L] = R.right_boundary(mps[L - 1])
    for i in range(L - 1, 0, -1):
        right[i] = E.overlap_mpo_right_step(mps[i], mps[i], right[i + 1], mpo[i])
    rec = SweepRecord()
    nmicro = 2 * (L - 2) if L > 2 else 1
    for sweep in range(p.nsweeps):
        Mmax = get_Mmax(p, sweep)
        cutoff = get_cutoff(p, sweep)
        for mi in range(nmicro):
            site = mi if mi < L - 1 else 2 * L - 4 - mi
            forward = mi < L - 1
            change = (mi == L - 2) or (mi == nmicro - 1)
            l2r = forward and not change
            ts = ts_mpo[site]
            psi = E.make_two_site_mps(mps[site], mps[site + 1])

            def apply_h(x, _l=left[site], _r=right[site + 2], _w=ts):
                return E.site_hamil2(x, _l, _r, _w)

            ortho = ovl.vectors(site, psi) if ovl else None
            theta, u, iters = R.jcd_solve(apply_h, psi, p.ietl_jcd_tol, p.ietl_jcd_maxiter, ortho)
            rec.energies.append(theta + mpo.core_energy)
            u.make_left_paired()
            A0, B0 = mps[site], mps[site + 1]
            if ab:
                tst = u.data
            else:
                _, tst = R.unreduce_left(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, u.data)
            if p.twosite_truncation == "svd":
                A, B, trunc = R.split_mps(tst, A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, Mmax, cutoff, l2r)
            else:
                # sba/SweepMPSUpdater.h:192-203: left boundary of the pair and the left
                # site's MPO tensor going right; right boundary and right site going left
                bnd, w = (left[site], mpo[site]) if l2r else (right[site + 2], mpo[site + 1])
                A, B, trunc = R.predict_split_mps(tst, A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, Mmax, cutoff,
                                                  l2r, get_alpha(p, sweep), bnd, w)
            mps[site], mps[site + 1] = A, B
            rec.truncated_weight.append(trunc.truncated_weight)
            rec.bond_dimension.append(trunc.bond_dimension)
            if l2r:
                left[site + 1] = E.overlap_mpo_left_step(mps[site], mps[site], left[site], mpo[site])
            else:
                right[site + 1] = E.overlap_mpo_right_step(mps[site + 1], mps[site + 1], right[site + 2],
                                                           mpo[site + 1])
            if ovl:
                # SweepBasedEnergyMinimization::propagateOtherTensors
                if l2r:
                    ovl.update_left(site + 1)
                else:
                    ovl.update_right(site + 1)
            if l2r:
                if site + 2 < L:
                    t = R.left_normalize_and_return(mps[site + 1])
                    R.multiply_from_left(mps[site + 2], t)
                else:
                    R.left_normalize_and_return(mps[site + 1])
            else:
                if site > 0:
                    t = R.right_normalize_and_return(mps[site])
                    R.multiply_from_right(mps[site - 1], t)
                else:
                    R.right_normalize_and_return(mps[site])
            if callback:
                callback(sweep, mi, rec)
        e = expval(mps, mpo) / overlap(mps) + mpo.core_energy
        rec.sweep_energy.append(e)
        rec.sweep_truncated_weight.append(max(rec.truncated_weight[-nmicro:]))
    return rec, mps


def run_dmrg_single_site(model, mpo, p: SweepParams, nelec: int, twoS: int = 0, mps=None,
                         callback=None) -> (SweepRecord, List[R.MPSTensor]):
    """Single-site sweeps: ``SweepOptimizationTypeTrait<SingleSite>``
    (``sba/SweepOptimizationTypeTrait.h:23-84``: 2(L-1) microiterations, site i going
    right and 2L-2-i going left) with ``SweepMPSUpdater<SingleSite>``
    (``sba/SweepMPSUpdater.h:32-155``): the local problem on one site with L[i],
    R[i+1] and the site's MPO tensor, the density-matrix prediction with the
    sweep's noise alpha (``R.predict_new_state``), the boundary update, and the
    zero-site factor merged into the neighbour."""
    L = model.L
    if mps is None:
        mps = initial_state(model, mpo, p, nelec, twoS)
    left: List = [None] * (L + 1)
    right: List = [None] * (L + 1)
    left[0] = R.left_boundary(mps[0])
    right[L] = R.right_boundary(mps[L - 1])
    for i in range(L - 1, 0, -1):
        right[i] = R.overlap_mpo_right_step(mps[i], mps[i], right[i + 1], mpo[i])
    rec = SweepRecord()
    nmicro = 1 if L == 1 else (2 if L == 2 else 2 * (L - 1))
    for sweep in range(p.nsweeps):
        Mmax = get_Mmax(p, sweep)
        cutoff = get_cutoff(p, sweep)
        alpha = get_alpha(p, sweep)
        for mi in range(nmicro):
            site = mi if mi < L else 2 * L - 2 - mi
            forward = mi < L
            change = (mi == L - 1) or (mi == nmicro - 1)
            l2r = forward and not change

            def apply_h(x, _l=left[site], _r=right[site + 1], _w=mpo[site]):
                return R.site_hamil2(x, _l, _r, _w)

            theta, u, iters = R.jcd_solve(apply_h, mps[site], p.ietl_jcd_tol, p.ietl_jcd_maxiter)
            rec.energies.append(theta + mpo.core_energy)
            mps[site] = u
            if l2r and site < L - 1:
                new, zero, trunc = R.predict_new_state(u, mpo[site], left[site], right[site + 1], alpha, cutoff,
                                                       Mmax, True)
                mps[site] = new
                left[site + 1] = R.overlap_mpo_left_step(mps[site], mps[site], left[site], mpo[site])
                R.multiply_from_left(mps[site + 1], zero)
            elif not l2r and site > 0:
                new, zero, trunc = R.predict_new_state(u, mpo[site], left[site], right[site + 1], alpha, cutoff,
                                                       Mmax, False)
                mps[site] = new
                right[site] = R.overlap_mpo_right_step(mps[site], mps[site], right[site + 1], mpo[site])
                R.multiply_from_right(mps[site - 1], zero)
            else:
                trunc = None
            if trunc is not None:
                rec.truncated_weight.append(trunc.truncated_weight)
                rec.bond_dimension.append(trunc.bond_dimension)
            if callback:
                callback(sweep, mi, rec)
        e = expval(mps, mpo) / overlap(mps) + mpo.core_energy
        rec.sweep_energy.append(e)
        rec.sweep_truncated_weight.append(max(rec.truncated_weight[-(nmicro - 1):] or [0.0]))
    return rec, mps
