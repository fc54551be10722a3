"""The MPS-level plans (two-site tensor, split prologue, split assembly) against the
oracle, executed by the host-side task-table interpreter (no GPU).

* ``qcm_plan_two_site`` = ``TwoSiteTensor(mps1, mps2)`` + ``make_mps``
  (``mt/twositetensor.hpp:22-31, 132-139``; oracle ``make_two_site_mps``);
* ``qcm_plan_split_theta`` = ``unreduce_left`` + ``reshape_left_to_both``
  (``mt/ts_reduction.h:143-251``, ``mt/ts_reshape.h:89-145``);
* ``qcm_plan_split_assemble`` = the epilogue of ``split_mps_l2r/r2l``
  (``mt/twositetensor.hpp:141-180``) on the same SVD factors the oracle uses.

Layouts must be equal block for block and indices equal; values to 1e-13
relative (sums of at most two 6j-scaled terms per element)."""
import numpy as np
import pytest

from qcmaquis_gb300 import native as N
from oracle import dmrg_ref as R
from oracle.sweep import SweepParams, initial_state
from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model import QCModel
from qcmaquis_gb300.mpo import make_mpo

from plan_interp import run_plan


def _mps(L=6, N_=6, m=16, seed=3):
    model = QCModel(L, synthetic_integral_map(L, seed=seed), N_)
    mpo = make_mpo(model)
    return model, initial_state(model, mpo, SweepParams(init_bond_dimension=m, seed=11), N_, 0)


def _run(plan, inputs):
    bufs = [np.full(max(plan.out_elems, 1), np.nan) if i == 3 else None for i in range(8)]
    for slot, arr in inputs.items():
        bufs[slot] = arr
    for i, s in enumerate(plan.scratch):
        bufs[4 + i] = np.full(max(s, 1), np.nan)
    run_plan(plan, bufs)
    return bufs


def _same_layout(lay, bm):
    assert list(lay.keys) == list(bm.keys)
    assert list(lay.shapes) == [b.shape for b in bm.blocks]


@pytest.mark.parametrize("L,N_,m,site", [(6, 6, 16, 2), (6, 6, 16, 0), (6, 6, 16, 4), (5, 4, 12, 1), (4, 2, 8, 2)])
def test_two_site_plan_matches_oracle(L, N_, m, site):
    model, mps = _mps(L, N_, m)
    A = mps[site].copy().make_left_paired()
    B = mps[site + 1].copy().make_left_paired()
    la, lb = N.Layout.of(A.data), N.Layout.of(B.data)
    p = N.plan_two_site(A.phys_i, A.left_i, A.right_i, la, B.phys_i, B.left_i, B.right_i, lb)
    ref = R.make_two_site_mps(mps[site], mps[site + 1]).make_left_paired()
    phys, left, right, lay = N.out_tensor(p)
    assert phys == ref.phys_i and left == ref.left_i and right == ref.right_i
    _same_layout(lay, ref.data)
    bufs = _run(p, {0: la.pack(A.data), 1: lb.pack(B.data)})
    want = lay.pack(ref.data)
    got = bufs[3][:lay.size]
    assert np.all(np.isfinite(got))
    assert np.linalg.norm(got - want) <= 1e-13 * np.linalg.norm(want)


@pytest.mark.parametrize("site", [0, 1, 2, 4])
def test_split_theta_plan_matches_oracle(site):
    model, mps = _mps()
    psi = R.make_two_site_mps(mps[site], mps[site + 1]).make_left_paired()
    A0, B0 = mps[site], mps[site + 1]
    lu = N.Layout.of(psi.data)
    p = N.plan_split_theta(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, lu)
    _, tst = R.unreduce_left(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, psi.data)
    both = R._reshape_left_to_both(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, tst)
    _, _, _, lay = N.out_tensor(p)
    _same_layout(lay, both)
    bufs = _run(p, {0: lu.pack(psi.data)})
    want = lay.pack(both)
    assert np.linalg.norm(bufs[3][:lay.size] - want) <= 1e-13 * np.linalg.norm(want)


@pytest.mark.parametrize("l2r", [True, False])
@pytest.mark.parametrize("Mmax", [6, 40])
def test_split_assembly_matches_oracle(l2r, Mmax):
    model, mps = _mps(m=24)
    site = 2
    psi = R.make_two_site_mps(mps[site], mps[site + 1]).make_left_paired()
    A0, B0 = mps[site], mps[site + 1]
    lu = N.Layout.of(psi.data)
    sp = N.plan_split_theta(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, lu)
    _, _, _, lay = N.out_tensor(sp)
    theta = _run(sp, {0: lu.pack(psi.data)})[3]
    # the SVD factors, packed the way qcm_svd writes them (U: rows x k, S, Vt: k x cols)
    U, S, Vt, u_off, s_off, vt_off, svals = [], [], [], [], [], [], []
    uo = so = vo = 0
    for (r, c), o in zip(lay.shapes, lay.offsets):
        u, s, vt = np.linalg.svd(theta[o:o + r * c].reshape((c, r)).T, full_matrices=False)
        u_off.append(uo); s_off.append(so); vt_off.append(vo)
        U.append(u.ravel(order="F")); S.append(s); Vt.append(vt.ravel(order="F"))
        uo += u.size; so += s.size; vo += vt.size
        svals.append(s)
    Uf, Sf, Vtf = np.concatenate(U), np.concatenate(S), np.concatenate(Vt)
    allv = np.sort(Sf)[::-1]
    cut = max(1e-16 * allv[0], allv[Mmax] if allv.size > Mmax else 0.0)
    keep = [int(np.sum(s >= cut)) for s in svals]
    ap = N.plan_split_assemble(sp, u_off, vt_off, keep, Sf, s_off, l2r)
    bufs = _run(ap, {0: Uf, 1: Vtf})
    tst = R.unreduce_left(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, psi.data)[1]
    Ar, Br, tr = R.split_mps(tst, A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, Mmax, 1e-16, l2r)
    assert sum(keep) == tr.bond_dimension
    Ar, Br = Ar.make_left_paired(), Br.make_left_paired()
    for which, ref, buf in ((0, Ar, bufs[3]), (1, Br, bufs[6])):
        phys, left, right, ol = N.out_tensor(ap, which)
        assert phys == ref.phys_i and left == ref.left_i and right == ref.right_i, which
        _same_layout(ol, ref.data)
        want = ol.pack(ref.data)
        assert np.linalg.norm(buf[:ol.size] - want) <= 1e-13 * np.linalg.norm(want), which


# ``qcm_plan_mps_multiply`` / ``qcm_plan_mps_reshape``: the two halves of
# mergeUnitaryFactor (``sba/SweepMPSUpdater.h:237-250``) against the oracle's
# ``multiply_from_left`` / ``multiply_from_right`` (``mt/mpstensor.hpp:302-321``)
# and its reshapes, on the oracle's own QR / LQ factors.
@pytest.mark.parametrize("site", [0, 2, 3])
def test_multiply_from_left_plan_matches_oracle(site):
    model, mps = _mps()
    A = mps[site].copy()
    t = R.left_normalize_and_return(A)
    T = mps[site + 1].copy().make_left_paired()
    lt, ln = N.Layout.of(T.data), N.Layout.of(t)
    p = N.plan_mps_multiply(T.phys_i, T.left_i, T.right_i, lt, ln, True)
    ref = T.copy()
    R.multiply_from_left(ref, t)
    ref.make_left_paired()
    phys, left, right, lay = N.out_tensor(p)
    assert phys == ref.phys_i and left == ref.left_i and right == ref.right_i
    _same_layout(lay, ref.data)
    bufs = _run(p, {0: lt.pack(T.data), 1: ln.pack(t)})
    want = lay.pack(ref.data)
    assert np.linalg.norm(bufs[3][:lay.size] - want) <= 1e-13 * np.linalg.norm(want)


@pytest.mark.parametrize("site", [1, 3, 5])
def test_multiply_from_right_plan_matches_oracle(site):
    model, mps = _mps()
    B = mps[site].copy()
    lm = R.right_normalize_and_return(B)
    T = mps[site - 1].copy().make_left_paired()
    lt, ln = N.Layout.of(T.data), N.Layout.of(lm)
    p = N.plan_mps_multiply(T.phys_i, T.left_i, T.right_i, lt, ln, False)
    ref = T.copy()
    R.multiply_from_right(ref, lm)
    ref.make_left_paired()
    phys, left, right, lay = N.out_tensor(p)
    assert phys == ref.phys_i and left == ref.left_i and right == ref.right_i
    _same_layout(lay, ref.data)
    bufs = _run(p, {0: lt.pack(T.data), 1: ln.pack(lm)})
    want = lay.pack(ref.data)
    assert np.linalg.norm(bufs[3][:lay.size] - want) <= 1e-13 * np.linalg.norm(want)


@pytest.mark.parametrize("site", [0, 2, 5])
def test_reshape_plans_match_oracle(site):
    model, mps = _mps()
    T = mps[site].copy().make_left_paired()
    lt = N.Layout.of(T.data)
    rp = T.copy().make_right_paired()
    p = N.plan_mps_reshape(T.phys_i, T.left_i, T.right_i, lt, True)
    _, _, _, lay = N.out_tensor(p)
    _same_layout(lay, rp.data)
    got = _run(p, {0: lt.pack(T.data)})[3][:lay.size]
    assert np.array_equal(got, lay.pack(rp.data))
    back = N.plan_mps_reshape(T.phys_i, T.left_i, T.right_i, lay, False)
    _, _, _, lay2 = N.out_tensor(back)
    _same_layout(lay2, T.data)
    assert np.array_equal(_run(back, {0: got})[3][:lay2.size], lt.pack(T.data))
