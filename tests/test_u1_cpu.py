"""The abelian path with U1 charges (symmetry "u1": spin orbitals as sites, charge
(N, 0)) on the CPU.

* The U1 spin-orbital model's MPO, contracted to a dense operator on the 2^(2L)
  Fock space, has in every electron-number sector exactly the lowest eigenvalue
  of exact diagonalisation over all total spins: model and MPO builder are pinned
  independently of any DMRG code.
* The oracle's abelian engine run as a DMRG over the spin-orbital sites
  reproduces FCI and the reference's golden H2 and LiH ground-state energies
  (``dmrg/tests/test1.cpp:93``, ``dmrg/tests/test2.cpp:57``; two electrons).
* The native plans with ``QCM_SYM_U1`` (sigma, both boundary steps, the two-site
  tensor, the split prologue, the two-site MPO builder) give the oracle's layouts
  and values, checked by interpreting the exported task tables; an MPO of an
  unknown group is refused by the planner.
"""
import itertools

import numpy as np
import pytest

from qcmaquis_gb300 import native as N
from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model_u1 import STATES, U1SpinOrbitalModel
from qcmaquis_gb300.mpo import TaggedMPOMaker

from conftest import integral_map
from oracle import abelian as A
from oracle import dmrg_ref as R
from oracle import fci
from oracle import ts_mpo as OTS
from oracle.sweep import SweepParams, initial_state, run_dmrg
from plan_interp import run_plan


def fci_ground(L, ints, nelec):
    """Lowest eigenvalue of the nelec-electron space over every total spin."""
    return min(e for twoS in range(nelec % 2, nelec + 1, 2) for e in fci.fci_energies(L, ints, nelec, twoS, 1))


def _dense_hamiltonian(mpo):
    """The MPO as a dense operator on the 2^sites product basis (site 0 most significant)."""
    def dense(op):
        m = np.zeros((2, 2))
        for (i, o), b in zip(op.bm.keys, op.bm.blocks):
            m[STATES.index(o), STATES.index(i)] = b[0, 0]
        return m
    T = [np.eye(1)]
    for W in mpo:
        nxt = [np.zeros((T[0].shape[0] * 2,) * 2) for _ in range(W.col_dim)]
        for b2 in range(W.col_dim):
            for b1 in W.column(b2):
                for tag, sc in W.at(b1, b2):
                    nxt[b2] += sc * np.kron(T[b1], dense(W.op(tag)))
        T = nxt
    return T[0] + mpo.core_energy * np.eye(T[0].shape[0])


@pytest.mark.parametrize("merge", [True, False])
def test_u1_mpo_has_the_fci_spectrum(merge):
    L = 3
    ints = synthetic_integral_map(L, seed=3)
    model = U1SpinOrbitalModel(L, ints, 3)
    mpo = TaggedMPOMaker(model, merge_site_terms=merge).create_mpo()
    assert len(mpo) == 2 * L and all(w.symmetry == "u1" for w in mpo)
    H = _dense_hamiltonian(mpo)
    assert np.abs(H - H.T).max() < 1e-13
    n = np.array([sum(STATES[s][0] for s in st) for st in itertools.product(range(2), repeat=2 * L)])
    for ne in range(1, 2 * L):
        sel = n == ne
        got = np.linalg.eigvalsh(H[np.ix_(sel, sel)])[0]
        assert abs(got - fci_ground(L, ints, ne)) < 1e-10, ne


@pytest.mark.parametrize("L,ne", [(3, 4), (4, 3)])
def test_oracle_u1_dmrg_equals_fci(L, ne):
    ints = synthetic_integral_map(L, seed=3)
    model = U1SpinOrbitalModel(L, ints, ne)
    mpo = TaggedMPOMaker(model).create_mpo()
    p = SweepParams(nsweeps=3, max_bond_dimension=64, init_bond_dimension=8, ietl_jcd_tol=1e-10,
                    ietl_jcd_maxiter=20)
    rec, _ = run_dmrg(model, mpo, p, ne)
    assert abs(rec.sweep_energy[-1] - fci_ground(L, ints, ne)) < 1e-9


@pytest.mark.parametrize("name", ["h2", "lih"])
def test_oracle_u1_reproduces_the_reference_golden_energy(golden, name):
    g = golden[name]
    model = U1SpinOrbitalModel(g["L"], integral_map(g["integrals"]), 2)
    mpo = TaggedMPOMaker(model).create_mpo()
    rec, _ = run_dmrg(model, mpo, SweepParams(nsweeps=3, max_bond_dimension=100, init_bond_dimension=8,
                                              ietl_jcd_tol=1e-10, ietl_jcd_maxiter=20), 2)
    assert abs(rec.sweep_energy[-1] - g["energy"]) <= 1e-9 * abs(g["energy"])


def _u1_problem(L=4, ne=4, m=12, site=3, herm=True, seed=3):
    """A random right-normalised U1 MPS (2L spin-orbital sites) with the oracle's
    boundaries around (site, site+1)."""
    ints = synthetic_integral_map(L, seed=seed)
    model = U1SpinOrbitalModel(L, ints, ne)
    mpo = TaggedMPOMaker(model).create_mpo()
    mps = initial_state(model, mpo, SweepParams(init_bond_dimension=m, seed=11), ne, 0)
    left = R.left_boundary(mps[0])
    for i in range(site):
        t = R.left_normalize_and_return(mps[i])
        R.multiply_from_left(mps[i + 1], t)
        left = A.overlap_mpo_left_step(mps[i], mps[i], left, mpo[i], is_hermitian=herm)
    right = R.right_boundary(mps[model.L - 1])
    for i in range(model.L - 1, site + 1, -1):
        right = A.overlap_mpo_right_step(mps[i], mps[i], right, mpo[i], is_hermitian=herm)
    return model, mpo, mps, left, right


def test_native_twosite_mpo_is_the_abelian_product():
    model, mpo, mps, left, right = _u1_problem()
    f = N.make_twosite_fmpo(N.FMpo(mpo[3]), N.FMpo(mpo[4]), model.phys)
    fk = N.make_twosite_fmpo(N.FMpo(mpo[3]), N.FMpo(mpo[4]), model.phys, native_kron=True)
    assert f.symmetry == N.SYM_U1 and fk.symmetry == N.SYM_U1
    assert np.array_equal(f.ent_coeff, fk.ent_coeff) and np.array_equal(f.blk_q, fk.blk_q)
    # every charge is (N, 0)
    assert np.all(f.blk_q.reshape(-1, 4)[:, [1, 3]] == 0)
    ots = OTS.make_twosite_mpo(mpo[3], mpo[4], model.phys, model.phys)
    assert ots.symmetry == "u1"
    psi = A.make_two_site_mps(mps[3], mps[4]).make_left_paired()
    lay = N.Layout.of(psi.data)
    Ll, Rl = N.BoundaryLayout.of(left), N.BoundaryLayout.of(right)
    p = N.plan_sigma(psi.phys_i, psi.left_i, psi.right_i, lay, Ll, Rl, f, True)
    bufs = [lay.pack(psi.data), Ll.pack(left), Rl.pack(right), np.zeros(p.out_elems)] + \
        [np.full(max(s, 1), np.nan) for s in p.scratch]
    run_plan(p, bufs)
    ref = lay.pack(A.site_hamil2(psi, left, right, ots).data)
    assert np.linalg.norm(bufs[3] - ref) <= 1e-13 * np.linalg.norm(ref)


@pytest.mark.parametrize("herm", [True, False])
@pytest.mark.parametrize("site,m", [(1, 8), (3, 12), (5, 10)])
def test_u1_sigma_plan_matches_oracle(herm, site, m):
    model, mpo, mps, left, right = _u1_problem(site=site, m=m, herm=herm)
    ts = N.make_twosite_fmpo(N.FMpo(mpo[site]), N.FMpo(mpo[site + 1]), model.phys)
    ots = OTS.make_twosite_mpo(mpo[site], mpo[site + 1], model.phys, model.phys)
    psi = A.make_two_site_mps(mps[site], mps[site + 1]).make_left_paired()
    lay = N.Layout.of(psi.data)
    Ll, Rl = N.BoundaryLayout.of(left), N.BoundaryLayout.of(right)
    p = N.plan_sigma(psi.phys_i, psi.left_i, psi.right_i, lay, Ll, Rl, ts, herm)
    bufs = [lay.pack(psi.data), Ll.pack(left), Rl.pack(right), np.zeros(p.out_elems)] + \
        [np.full(max(s, 1), np.nan) for s in p.scratch]
    run_plan(p, bufs)
    ref = lay.pack(A.site_hamil2(psi, left, right, ots, is_hermitian=herm).data)
    assert np.linalg.norm(bufs[3] - ref) <= 1e-13 * np.linalg.norm(ref)


@pytest.mark.parametrize("herm", [True, False])
def test_u1_boundary_plans_match_oracle(herm):
    L, ne = 4, 4
    model = U1SpinOrbitalModel(L, synthetic_integral_map(L, seed=3), ne)
    mpo = TaggedMPOMaker(model).create_mpo()
    mps = initial_state(model, mpo, SweepParams(init_bond_dimension=12, seed=11), ne, 0)
    left = R.left_boundary(mps[0])
    for i in range(4):
        T = mps[i].copy().make_left_paired()
        lay, Ll = N.Layout.of(T.data), N.BoundaryLayout.of(left)
        p = N.plan_boundary_left(T.phys_i, T.left_i, T.right_i, lay, Ll, N.FMpo(mpo[i]), herm)
        ol = p.out_layout()
        bufs = [lay.pack(T.data), Ll.pack(left), None, np.zeros(max(p.out_elems, 1))] + \
            [np.zeros(max(s, 1)) for s in p.scratch]
        run_plan(p, bufs)
        ref = A.overlap_mpo_left_step(mps[i], mps[i], left, mpo[i], herm)
        assert [g.keys for g in ol.unpack(bufs[3])] == [r.keys for r in ref]
        assert np.allclose(ol.pack(ref), bufs[3][:ol.size], rtol=0, atol=1e-13)
        left = ref
    right = R.right_boundary(mps[model.L - 1])
    for i in range(model.L - 1, 3, -1):
        T = mps[i].copy().make_left_paired()
        lay, Rl = N.Layout.of(T.data), N.BoundaryLayout.of(right)
        p = N.plan_boundary_right(T.phys_i, T.left_i, T.right_i, lay, Rl, N.FMpo(mpo[i]), herm)
        ol = p.out_layout()
        bufs = [lay.pack(T.data), None, Rl.pack(right), np.zeros(max(p.out_elems, 1))] + \
            [np.zeros(max(s, 1)) for s in p.scratch]
        run_plan(p, bufs)
        ref = A.overlap_mpo_right_step(mps[i], mps[i], right, mpo[i], herm)
        assert [g.keys for g in ol.unpack(bufs[3])] == [r.keys for r in ref]
        assert np.allclose(ol.pack(ref), bufs[3][:ol.size], rtol=0, atol=1e-13)
        right = ref


def _run(plan, slots):
    bufs = [None] * 8
    for k, v in slots.items():
        bufs[k] = v
    bufs[3] = np.full(max(plan.out_elems, 1), np.nan)
    for i, s in enumerate(plan.scratch):
        bufs[4 + i] = np.full(max(s, 1), np.nan)
    run_plan(plan, bufs)
    return bufs


@pytest.mark.parametrize("site", [0, 3, 6])
def test_u1_two_site_and_split_plans_match_oracle(site):
    model, mpo, mps, _, _ = _u1_problem(site=site)
    Ta = mps[site].copy().make_left_paired()
    Tb = mps[site + 1].copy().make_left_paired()
    la, lb = N.Layout.of(Ta.data), N.Layout.of(Tb.data)
    p = N.plan_two_site(Ta.phys_i, Ta.left_i, Ta.right_i, la, Tb.phys_i, Tb.left_i, Tb.right_i, lb, N.SYM_U1)
    ref = A.make_two_site_mps(mps[site], mps[site + 1]).make_left_paired()
    phys, left, right, lay = N.out_tensor(p)
    assert phys == ref.phys_i
    assert list(lay.keys) == list(ref.data.keys)
    bufs = _run(p, {0: la.pack(Ta.data), 1: lb.pack(Tb.data)})
    want = lay.pack(ref.data)
    assert np.linalg.norm(bufs[3][:lay.size] - want) <= 1e-13 * np.linalg.norm(want)
    A0, B0 = mps[site], mps[site + 1]
    sp = N.plan_split_theta(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, lay, N.SYM_U1)
    both = R._reshape_left_to_both(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, ref.data)
    _, _, _, blay = N.out_tensor(sp)
    assert list(blay.keys) == list(both.keys)
    out = _run(sp, {0: want})
    wb = blay.pack(both)
    assert np.linalg.norm(out[3][:blay.size] - wb) <= 1e-13 * np.linalg.norm(wb)


def test_mpo_of_unknown_group_is_refused_by_the_planner():
    model, mpo, mps, left, right = _u1_problem()
    f = N.FMpo(mpo[3])
    f.symmetry = 7
    f._make_c()
    T = mps[3].copy().make_left_paired()
    lay, Ll = N.Layout.of(T.data), N.BoundaryLayout.of(left)
    with pytest.raises(RuntimeError, match="unknown symmetry"):
        N.plan_boundary_left(T.phys_i, T.left_i, T.right_i, lay, Ll, f, True)
