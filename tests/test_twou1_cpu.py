"""The abelian TwoU1 path on the CPU (symmetry "2u1": charges (N_up, N_down)).

* The TwoU1 model's MPO, contracted to a dense operator, has exactly the
  exact-diagonalisation spectrum in every (N_up, N_down) sector: the model
  and the MPO builder are pinned independently of any DMRG code.
* The oracle's abelian engine (``oracle/abelian.py``) run as a DMRG reproduces
  FCI, and the reference's golden H2 and LiH energies with the reference's 2u1
  settings (u1_total_charge1 = u1_total_charge2 = 1, ``dmrg/tests/test1.cpp:63-64``,
  ``dmrg/tests/Fixtures/LiHFixture.h:105-106``; energies ``test1.cpp:93``,
  ``test2.cpp:57``).
* The native plans with ``QCM_SYM_TWOU1`` (sigma, both boundary steps, the
  two-site tensor, the split prologue and the two-site MPO builder) give the
  oracle's layouts and values, checked by interpreting the exported task tables.
"""
import itertools

import numpy as np
import pytest

from qcmaquis_gb300 import native as N
from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model_2u1 import STATES, TwoU1Model
from qcmaquis_gb300.mpo import TaggedMPOMaker

from conftest import integral_map
from oracle import abelian as A
from oracle import dmrg_ref as R
from oracle import fci
from oracle import ts_mpo as OTS
from oracle.sweep import SweepParams, initial_state, run_dmrg
from plan_interp import run_plan


def _dense_hamiltonian(mpo):
    """The MPO as a dense operator on the 4^L product basis (site 0 most significant)."""
    def dense(op):
        m = np.zeros((4, 4))
        for (i, o), b in zip(op.bm.keys, op.bm.blocks):
            m[STATES.index(o), STATES.index(i)] = b[0, 0]
        return m
    T = [np.eye(1)]
    for W in mpo:
        nxt = [np.zeros((T[0].shape[0] * 4,) * 2) for _ in range(W.col_dim)]
        for b2 in range(W.col_dim):
            for b1 in W.column(b2):
                for tag, sc in W.at(b1, b2):
                    nxt[b2] += sc * np.kron(T[b1], dense(W.op(tag)))
        T = nxt
    return T[0] + mpo.core_energy * np.eye(T[0].shape[0])


@pytest.mark.parametrize("merge", [True, False])
def test_twou1_mpo_has_the_fci_spectrum(merge):
    L = 4
    ints = synthetic_integral_map(L, seed=3)
    model = TwoU1Model(L, ints, 2, 2)
    mpo = TaggedMPOMaker(model, merge_site_terms=merge).create_mpo()
    assert all(w.symmetry == "2u1" for w in mpo)
    H = _dense_hamiltonian(mpo)
    assert np.abs(H - H.T).max() < 1e-13
    nu = np.array([sum(STATES[s][0] for s in st) for st in itertools.product(range(4), repeat=L)])
    nd = np.array([sum(STATES[s][1] for s in st) for st in itertools.product(range(4), repeat=L)])
    for a, b in [(2, 2), (3, 1), (1, 1), (2, 1), (3, 2)]:
        sel = (nu == a) & (nd == b)
        got = np.linalg.eigvalsh(H[np.ix_(sel, sel)])[0]
        # the lowest state of the sector is the lowest of total spin S = Sz = (a-b)/2
        want = fci.fci_energies(L, ints, a + b, a - b, 1)[0]
        assert abs(got - want) < 1e-10, (a, b, got, want)


@pytest.mark.parametrize("L,nu,nd", [(4, 2, 2), (5, 2, 1)])
def test_oracle_twou1_dmrg_equals_fci(L, nu, nd):
    ints = synthetic_integral_map(L, seed=3)
    model = TwoU1Model(L, ints, nu, nd)
    mpo = TaggedMPOMaker(model).create_mpo()
    p = SweepParams(nsweeps=3, max_bond_dimension=64, init_bond_dimension=8, ietl_jcd_tol=1e-10,
                    ietl_jcd_maxiter=20)
    rec, _ = run_dmrg(model, mpo, p, nu + nd)
    want = fci.fci_energies(L, ints, nu + nd, nu - nd, 1)[0]
    assert abs(rec.sweep_energy[-1] - want) < 1e-9


@pytest.mark.parametrize("name", ["h2", "lih"])
def test_oracle_twou1_reproduces_the_reference_golden_energy(golden, name):
    g = golden[name]
    model = TwoU1Model(g["L"], integral_map(g["integrals"]), 1, 1)
    mpo = TaggedMPOMaker(model).create_mpo()
    rec, _ = run_dmrg(model, mpo, SweepParams(nsweeps=3, max_bond_dimension=100, init_bond_dimension=8,
                                              ietl_jcd_tol=1e-10, ietl_jcd_maxiter=20), 2)
    assert abs(rec.sweep_energy[-1] - g["energy"]) <= 1e-9 * abs(g["energy"])


def _twou1_problem(L=6, nu=3, nd=3, m=12, site=2, herm=True, seed=3):
    """A random right-normalised TwoU1 MPS with the oracle's boundaries around (site, site+1)."""
    ints = synthetic_integral_map(L, seed=seed)
    model = TwoU1Model(L, ints, nu, nd)
    mpo = TaggedMPOMaker(model).create_mpo()
    mps = initial_state(model, mpo, SweepParams(init_bond_dimension=m, seed=11), nu + nd, 0)
    left = R.left_boundary(mps[0])
    for i in range(site):
        t = R.left_normalize_and_return(mps[i])
        R.multiply_from_left(mps[i + 1], t)
        left = A.overlap_mpo_left_step(mps[i], mps[i], left, mpo[i], is_hermitian=herm)
    right = R.right_boundary(mps[L - 1])
    for i in range(L - 1, site + 1, -1):
        right = A.overlap_mpo_right_step(mps[i], mps[i], right, mpo[i], is_hermitian=herm)
    return model, mpo, mps, left, right


def test_native_twosite_mpo_is_the_abelian_product():
    """The native builder's TwoU1 two-site tensor acts like the oracle's: the same
    sigma on the same site problem (both built from the same single-site tensors)."""
    model, mpo, mps, left, right = _twou1_problem()
    f = N.make_twosite_fmpo(N.FMpo(mpo[2]), N.FMpo(mpo[3]), model.phys)
    fk = N.make_twosite_fmpo(N.FMpo(mpo[2]), N.FMpo(mpo[3]), model.phys, native_kron=True)
    assert f.symmetry == N.SYM_TWOU1 and fk.symmetry == N.SYM_TWOU1
    assert np.array_equal(f.ent_coeff, fk.ent_coeff) and np.array_equal(f.blk_q, fk.blk_q)
    ots = OTS.make_twosite_mpo(mpo[2], mpo[3], model.phys, model.phys)
    assert ots.symmetry == "2u1"
    psi = A.make_two_site_mps(mps[2], mps[3]).make_left_paired()
    lay = N.Layout.of(psi.data)
    Ll, Rl = N.BoundaryLayout.of(left), N.BoundaryLayout.of(right)
    p = N.plan_sigma(psi.phys_i, psi.left_i, psi.right_i, lay, Ll, Rl, f, True)
    bufs = [lay.pack(psi.data), Ll.pack(left), Rl.pack(right), np.zeros(p.out_elems)] + \
        [np.full(max(s, 1), np.nan) for s in p.scratch]
    run_plan(p, bufs)
    ref = lay.pack(A.site_hamil2(psi, left, right, ots).data)
    assert np.linalg.norm(bufs[3] - ref) <= 1e-13 * np.linalg.norm(ref)


@pytest.mark.parametrize("herm", [True, False])
@pytest.mark.parametrize("site,m", [(1, 8), (2, 12), (3, 10)])
def test_twou1_sigma_plan_matches_oracle(herm, site, m):
    model, mpo, mps, left, right = _twou1_problem(site=site, m=m, herm=herm)
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


def test_twou1_hermitian_partners_are_transposes():
    """With exact adjoint pairs and unit phases, sigma is the same with and without
    the Hermitian shortcut (the skipped boundaries replaced by partners' transposes)."""
    model, mpo, mps, left_h, right_h = _twou1_problem(herm=True)
    _, _, _, left_f, right_f = _twou1_problem(herm=False)
    ots = OTS.make_twosite_mpo(mpo[2], mpo[3], model.phys, model.phys)
    psi = A.make_two_site_mps(mps[2], mps[3]).make_left_paired()
    a = A.site_hamil2(psi, left_h, right_h, ots, is_hermitian=True)
    b = A.site_hamil2(psi, left_f, right_f, ots, is_hermitian=False)
    assert a.copy().axpy(-1.0, b).norm() <= 1e-12 * a.norm()


@pytest.mark.parametrize("herm", [True, False])
def test_twou1_boundary_plans_match_oracle(herm):
    L, nu, nd = 6, 3, 3
    model = TwoU1Model(L, synthetic_integral_map(L, seed=3), nu, nd)
    mpo = TaggedMPOMaker(model).create_mpo()
    mps = initial_state(model, mpo, SweepParams(init_bond_dimension=12, seed=11), nu + nd, 0)
    left = R.left_boundary(mps[0])
    for i in range(3):
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
    right = R.right_boundary(mps[L - 1])
    for i in range(L - 1, 2, -1):
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


@pytest.mark.parametrize("site", [0, 2, 4])
def test_twou1_two_site_and_split_plans_match_oracle(site):
    model, mpo, mps, _, _ = _twou1_problem(site=site)
    Ta = mps[site].copy().make_left_paired()
    Tb = mps[site + 1].copy().make_left_paired()
    la, lb = N.Layout.of(Ta.data), N.Layout.of(Tb.data)
    p = N.plan_two_site(Ta.phys_i, Ta.left_i, Ta.right_i, la, Tb.phys_i, Tb.left_i, Tb.right_i, lb, N.SYM_TWOU1)
    ref = A.make_two_site_mps(mps[site], mps[site + 1]).make_left_paired()
    phys, left, right, lay = N.out_tensor(p)
    assert phys == ref.phys_i
    assert list(lay.keys) == list(ref.data.keys)
    bufs = _run(p, {0: la.pack(Ta.data), 1: lb.pack(Tb.data)})
    want = lay.pack(ref.data)
    assert np.linalg.norm(bufs[3][:lay.size] - want) <= 1e-13 * np.linalg.norm(want)
    # the split prologue: no unreduce, the reshape to both-paired
    A0, B0 = mps[site], mps[site + 1]
    sp = N.plan_split_theta(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, lay, N.SYM_TWOU1)
    both = R._reshape_left_to_both(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, ref.data)
    _, _, _, blay = N.out_tensor(sp)
    assert list(blay.keys) == list(both.keys)
    out = _run(sp, {0: want})
    wb = blay.pack(both)
    assert np.linalg.norm(out[3][:blay.size] - wb) <= 1e-13 * np.linalg.norm(wb)


def test_unknown_symmetry_is_rejected():
    model, mpo, mps, _, _ = _twou1_problem()
    Ta = mps[2].copy().make_left_paired()
    Tb = mps[3].copy().make_left_paired()
    la, lb = N.Layout.of(Ta.data), N.Layout.of(Tb.data)
    with pytest.raises(RuntimeError, match="unknown symmetry"):
        N.plan_two_site(Ta.phys_i, Ta.left_i, Ta.right_i, la, Tb.phys_i, Tb.left_i, Tb.right_i, lb, 7)


@pytest.mark.parametrize("kind", ["2u1", "u1"])
def test_memoised_local_operators_give_the_same_model(kind, monkeypatch):
    """The abelian term builder's memoised local operators (per-site operator
    patterns) give the same terms, coefficients, provenance and operator table
    as recomputing every product."""
    import math
    from qcmaquis_gb300.model_2u1 import AbelianChemModel
    from qcmaquis_gb300.model_u1 import U1SpinOrbitalModel

    def make():
        if kind == "2u1":
            return TwoU1Model(7, synthetic_integral_map(7, seed=7), 4, 3)
        return U1SpinOrbitalModel(4, synthetic_integral_map(4, seed=4), 3)
    monkeypatch.setattr(AbelianChemModel, "_memo_enabled", False)
    a = make()
    monkeypatch.setattr(AbelianChemModel, "_memo_enabled", True)
    b = make()
    assert len(a.terms) == len(b.terms)
    for x, y in zip(a.terms, b.terms):
        assert x.ops == y.ops
        assert (x.coeff, math.copysign(1.0, x.coeff)) == (y.coeff, math.copysign(1.0, y.coeff))
        assert list(x.src.items()) == list(y.src.items())
    assert len(a.tag_handler.ops) == len(b.tag_handler.ops)
    assert a.tag_handler.herm == b.tag_handler.herm and a.tag_handler.sign == b.tag_handler.sign
