"""The oracle against the reference's golden values and exact diagonalisation."""
import numpy as np
import pytest

from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model import QCModel
from qcmaquis_gb300.mpo import make_mpo, make_ts_cache_mpo
from qcmaquis_gb300.wigner import wigner9j
from oracle import ts_mpo as OTS
from oracle import su2 as OSU2

from oracle import dmrg_ref as R
from oracle.fci import fci_energies
from oracle.sweep import SweepParams, run_dmrg, initial_state

from conftest import integral_map


def test_wigner9j_reference_table(golden):
    # dmrg/tests/test_wigner.cpp:21-45, BOOST_CHECK_CLOSE tolerance 1e-6 percent
    for args, val in golden["wigner9j"]["cases"]:
        got = wigner9j(*args)
        if val == 0.0:
            assert abs(got) < 1e-12
        else:
            assert abs(got - val) <= 1e-8 * abs(val) + 5e-11, (args, got, val)


def test_oracle_wigner_symbols_pinned(golden):
    """The oracle's own 9j (oracle.su2) reproduces the reference's 9j table, and its
    6j/9j equal an independent exact evaluation (sympy, where installed) on a
    sweep of small doubled spins."""
    for args, val in golden["wigner9j"]["cases"]:
        got = OSU2.ninej(*args)
        assert abs(got - val) <= 1e-8 * abs(val) + 5e-11, (args, got, val)
    wig = pytest.importorskip("sympy.physics.wigner")
    from sympy import Rational
    rng = np.random.default_rng(5)
    h = lambda x: Rational(int(x), 2)
    from oracle.qn import triangle as tri
    valid6, valid9 = [], []
    while len(valid6) < 300:
        a = [int(v) for v in rng.integers(0, 9, 6)]
        if all(tri(*t) for t in ((a[0], a[1], a[2]), (a[0], a[4], a[5]), (a[3], a[1], a[5]), (a[3], a[4], a[2]))):
            valid6.append(a)
    while len(valid9) < 120:
        a = [int(v) for v in rng.integers(0, 6, 9)]
        rows = ((a[0], a[1], a[2]), (a[3], a[4], a[5]), (a[6], a[7], a[8]))
        cols = ((a[0], a[3], a[6]), (a[1], a[4], a[7]), (a[2], a[5], a[8]))
        if all(tri(*t) for t in rows + cols):
            valid9.append(a)
    for a in valid6:
        exact = float(wig.wigner_6j(*map(h, a)))
        assert abs(OSU2.sixj(*a) - exact) <= 1e-14 * max(1.0, abs(exact)), (a, exact)
    for a in valid9:
        exact = float(wig.wigner_9j(*map(h, a)))
        assert abs(OSU2.ninej(*a) - exact) <= 1e-14 * max(1.0, abs(exact)), (a, exact)


@pytest.mark.parametrize("L,N,site", [(6, 6, 0), (6, 6, 2), (6, 4, 4), (4, 2, 1)])
def test_oracle_two_site_mpo_matches_product_builder(L, N, site):
    """The oracle's two-site MPO tensor (oracle.ts_mpo, written from mt/ts_ops.h and the
    SU(2) op_kron) and the product's (Python builder; the native builder equals it
    array for array) give the same operator per (b1, b3, product spin), and the
    oracle's sigma with either tensor agrees to 1e-13."""
    ints = synthetic_integral_map(L, seed=L + site)
    model = QCModel(L, ints, N)
    mpo = make_mpo(model)
    prod = make_ts_cache_mpo(mpo, model.phys)[site]
    orc = OTS.make_twosite_mpo(mpo[site], mpo[site + 1], model.phys, model.phys)
    assert (orc.row_dim, orc.col_dim) == (prod.row_dim, prod.col_dim)
    assert set(orc.elements) == set(prod.elements)
    for key in orc.elements:
        a = {orc.op(t).spin.get(): orc.op(t) for t, _ in orc.at(*key)}
        b = {prod.op(t).spin.get(): prod.op(t) for t, _ in prod.at(*key)}
        assert sorted(a) == sorted(b), key
        for s in a:
            oa, ob = a[s], b[s]
            sa = OTS.sparse_of(oa)
            sb = prod.sparse(dict((prod.op(t).spin.get(), t) for t, _ in prod.at(*key))[s])
            assert list(oa.bm.keys) == list(ob.bm.keys), key
            for ea, eb in zip(sa, sb):
                assert [e[:4] for e in ea] == [e[:4] for e in eb], key
                assert np.allclose([e[4] for e in ea], [e[4] for e in eb], rtol=1e-14, atol=1e-15), key
    psi, left, right, ts, ots = _random_site_problem(L=L, N=N, m=12, site=site, seed=L + site)
    s1 = R.site_hamil2(psi.copy(), left, right, ots)
    s2 = R.site_hamil2(psi.copy(), left, right, ts)
    assert s1.copy().axpy(-1.0, s2).norm() <= 1e-13 * s1.norm()


@pytest.mark.parametrize("name", ["lih", "h2"])
def test_fci_pins_golden_energy(golden, name):
    g = golden[name]
    ints = integral_map(g["integrals"])
    e = fci_energies(g["L"], ints, g["nelec"], g["spin"])[0]
    assert abs(e - g["energy"]) < 1e-9


@pytest.mark.parametrize("name", ["lih", "h2"])
def test_oracle_dmrg_golden_energy(golden, name):
    # dmrg/tests/test2.cpp:57 (LiH) and dmrg/tests/test1.cpp:93 (H2), BOOST_CHECK_CLOSE 1e-7 percent
    g = golden[name]
    ints = integral_map(g["integrals"])
    m = QCModel(g["L"], ints, g["nelec"])
    mpo = make_mpo(m)
    rec, _ = run_dmrg(m, mpo, SweepParams(nsweeps=2, max_bond_dimension=100), nelec=g["nelec"])
    assert abs(rec.sweep_energy[-1] - g["energy"]) < 1e-9 * abs(g["energy"])


def test_oracle_dmrg_matches_fci_L6():
    L, N = 6, 6
    ints = synthetic_integral_map(L, seed=3)
    e_fci = fci_energies(L, ints, N, 0)[0]
    m = QCModel(L, ints, N)
    mpo = make_mpo(m)
    rec, _ = run_dmrg(m, mpo, SweepParams(nsweeps=2, max_bond_dimension=64), nelec=N)
    assert abs(rec.sweep_energy[-1] - e_fci) < 1e-10


def test_oracle_triplet_matches_fci():
    L, N = 5, 4
    ints = synthetic_integral_map(L, seed=5)
    e_fci = fci_energies(L, ints, N, 2)[0]
    m = QCModel(L, ints, N)
    mpo = make_mpo(m)
    rec, _ = run_dmrg(m, mpo, SweepParams(nsweeps=2, max_bond_dimension=64), nelec=N, twoS=2)
    assert abs(rec.sweep_energy[-1] - e_fci) < 1e-10


def _random_site_problem(L=6, N=6, seed=3, m=16, site=2, herm=True):
    ints = synthetic_integral_map(L, seed=seed)
    model = QCModel(L, ints, N)
    mpo = make_mpo(model)
    p = SweepParams(init_bond_dimension=m, seed=11)
    mps = initial_state(model, mpo, p, N, 0)
    left = R.left_boundary(mps[0])
    for i in range(site):
        # move the orthogonality centre along with the boundary
        t = R.left_normalize_and_return(mps[i])
        R.multiply_from_left(mps[i + 1], t)
        left = R.overlap_mpo_left_step(mps[i], mps[i], left, mpo[i], is_hermitian=herm)
    right = R.right_boundary(mps[L - 1])
    for i in range(L - 1, site + 1, -1):
        right = R.overlap_mpo_right_step(mps[i], mps[i], right, mpo[i], is_hermitian=herm)
    ts = make_ts_cache_mpo(mpo, model.phys)[site]
    # the oracle's own two-site tensor (oracle.ts_mpo), for the oracle's side of a comparison
    ots = OTS.make_twosite_mpo(mpo[site], mpo[site + 1], model.phys, model.phys)
    psi = R.make_two_site_mps(mps[site], mps[site + 1])
    return psi, left, right, ts, ots


def test_lbtm_equals_rbtm():
    psi, left, right, ts, ots = _random_site_problem()
    a = R.site_hamil_lbtm(psi, left, right, ots)
    b = R.site_hamil_rbtm(psi, left, right, ots)
    diff = a.copy().axpy(-1.0, b)
    assert diff.norm() <= 1e-12 * a.norm()


def test_sigma_is_symmetric():
    psi, left, right, ts, ots = _random_site_problem()
    rng = np.random.default_rng(0)
    x = psi.copy().make_left_paired()
    y = psi.copy().make_left_paired()
    for k in range(y.data.n_blocks()):
        y.data.blocks[k] = rng.standard_normal(y.data.blocks[k].shape)
    hx = R.site_hamil2(x, left, right, ots)
    hy = R.site_hamil2(y, left, right, ots)
    assert abs(y.dot(hx) - x.dot(hy)) < 1e-12 * max(1.0, abs(y.dot(hx)))


def test_hermitian_skip_matches_full_boundary():
    # dmrg/tests/test_mps_mpo_ops/test_mps_mpo_ops_electronic.cpp:39-99: skipping
    # Hermitian partners must not change sigma
    psi, left, right, ts, ots = _random_site_problem(herm=True)
    psi2, left2, right2, ts2, ots2 = _random_site_problem(herm=False)
    a = R.site_hamil_lbtm(psi, left, right, ots, is_hermitian=True)
    b = R.site_hamil_lbtm(psi2, left2, right2, ots2, is_hermitian=False)
    assert a.copy().axpy(-1.0, b).norm() <= 1e-12 * a.norm()


def test_single_site_sweeps_reach_exact_diagonalisation():
    """The oracle's single-site sweeps (noise-driven bond growth from m=5) reach the
    exact ground state of an L=6, N=6 singlet."""
    from oracle.fci import fci_energies
    from oracle.sweep import SweepParams as OP, run_dmrg_single_site
    L, N = 6, 6
    ints = synthetic_integral_map(L, seed=3)
    model = QCModel(L, ints, N)
    rec, _ = run_dmrg_single_site(model, make_mpo(model), OP(nsweeps=5, max_bond_dimension=64,
                                                             alpha_main=0.0, alpha_final=0.0), nelec=N)
    assert abs(rec.sweep_energy[-1] - fci_energies(L, ints, N, 0, 1)[0]) < 1e-9


def test_single_and_two_site_lih_agree(golden):
    """dmrg/tests/ElectronicDMRG/testLiH.cpp:27-47: single-site and two-site
    optimisation of LiH reach the same energy (the reference's tolerance, 1e-8 %),
    both the reference's golden energy."""
    from conftest import integral_map
    from oracle.sweep import SweepParams as OP, run_dmrg, run_dmrg_single_site
    g = golden["lih"]
    model = QCModel(g["L"], integral_map(g["integrals"]), g["nelec"])
    mpo = make_mpo(model)
    ts, _ = run_dmrg(model, mpo, OP(nsweeps=4, max_bond_dimension=32, ietl_jcd_tol=1e-12), nelec=g["nelec"])
    ss, _ = run_dmrg_single_site(model, mpo, OP(nsweeps=6, max_bond_dimension=32, ietl_jcd_tol=1e-12,
                                                alpha_main=0.0, alpha_final=0.0), nelec=g["nelec"])
    e_ts, e_ss = ts.sweep_energy[-1], ss.sweep_energy[-1]
    assert abs(e_ss - e_ts) <= 1e-10 * abs(e_ts)
    assert abs(e_ts - g["energy"]) <= 1e-10 * abs(g["energy"])


def _zero_site_problem(L=6, N=6, seed=3, m=16, bond=2, herm=True):
    """State, bond matrix C between sites ``bond`` and ``bond + 1``, L[bond+1], R[bond+1]
    and the MPO, as ``test_siteproblem.cpp:97-154`` prepares them: the sites left of
    the bond left-normalised, C the R factor of the QR of site ``bond``."""
    ints = synthetic_integral_map(L, seed=seed)
    model = QCModel(L, ints, N)
    mpo = make_mpo(model)
    mps = initial_state(model, mpo, SweepParams(init_bond_dimension=m, seed=11), N, 0)
    full = [t.copy() for t in mps]
    left = R.left_boundary(mps[0])
    for i in range(bond):
        t = R.left_normalize_and_return(mps[i])
        R.multiply_from_left(mps[i + 1], t)
        left = R.overlap_mpo_left_step(mps[i], mps[i], left, mpo[i], is_hermitian=herm)
    C = R.left_normalize_and_return(mps[bond])
    left = R.overlap_mpo_left_step(mps[bond], mps[bond], left, mpo[bond], is_hermitian=herm)
    right = R.right_boundary(mps[L - 1])
    for i in range(L - 1, bond, -1):
        right = R.overlap_mpo_right_step(mps[i], mps[i], right, mpo[i], is_hermitian=herm)
    return full, C, left, right, mpo


def _bm_dot(a, b) -> float:
    s = 0.0
    for key, blk in zip(a.keys, a.blocks):
        k = b.find_block(*key)
        if k < b.n_blocks():
            s += float(np.sum(blk * b.blocks[k]))
    return s


@pytest.mark.parametrize("herm", [True, False])
@pytest.mark.parametrize("bond", [0, 2, 4])
def test_zero_site_energy_equals_expval(herm, bond):
    """``test_siteproblem.cpp:97-154``: <C|H_0 C> / <C|C> is the energy of the state."""
    from oracle.sweep import expval, overlap
    full, C, left, right, mpo = _zero_site_problem(bond=bond, herm=herm)
    sig = R.zerosite_hamil(C, left, right, mpo[bond], mpo[bond + 1], is_hermitian=herm)
    e0 = _bm_dot(C, sig) / _bm_dot(C, C)
    e = expval(full, mpo) / overlap(full)
    assert abs(e0 - e) < 1e-10 * max(1.0, abs(e))


def test_zero_site_hermitian_partners_match_full_boundary():
    """The zero-site sigma with Hermitian partners (no phases, as the reference
    contracts them) equals the one over all bond indices."""
    _, C, left, right, mpo = _zero_site_problem(bond=2, herm=True)
    _, C2, left2, right2, _ = _zero_site_problem(bond=2, herm=False)
    a = R.zerosite_hamil(C, left, right, mpo[2], mpo[3], is_hermitian=True)
    b = R.zerosite_hamil(C2, left2, right2, mpo[2], mpo[3], is_hermitian=False)
    assert a.keys == b.keys
    diff = max(float(np.abs(x - y).max()) for x, y in zip(a.blocks, b.blocks))
    assert diff <= 1e-12 * a.norm()


def test_fci_pins_golden_excited_state(golden):
    """The second singlet root of LiH is the reference's excited-state energy
    (``dmrg/tests/test2.cpp:138``), independently of any DMRG code."""
    g = golden["lih"]
    e = fci_energies(g["L"], integral_map(g["integrals"]), g["nelec"], g["spin"], 2)[1]
    assert abs(e - golden["lih_s1"]["energy"]) < 1e-9 * abs(e)


def test_oracle_excited_state_golden_lih(golden):
    """``dmrg/tests/test2.cpp:122-139``: optimised orthogonal to the ground state
    (one orthogonal state), the LiH sweeps reach the reference's S1 energy
    (BOOST_CHECK_CLOSE 1e-7 percent)."""
    g = golden["lih"]
    m = QCModel(g["L"], integral_map(g["integrals"]), g["nelec"])
    mpo = make_mpo(m)
    _, gs = run_dmrg(m, mpo, SweepParams(nsweeps=2, max_bond_dimension=100), nelec=g["nelec"])
    rec, _ = run_dmrg(m, mpo, SweepParams(nsweeps=2, max_bond_dimension=100, seed=7), nelec=g["nelec"],
                      ortho_states=[gs])
    s1 = golden["lih_s1"]["energy"]
    assert abs(rec.sweep_energy[-1] - s1) < 1e-9 * abs(s1)


def test_oracle_excited_states_match_fci_L6():
    """Sequential constrained sweeps: S1 orthogonal to S0, S2 orthogonal to both,
    against exact diagonalisation (L=6, N=6 singlet)."""
    L, N = 6, 6
    ints = synthetic_integral_map(L, seed=3)
    model = QCModel(L, ints, N)
    mpo = make_mpo(model)
    exact = fci_energies(L, ints, N, 0, 3)
    _, s0 = run_dmrg(model, mpo, SweepParams(nsweeps=3, max_bond_dimension=64), nelec=N)
    r1, s1 = run_dmrg(model, mpo, SweepParams(nsweeps=3, max_bond_dimension=64, seed=5), nelec=N, ortho_states=[s0])
    r2, _ = run_dmrg(model, mpo, SweepParams(nsweeps=3, max_bond_dimension=64, seed=9), nelec=N,
                     ortho_states=[s0, s1])
    assert abs(r1.sweep_energy[-1] - exact[1]) < 1e-9
    assert abs(r2.sweep_energy[-1] - exact[2]) < 1e-9


@pytest.mark.parametrize("site,m", [(2, 8), (1, 12)])
def test_diagonal_hamiltonian_is_the_diagonal_of_sigma(site, m):
    """``ref_diag`` (``fw/optimize/ietl_davidson.h:25-58``): every element of
    ``diagonal_hamiltonian`` equals (H e_ij)(i, j) for the unit tensor e_ij, to 1e-12
    (full boundaries)."""
    psi, left, right, ts, ots = _random_site_problem(site=site, m=m, herm=False)
    psi = psi.copy().make_left_paired()
    d = R.diagonal_hamiltonian(left, right, ots, psi)
    assert d.keys == psi.data.keys
    rng = np.random.default_rng(site)
    for key, blk in zip(psi.data.keys, psi.data.blocks):
        r, c = blk.shape
        for _ in range(3):
            i, j = int(rng.integers(r)), int(rng.integers(c))
            e = psi.copy()
            for q in range(e.data.n_blocks()):
                e.data.blocks[q] = np.zeros_like(e.data.blocks[q])
            e.data.blocks[e.data.find_block(*key)][i, j] = 1.0
            h = R.site_hamil2(e, left, right, ots, is_hermitian=False).make_left_paired()
            want = h.data.blocks[h.data.find_block(*key)][i, j]
            assert abs(d.blocks[d.find_block(*key)][i, j] - want) < 1e-12 * max(1.0, abs(want))


def test_constrained_jcd_skips_a_fully_constrained_start():
    """``ietl_jacobi_davidson.h:41-47, 58-64``: when the constraints remove the whole start
    vector the solve is skipped and <init|H|init> returned with ``init``; a constraint
    the start vector is orthogonal to leaves the solve unchanged."""
    psi, left, right, ts, ots = _random_site_problem()
    apply_h = lambda x: R.site_hamil2(x, left, right, ots)
    x0 = psi.copy().make_left_paired()
    theta, u, it = R.jcd_solve(apply_h, x0, 1e-8, 6, ortho=[x0.scaled(2.0)])
    assert it == 0 and abs(theta - x0.dot(apply_h(x0))) < 1e-12 * max(1.0, abs(theta))
    zero = x0.scaled(0.0)
    t1, _, i1 = R.jcd_solve(apply_h, x0, 1e-8, 6)
    t2, _, i2 = R.jcd_solve(apply_h, x0, 1e-8, 6, ortho=[zero])
    assert i1 == i2 and abs(t1 - t2) < 1e-12 * abs(t1)
