"""The adjoint of the local energy: dE/d(MPO term scale) from the energy-gradient
plan (K1, the adjoint of K3, per-term dots of the K2 tables), and through the MPO
builder's term labels and the model's integral provenance dE/d(t_pq),
dE/d(V_pqrs).

E = <psi| H_eff psi> is linear in every MPO term scale, so the gradient is
checked exactly through the pinned sigma path: for any direction d of the
scales, <grad, d> = <psi, H_eff(d) psi>, the sigma with the scales replaced by
d (the oracle's sigma, pinned against the reference's golden values).  The
integral gradient is checked against central differences of the energy of a
fixed MPS (exact up to rounding: the energy is linear in the integrals) and,
at the converged LiH ground state, against the 2-RDM of exact
diagonalisation."""
import numpy as np
import pytest

from qcmaquis_gb300 import native as N
from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model import QCModel
from qcmaquis_gb300.mpo import TaggedMPOMaker

from oracle import dmrg_ref as R
from oracle.sweep import SweepParams, initial_state
from plan_interp import run_plan


def _single_site_problem(L=6, Ne=6, m=16, site=2, seed=3, merge=False):
    """Site tensor j with the full environments L[j], R[j+1] of a random MPS."""
    model = QCModel(L, synthetic_integral_map(L, seed=seed), Ne)
    mpo = TaggedMPOMaker(model, merge_site_terms=merge).create_mpo()
    mps = initial_state(model, mpo, SweepParams(init_bond_dimension=m, seed=11), Ne, 0)
    left = R.left_boundary(mps[0])
    for i in range(site):
        left = R.overlap_mpo_left_step(mps[i], mps[i], left, mpo[i])
    right = R.right_boundary(mps[L - 1])
    for i in range(L - 1, site, -1):
        right = R.overlap_mpo_right_step(mps[i], mps[i], right, mpo[i])
    return model, mpo, mps, left, right


def _with_scales(t, scales, f):
    """A copy of MPO tensor t whose term scales are ``scales`` (FMpo's flattened order)."""
    import copy
    c = copy.copy(t)
    c.elements = {k: list(v) for k, v in t.elements.items()}
    for (b1, b2, pos), s in zip(f.term_key, scales):
        tag, _ = c.elements[(b1, b2)][pos]
        c.elements[(b1, b2)][pos] = (tag, float(s))
    return c


def _interp_gradient(psi, left, right, w, herm=True):
    lay = N.Layout.of(psi.data)
    Ll, Rl = N.BoundaryLayout.of(left), N.BoundaryLayout.of(right)
    f = N.FMpo(w)
    p = N.plan_energy_gradient(psi.phys_i, psi.left_i, psi.right_i, lay, Ll, Rl, f, herm)
    assert p.out_elems == f.n_terms
    bufs = [lay.pack(psi.data), Ll.pack(left), Rl.pack(right), np.full(p.out_elems, np.nan)] + \
        [np.full(max(s, 1), np.nan) for s in p.scratch]
    run_plan(p, bufs)
    return bufs[3][:p.out_elems].copy(), f


@pytest.mark.parametrize("site", [0, 2, 5])
def test_gradient_plan_gives_every_directional_derivative(site):
    model, mpo, mps, left, right = _single_site_problem(site=site)
    psi = mps[site].copy().make_left_paired()
    g, f = _interp_gradient(psi, left, right, mpo[site])
    # Euler: E is linear in the scales
    e = psi.dot(R.site_hamil2(psi.copy(), left, right, mpo[site]))
    assert abs(float(np.dot(f.term_scale, g)) - e) <= 1e-11 * abs(e)
    rng = np.random.default_rng(site)
    for _ in range(3):
        d = rng.standard_normal(f.n_terms)
        ed = psi.dot(R.site_hamil2(psi.copy(), left, right, _with_scales(mpo[site], d, f)))
        assert abs(float(np.dot(d, g)) - ed) <= 1e-11 * max(1.0, abs(ed), np.abs(d).sum() * np.abs(g).max())


def test_local_energy_is_the_expectation_value():
    """With full environments, <psi_j| H_eff psi_j> is <Psi|H|Psi> of the whole MPS at every j."""
    from oracle.sweep import expval
    model, mpo, mps, left, right = _single_site_problem(site=3)
    psi = mps[3].copy().make_left_paired()
    e = psi.dot(R.site_hamil2(psi.copy(), left, right, mpo[3]))
    assert abs(e - expval(mps, mpo)) <= 1e-11 * abs(e)


def test_every_model_term_is_a_labelled_mpo_scale():
    model = QCModel(6, synthetic_integral_map(6, seed=3), 6)
    mpo = TaggedMPOMaker(model, merge_site_terms=False).create_mpo()
    seen = {}
    for j, t in enumerate(mpo):
        for key, labs in t.labels.items():
            for pos, lab in enumerate(labs):
                if lab is not None:
                    assert lab not in seen
                    seen[lab] = (j, key, pos)
                    assert t.elements[key][pos][1] == model.terms[lab].coeff
    assert set(seen) | set(mpo.core_labels) == set(range(len(model.terms)))
    # the coefficients are the recorded linear combinations of the integrals
    for term in model.terms:
        assert abs(sum(f * model.integrals[u] for u, f in term.src.items()) - term.coeff) <= 1e-14 * max(
            1.0, abs(term.coeff))


def test_unmerged_site_terms_give_the_same_energy():
    from oracle.sweep import expval
    model = QCModel(6, synthetic_integral_map(6, seed=3), 6)
    a = TaggedMPOMaker(model).create_mpo()
    b = TaggedMPOMaker(model, merge_site_terms=False).create_mpo()
    mps = initial_state(model, a, SweepParams(init_bond_dimension=12, seed=11), 6, 0)
    assert abs(expval(mps, a) - expval(mps, b)) <= 1e-12 * abs(expval(mps, a))


# ------------------------------------------------------------------ integrals
def _oracle_integral_gradient(model, mps, nelec):
    """The gradient driver's chain on the CPU: oracle environments, the plans run by the
    task-table interpreter, then chain_to_integrals."""
    from qcmaquis_gb300.gradient import chain_to_integrals
    from oracle.sweep import overlap
    mpo = TaggedMPOMaker(model, merge_site_terms=False).create_mpo()
    L = model.L
    right = [None] * (L + 1)
    right[L] = R.right_boundary(mps[L - 1])
    for j in range(L - 1, 0, -1):
        right[j] = R.overlap_mpo_right_step(mps[j], mps[j], right[j + 1], mpo[j])
    left = R.left_boundary(mps[0])
    grads, fmpos = [], []
    for j in range(L):
        psi = mps[j].copy().make_left_paired()
        g, f = _interp_gradient(psi, left, right[j + 1], mpo[j])
        grads.append(g)
        fmpos.append(f)
        left = R.overlap_mpo_left_step(mps[j], mps[j], left, mpo[j])
    return chain_to_integrals(model, mpo, grads, fmpos, overlap(mps))


def _energy(model_ints, L, nelec, mps):
    from oracle.sweep import expval, overlap
    m = QCModel(L, model_ints, nelec)
    mpo = TaggedMPOMaker(m).create_mpo()
    return expval(mps, mpo) / overlap(mps) + mpo.core_energy


def test_integral_gradient_matches_central_differences():
    """20 random integrals of an L=6 problem at a random MPS: the energy is linear in
    each integral, so central differences (step 1e-5) are exact up to rounding."""
    L, Ne = 6, 6
    ints = synthetic_integral_map(L, seed=3)
    model = QCModel(L, ints, Ne)
    mps = initial_state(model, TaggedMPOMaker(model).create_mpo(), SweepParams(init_bond_dimension=12, seed=5),
                        Ne, 0)
    _, d_int = _oracle_integral_gradient(model, mps, Ne)
    keys = sorted(ints)
    rng = np.random.default_rng(7)
    h = 1e-5
    for u in [keys[i] for i in rng.choice(len(keys), 20, replace=False)]:
        up, dn = dict(ints), dict(ints)
        up[u] += h
        dn[u] -= h
        fd = (_energy(up, L, Ne, mps) - _energy(dn, L, Ne, mps)) / (2 * h)
        assert abs(fd - d_int[u]) <= 1e-7 * max(1.0, abs(fd)), (u, fd, d_int[u])


def test_integral_gradient_at_the_lih_ground_state_is_the_reference_rdm(golden):
    """LiH (L=4, N=2): the converged oracle DMRG state's integral gradient equals the RDM
    sums of exact diagonalisation, and the exact 2-RDM equals the reference's own
    golden 2-RDM (test2.cpp:60-120), whose element (i,j,k,l) is the chemist-ordered
    Gamma[j,k,i,l] = sum_st <a+_js a+_it a_lt a_ks>."""
    from conftest import integral_map
    from oracle.fci import fci_rdms, fci_states
    from oracle.sweep import SweepParams as OP, run_dmrg
    from qcmaquis_gb300.gradient import rdm_sums_from_gamma
    g = golden["lih"]
    ints = integral_map(g["integrals"])
    L, Ne = g["L"], g["nelec"]
    model = QCModel(L, ints, Ne)
    rec, mps = run_dmrg(model, TaggedMPOMaker(model).create_mpo(),
                        OP(nsweeps=6, max_bond_dimension=32, ietl_jcd_tol=1e-13, ietl_jcd_maxiter=20), nelec=Ne)
    assert abs(rec.sweep_energy[-1] - g["energy"]) < 1e-9
    _, d_int = _oracle_integral_gradient(model, mps, Ne)
    (st,), dets = fci_states(L, ints, Ne, 0, 1)
    g1, g2 = fci_rdms(L, dets, st[1])
    want = rdm_sums_from_gamma(L, list(d_int), g1, g2)
    err = max(abs(d_int[u] - want[u]) for u in d_int)
    assert err < 1e-8, err
    ref = golden["lih_2rdm"]
    got = np.array([g2[j, k, i, l] for (i, j, k, l) in ref["index"]])
    assert np.max(np.abs(got - np.array(ref["value"]))) < 1e-8


# ------------------------------------------------------------------ GPU
@pytest.mark.gpu
@pytest.mark.parametrize("site", [0, 3])
def test_gpu_gradient_plan_matches_interpreter(site):
    import torch
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine
    model, mpo, mps, left, right = _single_site_problem(site=site, m=24)
    psi = mps[site].copy().make_left_paired()
    want, f = _interp_gradient(psi, left, right, mpo[site])
    eng = Engine("cuda:0")
    x, Lb, Rb = DeviceMPSTensor.from_host(psi), DeviceBoundary.from_host(left), DeviceBoundary.from_host(right)
    p = N.plan_energy_gradient(psi.phys_i, psi.left_i, psi.right_i, x.layout, Lb.layout, Rb.layout, f, True)
    p.upload()
    out = torch.empty(p.out_elems, dtype=torch.float64, device="cuda:0")
    eng.run(p, ket=x.data, left=Lb, right=Rb, out=out, precision=N.PREC_FP64)
    got = out.cpu().numpy()
    assert np.max(np.abs(got - want)) <= 1e-12 * max(1.0, np.abs(want).max())
    with pytest.raises(RuntimeError):
        eng.run(p, ket=x.data, left=Lb, right=Rb, out=out, precision=N.PREC_BF16X3)


@pytest.mark.gpu
def test_gpu_integral_gradient_matches_the_cpu_chain():
    from qcmaquis_gb300.engine import DeviceMPSTensor
    from qcmaquis_gb300.gradient import energy_gradient
    L, Ne = 6, 6
    ints = synthetic_integral_map(L, seed=3)
    model = QCModel(L, ints, Ne)
    mps = initial_state(model, TaggedMPOMaker(model).create_mpo(), SweepParams(init_bond_dimension=16, seed=5),
                        Ne, 0)
    _, want = _oracle_integral_gradient(model, mps, Ne)
    res = energy_gradient(model, [DeviceMPSTensor.from_host(t.copy().make_left_paired()) for t in mps], Ne)
    assert abs(res.energy - _energy(ints, L, Ne, mps)) <= 1e-11 * abs(res.energy)
    err = max(abs(res.d_integrals[u] - want[u]) for u in want)
    assert err <= 1e-11 * max(1.0, max(abs(v) for v in want.values()))


@pytest.mark.gpu
def test_gpu_lih_ground_state_gradient_is_the_rdm(golden):
    """GPU sweeps to the LiH ground state, the GPU gradient, and the RDM sums of exact
    diagonalisation (pinned to the reference's golden 2-RDM by the CPU test)."""
    from conftest import integral_map
    from oracle.fci import fci_rdms, fci_states
    from qcmaquis_gb300 import sweep as G
    from qcmaquis_gb300.gradient import energy_gradient, rdm_sums_from_gamma
    g = golden["lih"]
    ints = integral_map(g["integrals"])
    L, Ne = g["L"], g["nelec"]
    model = QCModel(L, ints, Ne)
    rec, mps = G.run_dmrg(model, TaggedMPOMaker(model).create_mpo(),
                          G.SweepParams(nsweeps=6, max_bond_dimension=32, ietl_jcd_tol=1e-13, ietl_jcd_maxiter=20),
                          nelec=Ne)
    assert abs(rec.sweep_energy[-1] - g["energy"]) < 1e-9
    res = energy_gradient(model, mps, Ne)
    (st,), dets = fci_states(L, ints, Ne, 0, 1)
    g1, g2 = fci_rdms(L, dets, st[1])
    want = rdm_sums_from_gamma(L, list(res.d_integrals), g1, g2)
    assert max(abs(res.d_integrals[u] - want[u]) for u in want) < 1e-8


# ------------------------------------------------------------------ RDMs
def _oracle_term_gradients(mpo, mps, herm=False):
    """Per-site term gradients of <Psi|O|Psi> on the CPU (oracle environments, plans run
    by the task-table interpreter); a measurement MPO is not Hermitian, so every bond
    is contracted."""
    L = len(mpo)
    right = [None] * (L + 1)
    right[L] = R.right_boundary(mps[L - 1])
    for j in range(L - 1, 0, -1):
        right[j] = R.overlap_mpo_right_step(mps[j], mps[j], right[j + 1], mpo[j], is_hermitian=herm)
    left = R.left_boundary(mps[0])
    grads, fmpos = [], []
    for j in range(L):
        g, f = _interp_gradient(mps[j].copy().make_left_paired(), left, right[j + 1], mpo[j], herm)
        grads.append(g)
        fmpos.append(f)
        left = R.overlap_mpo_left_step(mps[j], mps[j], left, mpo[j], is_hermitian=herm)
    return grads, fmpos


def _lih_ground_state(golden):
    from conftest import integral_map
    from oracle.sweep import SweepParams as OP, run_dmrg
    g = golden["lih"]
    ints = integral_map(g["integrals"])
    model = QCModel(g["L"], ints, g["nelec"])
    rec, mps = run_dmrg(model, TaggedMPOMaker(model).create_mpo(),
                        OP(nsweeps=6, max_bond_dimension=32, ietl_jcd_tol=1e-13, ietl_jcd_maxiter=20),
                        nelec=g["nelec"])
    assert abs(rec.sweep_energy[-1] - g["energy"]) < 1e-9
    return g, ints, model, mps


def test_rdm_measurement_reproduces_the_reference_lih_2rdm(golden):
    """One adjoint pass over a measurement MPO that holds every element's terms gives
    the reference's spin-free 2-RDM (twoptdm of dmrg/tests/test2.cpp:60-120), element
    for element and in the reference's element order; and the 1-RDM equals exact
    diagonalisation's spin-summed gamma_pq."""
    from oracle.fci import fci_rdms, fci_states
    from oracle.sweep import overlap
    from qcmaquis_gb300 import rdm as RD
    g, ints, model, mps = _lih_ground_state(golden)
    elems, terms, owner = RD.rdm_terms(model, 2)
    mpo = RD.measurement_mpo(model, terms)
    grads, fmpos = _oracle_term_gradients(mpo, mps)
    vals = RD.elements_from_term_gradients(mpo, terms, owner, len(elems), grads, fmpos, overlap(mps))
    ref = golden["lih_2rdm"]
    assert [tuple(x) for x in ref["index"]] == elems
    assert np.max(np.abs(vals - np.array(ref["value"]))) < 1e-8
    (st,), dets = fci_states(g["L"], ints, g["nelec"], 0, 1)
    g1, _ = fci_rdms(g["L"], dets, st[1])
    elems1, terms1, owner1 = RD.rdm_terms(model, 1)
    mpo1 = RD.measurement_mpo(model, terms1)
    grads1, fmpos1 = _oracle_term_gradients(mpo1, mps)
    v1 = RD.elements_from_term_gradients(mpo1, terms1, owner1, len(elems1), grads1, fmpos1, overlap(mps))
    for (p, q), v in zip(elems1, v1):
        assert abs(v - g1[p, q]) < 1e-8, ((p, q), v, g1[p, q])


def test_rdm_measurement_reproduces_the_reference_h2_values(golden):
    """The H2 checks of dmrg/tests/test1.cpp:95-118 on the measured RDMs of the
    H2 ground state: gamma_00 + gamma_11 = 2 and the 2-RDM element (0,0,0,0) =
    1.1796482258, to the reference's 1e-7 % (BOOST_CHECK_CLOSE)."""
    from conftest import integral_map
    from oracle.sweep import SweepParams as OP, overlap, run_dmrg
    from qcmaquis_gb300 import rdm as RD
    g = golden["h2"]
    model = QCModel(g["L"], integral_map(g["integrals"]), g["nelec"])
    rec, mps = run_dmrg(model, TaggedMPOMaker(model).create_mpo(),
                        OP(nsweeps=4, max_bond_dimension=16, ietl_jcd_tol=1e-13, ietl_jcd_maxiter=20),
                        nelec=g["nelec"])
    assert abs(rec.sweep_energy[-1] - g["energy"]) < 1e-9
    ref = golden["h2_rdm"]
    tol = ref["rel_tol_percent"] / 100.0
    values = {}
    for rank in (1, 2):
        elems, terms, owner = RD.rdm_terms(model, rank)
        mpo = RD.measurement_mpo(model, terms)
        grads, fmpos = _oracle_term_gradients(mpo, mps)
        vals = RD.elements_from_term_gradients(mpo, terms, owner, len(elems), grads, fmpos, overlap(mps))
        values.update({tuple(e): float(v) for e, v in zip(elems, vals)})
    trace = values[(0, 0)] + values[(1, 1)]
    assert abs(trace - ref["onerdm_00_plus_11"]) <= tol * abs(ref["onerdm_00_plus_11"])
    assert abs(values[(0, 0, 0, 0)] - ref["twordm_0000"]) <= tol * abs(ref["twordm_0000"])


@pytest.mark.gpu
def test_gpu_rdm_measurement_reproduces_the_reference_lih_2rdm(golden):
    from conftest import integral_map
    from qcmaquis_gb300 import sweep as G
    from qcmaquis_gb300.rdm import measure_rdm
    g = golden["lih"]
    model = QCModel(g["L"], integral_map(g["integrals"]), g["nelec"])
    rec, mps = G.run_dmrg(model, TaggedMPOMaker(model).create_mpo(),
                          G.SweepParams(nsweeps=6, max_bond_dimension=32, ietl_jcd_tol=1e-13, ietl_jcd_maxiter=20),
                          nelec=g["nelec"])
    rdm2 = measure_rdm(model, mps, g["nelec"], rank=2)
    ref = golden["lih_2rdm"]
    assert list(rdm2) == [tuple(x) for x in ref["index"]]
    assert np.max(np.abs(np.array(list(rdm2.values())) - np.array(ref["value"]))) < 1e-8


def _energy_from_rdms(L, ints, rdm1, rdm2):
    """core + sum t gamma + 1/2 sum (pq|rs) Gamma from the measured elements (their
    index symmetry pqrs = rspq = qpsr = srqp fills the rest)."""
    from oracle.fci import expand_integrals
    t, V, core = expand_integrals(L, ints)
    g1 = np.zeros((L, L))
    for (p, q), v in rdm1.items():
        g1[p, q] = g1[q, p] = v
    G = np.zeros((L, L, L, L))
    for (i, j, k, l), v in rdm2.items():
        # element (a,b,c,d) = chemist Gamma[b,c,a,d]
        for a, b, c, d in ((i, j, k, l), (k, l, i, j), (j, i, l, k), (l, k, j, i)):
            G[b, c, a, d] = v
    return core + float(np.sum(t * g1)) + 0.5 * float(np.sum(V * G))


def test_rdms_of_a_random_state_give_its_energy():
    """E = core + sum t gamma + 1/2 sum (pq|rs) Gamma holds for any state: the measured
    RDMs of a random L=6, N=6 MPS reproduce its expectation value."""
    from oracle.sweep import expval, overlap
    from qcmaquis_gb300 import rdm as RD
    L, Ne = 6, 6
    ints = synthetic_integral_map(L, seed=3)
    model = QCModel(L, ints, Ne)
    mpo = TaggedMPOMaker(model).create_mpo()
    mps = initial_state(model, mpo, SweepParams(init_bond_dimension=12, seed=5), Ne, 0)
    nrm = overlap(mps)
    out = []
    for rank in (1, 2):
        elems, terms, owner = RD.rdm_terms(model, rank)
        m = RD.measurement_mpo(model, terms)
        grads, fmpos = _oracle_term_gradients(m, mps)
        out.append(dict(zip(elems, RD.elements_from_term_gradients(m, terms, owner, len(elems), grads, fmpos, nrm))))
    e = expval(mps, mpo) / nrm + mpo.core_energy
    assert abs(_energy_from_rdms(L, ints, *out) - e) < 1e-10 * max(1.0, abs(e))


def test_measured_2rdm_is_the_exact_2rdm_at_l6():
    """At the L=6, N=6 ground state, the measured elements and their index images fill
    the whole chemist-ordered Gamma, equal to exact diagonalisation's."""
    from oracle.fci import fci_rdms, fci_states
    from oracle.sweep import SweepParams as OP, overlap, run_dmrg
    from qcmaquis_gb300 import rdm as RD
    L, Ne = 6, 6
    ints = synthetic_integral_map(L, seed=3)
    model = QCModel(L, ints, Ne)
    rec, mps = run_dmrg(model, TaggedMPOMaker(model).create_mpo(),
                        OP(nsweeps=6, max_bond_dimension=64, ietl_jcd_tol=1e-13, ietl_jcd_maxiter=20), nelec=Ne)
    (st,), dets = fci_states(L, ints, Ne, 0, 1)
    _, g2 = fci_rdms(L, dets, st[1])
    elems, terms, owner = RD.rdm_terms(model, 2)
    m = RD.measurement_mpo(model, terms)
    grads, fmpos = _oracle_term_gradients(m, mps)
    vals = RD.elements_from_term_gradients(m, terms, owner, len(elems), grads, fmpos, overlap(mps))
    G = np.full((L,) * 4, np.nan)
    for (i, j, k, l), v in zip(elems, vals):
        for a, b, c, d in ((i, j, k, l), (k, l, i, j), (j, i, l, k), (l, k, j, i)):
            G[b, c, a, d] = v
    assert not np.isnan(G).any()
    assert np.max(np.abs(G - g2)) < 1e-9


@pytest.mark.gpu
def test_gpu_gradient_with_recomputed_environments_is_unchanged():
    """Keeping every third right environment and recomputing the others gives the
    per-site term gradients of the keep-all pass bit for bit."""
    from qcmaquis_gb300.engine import DeviceMPSTensor, Engine
    from qcmaquis_gb300.gradient import term_gradients
    L, Ne = 8, 8
    model = QCModel(L, synthetic_integral_map(L, seed=5), Ne)
    mpo = TaggedMPOMaker(model, merge_site_terms=False).create_mpo()
    mps_host = initial_state(model, mpo, SweepParams(init_bond_dimension=12, seed=3), Ne, 0)
    mps = [DeviceMPSTensor.from_host(t.copy().make_left_paired()) for t in mps_host]
    eng = Engine("cuda:0")
    a = term_gradients(mpo, mps, Ne, 0, eng, store_every=1)
    b = term_gradients(mpo, mps, Ne, 0, eng, store_every=3)
    for ga, gb in zip(a[0], b[0]):
        assert np.array_equal(ga, gb)
    assert a[2] == b[2]


@pytest.mark.parametrize("L,k", [(30, 1), (30, 6), (30, 5), (7, 3), (2, 4), (1, 2)])
def test_checkpointed_right_environments_schedule(L, k):
    """Every R[i] read in the left-to-right order is the keep-all value, each site costs
    at most one extra step, and at most L//k + k + 1 environments are resident."""
    from qcmaquis_gb300.gradient import CheckpointedRight
    calls = []

    def step(j, b):
        calls.append(j)
        return (j, b)
    want = {L: "end"}
    for j in range(L - 1, 0, -1):
        want[j] = (j, want[j + 1])
    r = CheckpointedRight(step, "end", L, k)
    assert len(calls) == L - 1
    peak = r.resident()
    for i in range(1, L + 1):
        assert r[i] == want[i]
        peak = max(peak, r.resident())
        r.release(i)
    assert peak <= (L // k + k + 1 if k > 1 else L)
    assert len(calls) <= 2 * (L - 1)
    assert r.resident() == 0
