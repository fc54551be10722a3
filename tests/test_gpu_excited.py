"""Excited states on the GPU (``run_dmrg(ortho_states=...)``): the reference's LiH
S1 energy (``dmrg/tests/test2.cpp:122-139``), exact diagonalisation at L=6, and
the oracle's constrained sweeps per microiteration."""
import numpy as np
import pytest

from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model import QCModel
from qcmaquis_gb300.mpo import make_mpo

from conftest import integral_map

pytestmark = pytest.mark.gpu


def test_gpu_excited_state_golden_lih(golden):
    from qcmaquis_gb300 import sweep as G
    g = golden["lih"]
    m = QCModel(g["L"], integral_map(g["integrals"]), g["nelec"])
    mpo = make_mpo(m)
    _, gs = G.run_dmrg(m, mpo, G.SweepParams(nsweeps=2, max_bond_dimension=100), nelec=g["nelec"])
    rec, _ = G.run_dmrg(m, mpo, G.SweepParams(nsweeps=2, max_bond_dimension=100, seed=7), nelec=g["nelec"],
                        ortho_states=[gs])
    s1 = golden["lih_s1"]["energy"]
    assert abs(rec.sweep_energy[-1] - s1) < 1e-9 * abs(s1)


def test_gpu_excited_states_match_oracle_and_fci_L6():
    from qcmaquis_gb300 import sweep as G
    from oracle.fci import fci_energies
    from oracle.sweep import SweepParams as OP, run_dmrg as oracle_run
    L, Ne = 6, 6
    ints = synthetic_integral_map(L, seed=3)
    model = QCModel(L, ints, Ne)
    mpo = make_mpo(model)
    _, gs = G.run_dmrg(model, mpo, G.SweepParams(nsweeps=3, max_bond_dimension=64), nelec=Ne)
    rec, _ = G.run_dmrg(model, mpo, G.SweepParams(nsweeps=3, max_bond_dimension=64, seed=5), nelec=Ne,
                        ortho_states=[gs])
    _, ogs = oracle_run(model, mpo, OP(nsweeps=3, max_bond_dimension=64), nelec=Ne)
    orec, _ = oracle_run(model, mpo, OP(nsweeps=3, max_bond_dimension=64, seed=5), nelec=Ne, ortho_states=[ogs])
    assert np.max(np.abs(np.array(rec.energies) - np.array(orec.energies))) < 1e-9
    assert abs(rec.sweep_energy[-1] - fci_energies(L, ints, Ne, 0, 2)[1]) < 1e-9


def test_gpu_constrained_jcd_skip_and_empty_constraint():
    """The device eigensolver's constraint handling: a start vector inside the
    constraint span skips the solve (<init|H|init>, 0 iterations); a zero constraint
    is dropped and leaves the solve unchanged."""
    import torch
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine, SiteProblem
    from qcmaquis_gb300.jd import solve_ietl_jcd
    from test_oracle import _random_site_problem
    psi, left, right, ts, ots = _random_site_problem()
    x = DeviceMPSTensor.from_host(psi.copy().make_left_paired(), "cuda:0")
    eng = Engine("cuda:0")
    sp = SiteProblem(eng, DeviceBoundary.from_host(left, "cuda:0"), DeviceBoundary.from_host(right, "cuda:0"), ts)
    th, _, it = solve_ietl_jcd(sp, x, 1e-8, 6, ortho=[2.0 * x.data])
    ref = float(torch.dot(x.data, sp.apply(x).data))
    assert it == 0 and abs(th - ref) < 1e-12 * max(1.0, abs(ref))
    t1, _, i1 = solve_ietl_jcd(sp, x, 1e-8, 6)
    t2, _, i2 = solve_ietl_jcd(sp, x, 1e-8, 6, ortho=[torch.zeros_like(x.data)])
    assert i1 == i2 and abs(t1 - t2) < 1e-10 * abs(t1)
