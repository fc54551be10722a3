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
