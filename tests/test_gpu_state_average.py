"""State-averaged two-site DMRG (``qcmaquis_gb300.state_average``) on the GPU.

* The merged k-root sigma (one plan, shared boundaries) equals k single-root
  sigma vectors to 1e-14 relative.
* k = 3 roots of an L=6, N=6, S=0 SU2U1 Hamiltonian at a bond dimension that
  holds the whole space: every root's FP64 energy equals the corresponding
  singlet eigenvalue of exact diagonalisation to 1e-8 Eh.
* Two roots of a TwoU1 problem equal the two lowest eigenvalues of the
  (N_up, N_down) sector.
"""
import numpy as np
import pytest
import torch

from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model import QCModel
from qcmaquis_gb300.mpo import make_mpo

from oracle import fci

pytestmark = pytest.mark.gpu


def test_merged_sigma_equals_single_root_sigma():
    from qcmaquis_gb300 import native as N
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine
    from qcmaquis_gb300.state_average import SharedSigma
    from test_oracle import _random_site_problem
    psi, left, right, ts, _ = _random_site_problem(site=2, m=16)
    eng = Engine("cuda:0")
    x = DeviceMPSTensor.from_host(psi.copy().make_left_paired())
    Lb, Rb = DeviceBoundary.from_host(left), DeviceBoundary.from_host(right)
    k = 3
    gen = torch.Generator(device="cuda").manual_seed(3)
    X = torch.randn((k, x.n), dtype=torch.float64, device="cuda", generator=gen)
    sig = SharedSigma(eng, x, Lb, Rb, ts, k)
    Y = sig.apply(X.contiguous())
    for r in range(k):
        xr = DeviceMPSTensor(x.phys_i, x.left_i, x.right_i, x.layout, X[r].clone())
        want = eng.site_hamil2(xr, Lb, Rb, ts).data
        assert torch.linalg.norm(Y[r] - want) <= 1e-14 * torch.linalg.norm(want)


def test_state_averaged_roots_equal_exact_diagonalisation():
    from qcmaquis_gb300.state_average import run_sa_dmrg
    from qcmaquis_gb300.sweep import SweepParams
    L, N, k = 6, 6, 3
    ints = synthetic_integral_map(L, seed=3)
    model = QCModel(L, ints, N)
    mpo = make_mpo(model)
    p = SweepParams(nsweeps=5, max_bond_dimension=128, ietl_jcd_tol=1e-10, ietl_jcd_maxiter=40)
    rec, _, _, _ = run_sa_dmrg(model, mpo, p, N, 0, nroots=k)
    want = np.array(fci.fci_energies(L, ints, N, 0, k))
    got = rec.sweep_energies[-1]
    assert np.max(np.abs(got - want)) < 1e-8, (got, want)
    # one merged sigma launch per Davidson step
    assert all(c <= it + 1 for c, it in zip(rec.sigma_launches, rec.iterations))


def test_state_averaged_twou1_roots():
    from qcmaquis_gb300.model_2u1 import TwoU1Model
    from qcmaquis_gb300.mpo import TaggedMPOMaker
    from qcmaquis_gb300.state_average import run_sa_dmrg
    from qcmaquis_gb300.sweep import SweepParams
    L, nu, nd = 5, 2, 2
    ints = synthetic_integral_map(L, seed=4)
    model = TwoU1Model(L, ints, nu, nd)
    mpo = TaggedMPOMaker(model).create_mpo()
    p = SweepParams(nsweeps=4, max_bond_dimension=128, ietl_jcd_tol=1e-10, ietl_jcd_maxiter=40)
    rec, _, _, _ = run_sa_dmrg(model, mpo, p, nu + nd, nroots=2)
    # the two lowest states of the (2, 2) sector, of any total spin
    H_roots = sorted(fci.fci_energies(L, ints, nu + nd, 0, 2) + fci.fci_energies(L, ints, nu + nd, 2, 2)
                     + fci.fci_energies(L, ints, nu + nd, 4, 1))[:2]
    assert np.max(np.abs(rec.sweep_energies[-1] - np.array(H_roots))) < 1e-8
