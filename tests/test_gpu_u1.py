"""The abelian path with U1 charges (spin-orbital sites, charge (N, 0)) on the GPU
against the oracle's abelian engine.

* sigma (FP64: 1e-12 relative; BF16x3: 5e-6) and both boundary steps (1e-12
  absolute) on random U1 site problems;
* full two-site sweeps from the identical initial MPS: every microiteration and
  sweep energy within 1e-10 Eh of the oracle's, truncated weights to 1e-8
  relative (1e-14 absolute), equal bond dimensions; the final energy equals exact
  diagonalisation of the N-electron space;
* the reference's golden H2 and LiH energies (``dmrg/tests/test1.cpp:93``,
  ``dmrg/tests/test2.cpp:57``) over spin-orbital sites."""
import numpy as np
import pytest
import torch

from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model_u1 import U1SpinOrbitalModel
from qcmaquis_gb300.mpo import TaggedMPOMaker

from oracle import abelian as A
from oracle import dmrg_ref as R
from oracle import ts_mpo as OTS

from test_u1_cpu import _u1_problem, fci_ground

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("herm", [True, False])
def test_gpu_u1_sigma_matches_oracle(herm):
    from qcmaquis_gb300 import native as N
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine
    model, mpo, mps, left, right = _u1_problem(L=5, ne=5, m=24, site=4, herm=herm)
    ts = N.make_twosite_fmpo(N.FMpo(mpo[4]), N.FMpo(mpo[5]), model.phys)
    ots = OTS.make_twosite_mpo(mpo[4], mpo[5], model.phys, model.phys)
    psi = A.make_two_site_mps(mps[4], mps[5]).make_left_paired()
    ref = A.site_hamil2(psi, left, right, ots, is_hermitian=herm)
    for prec, tol in ((N.PREC_FP64, 1e-12), (N.PREC_BF16X3, 5e-6)):
        eng = Engine("cuda:0", precision=prec, hermitian=herm)
        x = DeviceMPSTensor.from_host(psi)
        got = eng.site_hamil2(x, DeviceBoundary.from_host(left), DeviceBoundary.from_host(right), ts)
        want = x.layout.pack(ref.data)
        err = np.linalg.norm(got.data.cpu().numpy() - want) / np.linalg.norm(want)
        assert err <= tol, (prec, err)


def test_gpu_u1_boundary_steps_match_oracle():
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine
    model, mpo, mps, _, _ = _u1_problem(L=4, ne=4, m=16, site=0)
    eng = Engine("cuda:0")
    left = R.left_boundary(mps[0])
    dl = DeviceBoundary.from_host(left)
    for i in range(4):
        dl = eng.overlap_mpo_left_step(DeviceMPSTensor.from_host(mps[i].copy().make_left_paired()), dl, mpo[i])
        left = A.overlap_mpo_left_step(mps[i], mps[i], left, mpo[i])
        got = dl.to_host()
        assert [g.keys for g in got] == [r.keys for r in left]
        for g, r in zip(got, left):
            for a, b in zip(g.blocks, r.blocks):
                assert np.max(np.abs(a - b), initial=0.0) <= 1e-12
    right = R.right_boundary(mps[model.L - 1])
    dr = DeviceBoundary.from_host(right)
    for i in range(model.L - 1, 3, -1):
        dr = eng.overlap_mpo_right_step(DeviceMPSTensor.from_host(mps[i].copy().make_left_paired()), dr, mpo[i])
        right = A.overlap_mpo_right_step(mps[i], mps[i], right, mpo[i])
        got = dr.to_host()
        assert [g.keys for g in got] == [r.keys for r in right]
        for g, r in zip(got, right):
            for a, b in zip(g.blocks, r.blocks):
                assert np.max(np.abs(a - b), initial=0.0) <= 1e-12


def test_gpu_u1_sweep_matches_oracle_and_fci():
    from qcmaquis_gb300 import sweep as G
    from oracle.sweep import SweepParams, run_dmrg
    # m = 64 holds the whole space at every bond of 8 spin-orbital sites (2^3 x 2^3)
    L, ne, m = 4, 5, 64
    ints = synthetic_integral_map(L, seed=5)
    model = U1SpinOrbitalModel(L, ints, ne)
    mpo = TaggedMPOMaker(model).create_mpo()
    gpu, _ = G.run_dmrg(model, mpo, G.SweepParams(nsweeps=3, max_bond_dimension=m), nelec=ne)
    ref, _ = run_dmrg(model, mpo, SweepParams(nsweeps=3, max_bond_dimension=m), nelec=ne)
    assert np.max(np.abs(np.array(gpu.energies) - np.array(ref.energies))) < 1e-10
    assert np.max(np.abs(np.array(gpu.sweep_energy) - np.array(ref.sweep_energy))) < 1e-10
    tg, tr = np.array(gpu.truncated_weight), np.array(ref.truncated_weight)
    assert np.all(np.abs(tg - tr) <= 1e-8 * np.abs(tr) + 1e-14)
    assert gpu.bond_dimension == ref.bond_dimension
    assert abs(gpu.sweep_energy[-1] - fci_ground(L, ints, ne)) < 1e-8


@pytest.mark.parametrize("name", ["h2", "lih"])
def test_gpu_u1_golden_energies(golden, name):
    from conftest import integral_map
    from qcmaquis_gb300 import sweep as G
    g = golden[name]
    model = U1SpinOrbitalModel(g["L"], integral_map(g["integrals"]), 2)
    mpo = TaggedMPOMaker(model).create_mpo()
    rec, _ = G.run_dmrg(model, mpo, G.SweepParams(nsweeps=3, max_bond_dimension=100), nelec=2)
    assert abs(rec.sweep_energy[-1] - g["energy"]) <= 1e-9 * abs(g["energy"])
    torch.cuda.synchronize()
