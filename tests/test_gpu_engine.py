"""GPU parity of the native sigma vector, boundary steps and vector kernels
against the oracle (FP64: relative tolerance 1e-12 on sigma, absolute 1e-12
on boundary blocks)."""
import numpy as np
import pytest
import torch

from qcmaquis_gb300 import native as N
from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model import QCModel
from qcmaquis_gb300.mpo import make_mpo

from oracle import dmrg_ref as R
from oracle.sweep import SweepParams, initial_state
from test_oracle import _random_site_problem

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def engine():
    from qcmaquis_gb300.engine import Engine
    return Engine("cuda:0")


@pytest.mark.parametrize("herm", [True, False])
@pytest.mark.parametrize("site,m", [(1, 8), (2, 16), (2, 40)])
def test_sigma_matches_oracle(engine, herm, site, m):
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine
    eng = engine if herm else Engine("cuda:0", hermitian=False)
    psi, left, right, ts, ots = _random_site_problem(site=site, m=m, herm=herm)
    psi = psi.copy().make_left_paired()
    dk = DeviceMPSTensor.from_host(psi)
    out = eng.site_hamil2(dk, DeviceBoundary.from_host(left), DeviceBoundary.from_host(right), ts)
    torch.cuda.synchronize()
    ref = dk.layout.pack(R.site_hamil2(psi, left, right, ots, is_hermitian=herm).data)
    got = out.data.cpu().numpy()
    assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)


def test_sigma_repeated_calls_are_bitwise_identical(engine):
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor
    psi, left, right, ts, ots = _random_site_problem(site=2, m=24)
    psi = psi.copy().make_left_paired()
    dk = DeviceMPSTensor.from_host(psi)
    L, Rb = DeviceBoundary.from_host(left), DeviceBoundary.from_host(right)
    a = engine.site_hamil2(dk, L, Rb, ts).data.clone()
    b = engine.site_hamil2(dk, L, Rb, ts).data.clone()
    assert torch.equal(a, b)


def test_boundary_steps_match_oracle(engine):
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor
    L, Ne = 6, 6
    m = QCModel(L, synthetic_integral_map(L, seed=3), Ne)
    mpo = make_mpo(m)
    mps = initial_state(m, mpo, SweepParams(init_bond_dimension=24, seed=11), Ne, 0)
    left = R.left_boundary(mps[0])
    dleft = DeviceBoundary.from_host(left)
    for i in range(3):
        A = mps[i].copy().make_left_paired()
        dleft = engine.overlap_mpo_left_step(DeviceMPSTensor.from_host(A), dleft, mpo[i])
        left = R.overlap_mpo_left_step(mps[i], mps[i], left, mpo[i])
        got = dleft.to_host()
        assert [g.keys for g in got] == [r.keys for r in left]
        assert np.allclose(dleft.layout.pack(left), dleft.data.cpu().numpy()[:dleft.layout.size], rtol=0,
                           atol=1e-12)
    right = R.right_boundary(mps[L - 1])
    dright = DeviceBoundary.from_host(right)
    for i in range(L - 1, 2, -1):
        A = mps[i].copy().make_left_paired()
        dright = engine.overlap_mpo_right_step(DeviceMPSTensor.from_host(A), dright, mpo[i])
        right = R.overlap_mpo_right_step(mps[i], mps[i], right, mpo[i])
        got = dright.to_host()
        assert [g.keys for g in got] == [r.keys for r in right]
        assert np.allclose(dright.layout.pack(right), dright.data.cpu().numpy()[:dright.layout.size], rtol=0,
                           atol=1e-12)


def test_vector_kernels():
    lib = N.lib()
    n = 1_000_003
    g = torch.Generator(device="cuda").manual_seed(0)
    x = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
    y = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
    out = torch.zeros(4, dtype=torch.float64, device="cuda")
    N.check(lib.qcm_dot(x.data_ptr(), y.data_ptr(), n, out.data_ptr(), None), "dot")
    N.check(lib.qcm_nrm2(x.data_ptr(), n, out[1:].data_ptr(), None), "nrm2")
    torch.cuda.synchronize()
    assert abs(out[0].item() - torch.dot(x, y).item()) < 1e-9
    assert abs(out[1].item() - torch.linalg.norm(x).item()) < 1e-9
    z = y.clone()
    N.check(lib.qcm_axpby(2.0, x.data_ptr(), -0.5, z.data_ptr(), n, None), "axpby")
    torch.cuda.synchronize()
    assert torch.allclose(z, 2.0 * x - 0.5 * y, rtol=0, atol=1e-12)
