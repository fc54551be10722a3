"""The zero-site problem on the GPU (``qcm_plan_zerosite`` through
``Engine.zerosite_hamil2`` / ``ZeroSiteProblem``) against the oracle's
``zerosite_hamil``: FP64 to 1e-12 relative, the tensor-core forms to their
stated accuracy, and the energy identity of ``test_siteproblem.cpp:97-154``;
and the diagonal of H_eff (``qcm_plan_diagonal``) against the oracle's."""
import numpy as np
import pytest
import torch

from oracle import dmrg_ref as R
from oracle.sweep import expval, overlap
from test_oracle import _zero_site_problem, _bm_dot

pytestmark = pytest.mark.gpu


def _device_problem(bond, herm, L=8, N=8, m=64):
    from qcmaquis_gb300.engine import DeviceBlockMatrix, DeviceBoundary, Engine, ZeroSiteProblem
    full, Cm, left, right, mpo = _zero_site_problem(L=L, N=N, m=m, bond=bond, herm=herm)
    eng = Engine("cuda:0", hermitian=herm)
    zsp = ZeroSiteProblem(eng, mpo[bond], mpo[bond + 1], DeviceBoundary.from_host(left, "cuda:0"),
                          DeviceBoundary.from_host(right, "cuda:0"))
    ref = R.zerosite_hamil(Cm, left, right, mpo[bond], mpo[bond + 1], is_hermitian=herm)
    return full, mpo, Cm, DeviceBlockMatrix.from_host(Cm, "cuda:0"), zsp, eng, ref


@pytest.mark.parametrize("herm", [True, False])
@pytest.mark.parametrize("bond", [0, 3, 6])
def test_zero_site_fp64_matches_oracle(herm, bond):
    full, mpo, Cm, x, zsp, eng, ref = _device_problem(bond, herm)
    got = zsp.apply(x).data.cpu().numpy()
    want = x.layout.pack(ref)
    assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want)
    e = expval(full, mpo) / overlap(full)
    assert abs(zsp.get_energy(x) - e) < 1e-10 * max(1.0, abs(e))
    assert _bm_dot(Cm, ref) / _bm_dot(Cm, Cm) == pytest.approx(e, abs=1e-10)


@pytest.mark.parametrize("prec,tol", [("BF16X3", 2e-5), ("BF16X2", 2e-4), ("TF32", 5e-3)])
def test_zero_site_mixed_forms(prec, tol):
    from qcmaquis_gb300 import native as N
    full, mpo, Cm, x, zsp, eng, ref = _device_problem(3, True)
    want = x.layout.pack(ref)
    got = eng.zerosite_hamil2(x, zsp.left, zsp.right, zsp.mpo_left, zsp.mpo_right,
                              precision=getattr(N, "PREC_" + prec)).data.cpu().numpy()
    assert np.linalg.norm(got - want) <= tol * np.linalg.norm(want)


@pytest.mark.parametrize("site,m", [(2, 16), (3, 24)])
def test_diagonal_hamiltonian_matches_oracle(site, m):
    """``qcm_plan_diagonal`` through ``Engine.diagonal_hamiltonian`` (full boundaries)
    against the oracle's ``diagonal_hamiltonian``, FP64 to 1e-12 relative; a mixed
    form is refused."""
    from qcmaquis_gb300 import native as N
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine
    from test_oracle import _random_site_problem
    psi, left, right, ts, ots = _random_site_problem(site=site, m=m, herm=False)
    psi = psi.copy().make_left_paired()
    eng = Engine("cuda:0", hermitian=False)
    x = DeviceMPSTensor.from_host(psi, "cuda:0")
    Lb, Rb = DeviceBoundary.from_host(left, "cuda:0"), DeviceBoundary.from_host(right, "cuda:0")
    got = eng.diagonal_hamiltonian(x, Lb, Rb, ts).data.cpu().numpy()
    want = x.layout.pack(R.diagonal_hamiltonian(left, right, ots, psi))
    assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want)
    p = N.plan_diagonal(psi.phys_i, psi.left_i, psi.right_i, x.layout, Lb.layout, Rb.layout, eng.fmpo(ts))
    p.upload()
    with pytest.raises(RuntimeError, match="FP64 form only"):
        eng.run(p, ket=x.data, left=Lb, right=Rb, out=torch.empty(p.out_elems, dtype=torch.float64, device="cuda:0"),
                precision=N.PREC_BF16X3)
