"""The zero-site problem on the GPU (``qcm_plan_zerosite`` through
``Engine.zerosite_hamil2`` / ``ZeroSiteProblem``) against the oracle's
``zerosite_hamil``: FP64 to 1e-12 relative, the tensor-core forms to their
stated accuracy, and the energy identity of ``test_siteproblem.cpp:97-154``."""
import numpy as np
import pytest

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
