"""Mixed-precision sigma vectors on the tcgen05 tensor cores against the FP64
sigma: BF16x3 (6 split products, FP32 accumulation) within 2e-5 relative,
TF32 within 5e-3 relative; the executor's bounded waits never time out."""
import ctypes as C

import numpy as np
import pytest
import torch

from qcmaquis_gb300 import native as N

from test_oracle import _random_site_problem

pytestmark = pytest.mark.gpu

TOL = {N.PREC_BF16X3: 2e-5, N.PREC_TF32: 5e-3}


def _status():
    s = C.c_int32(-1)
    N.check(N.lib().qcm_device_status(C.byref(s)), "qcm_device_status")
    return s.value


def _sigma_all_precisions(eng, psi, L, R, W):
    outs = {}
    for prec in (N.PREC_FP64, N.PREC_TF32, N.PREC_BF16X3):
        outs[prec] = eng.site_hamil2(psi, L, R, W, precision=prec).data.clone()
    torch.cuda.synchronize()
    return outs


@pytest.mark.parametrize("site,m", [(2, 16), (2, 40)])
def test_tensorcore_sigma_small(site, m):
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine
    psi, left, right, ts, ots = _random_site_problem(site=site, m=m)
    psi = psi.copy().make_left_paired()
    eng = Engine("cuda:0")
    o = _sigma_all_precisions(eng, DeviceMPSTensor.from_host(psi), DeviceBoundary.from_host(left),
                              DeviceBoundary.from_host(right), ts)
    ref = o[N.PREC_FP64]
    for prec, tol in TOL.items():
        err = (torch.linalg.norm(o[prec] - ref) / torch.linalg.norm(ref)).item()
        assert err < tol, (prec, err)
    assert _status() == 0


def test_tensorcore_sigma_multi_tile():
    """L=12, m=256: output blocks span several 128 x 64 tiles."""
    from qcmaquis_gb300.engine import Engine
    from qcmaquis_gb300.workloads import build_sigma_host, upload_sigma_workload
    w = build_sigma_host(L=12, nelec=12, m=256)
    eng = Engine("cuda:0")
    upload_sigma_workload(w, eng)
    o = _sigma_all_precisions(eng, w.psi, w.left, w.right, w.ts_mpo)
    ref = o[N.PREC_FP64]
    for prec, tol in TOL.items():
        err = (torch.linalg.norm(o[prec] - ref) / torch.linalg.norm(ref)).item()
        assert err < tol, (prec, err)
    assert _status() == 0


@pytest.mark.parametrize("L,m", [(12, 256), (16, 512)])
def test_image_executor_matches_in_kernel_split(L, m):
    """The BF16x3 image executor (bulk-copied pre-split operands, persistent
    warp-specialised kernel) and the in-kernel-split executor both stay within
    2e-5 of the FP64 sigma and agree with each other to the same order; the
    image executor is deterministic across calls."""
    from qcmaquis_gb300.engine import Engine
    from qcmaquis_gb300.workloads import build_sigma_host, upload_sigma_workload
    w = build_sigma_host(L=L, nelec=L, m=m)
    eng = Engine("cuda:0")
    upload_sigma_workload(w, eng)
    ref = eng.site_hamil2(w.psi, w.left, w.right, w.ts_mpo, precision=N.PREC_FP64).data.clone()
    eng.use_images = True
    a1 = eng.site_hamil2(w.psi, w.left, w.right, w.ts_mpo, precision=N.PREC_BF16X3).data.clone()
    a2 = eng.site_hamil2(w.psi, w.left, w.right, w.ts_mpo, precision=N.PREC_BF16X3).data.clone()
    eng.use_images = False
    b = eng.site_hamil2(w.psi, w.left, w.right, w.ts_mpo, precision=N.PREC_BF16X3).data.clone()
    torch.cuda.synchronize()
    nr = torch.linalg.norm(ref)
    assert (torch.linalg.norm(a1 - ref) / nr).item() < 2e-5
    assert (torch.linalg.norm(b - ref) / nr).item() < 2e-5
    assert (torch.linalg.norm(a1 - b) / nr).item() < 2e-5
    assert torch.equal(a1, a2)
    assert _status() == 0


def test_mixed_precision_boundary_steps_match_fp64():
    """Left and right boundary updates with BF16x3 block products (FP64 storage)
    within 2e-5 of the FP64 updates, L=12 m=256 middle sites."""
    from qcmaquis_gb300.engine import DeviceMPSTensor, Engine
    from qcmaquis_gb300.workloads import build_sigma_host, upload_sigma_workload
    w = build_sigma_host(L=12, nelec=12, m=256)
    eng = Engine("cuda:0")
    upload_sigma_workload(w, eng)
    A = DeviceMPSTensor.from_host(w.left_sites[-1])
    i = len(w.left_sites) - 1
    # the left boundary before site i: rebuild it from the start
    from qcmaquis_gb300.block_matrix import BlockMatrix
    from qcmaquis_gb300.engine import DeviceBoundary
    from qcmaquis_gb300.symmetry import Index
    one = lambda c: BlockMatrix.from_indices(Index([(c, 1)]), Index([(c, 1)]), fill=1.0)
    left = DeviceBoundary.from_host([one((0, 0))])
    for k in range(i):
        left = eng.overlap_mpo_left_step(DeviceMPSTensor.from_host(w.left_sites[k]), left, w.mpo[k])
    ref = eng.overlap_mpo_left_step(A, left, w.mpo[i]).data
    mix = eng.overlap_mpo_left_step(A, left, w.mpo[i], precision=N.PREC_BF16X3).data
    assert (torch.linalg.norm(mix - ref) / torch.linalg.norm(ref)).item() < 2e-5
    B = DeviceMPSTensor.from_host(w.right_sites[0])
    right = DeviceBoundary.from_host([one((w.nelec, 0))])
    for k in range(len(w.right_sites) - 1, 0, -1):
        right = eng.overlap_mpo_right_step(DeviceMPSTensor.from_host(w.right_sites[k]), right, w.mpo[w.site + 2 + k])
    ref = eng.overlap_mpo_right_step(B, right, w.mpo[w.site + 2]).data
    mix = eng.overlap_mpo_right_step(B, right, w.mpo[w.site + 2], precision=N.PREC_BF16X3).data
    assert (torch.linalg.norm(mix - ref) / torch.linalg.norm(ref)).item() < 2e-5
    assert _status() == 0
