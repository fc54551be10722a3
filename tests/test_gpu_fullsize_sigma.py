"""Parity of the sigma vector at the benchmark's full size (L=24, N=24, S=0, middle
sites (11, 12), m=1024) against one complete oracle sigma.

The boundaries carry the benchmark workload's layouts (L[11]: 612 MPO bonds,
34 M elements; R[13]: 792 bonds, 43 M elements) filled with seeded normal
values: sigma is linear in both boundaries, so random values exercise every
term of the contraction, and the oracle does not have to build m=1024
boundaries.  The oracle uses its own two-site MPO tensor (oracle.ts_mpo); the
GPU uses the product's.  One oracle sigma takes about a minute on the host.

Tolerances (relative 2-norm of sigma - sigma_oracle): FP64 1e-12 (measured
2.0e-15); the BF16x3 split (three BF16 slices, about 24 significant bits, per
FP32 operand; FP32 intermediates T and contr; FP32 accumulation over K of up
to a few thousand) 5e-6 (measured 2.1e-6 on these random boundaries, 1.1e-6
on canonical ones); the two-slice BF16x2 form (16 significant bits per
operand) 2e-5.
"""
import numpy as np
import pytest
import torch

from oracle import dmrg_ref as R
from oracle.cpu_sample import boundary_layouts
from oracle.ts_mpo import make_twosite_mpo as oracle_twosite

pytestmark = pytest.mark.gpu

TOL = {"fp64": 1e-12, "bf16x3": 5e-6, "bf16x2": 2e-5}


@pytest.fixture(scope="module")
def fullsize():
    from qcmaquis_gb300.workloads import build_sigma_host
    w = build_sigma_host(L=24, m=1024)
    Ll, Rl = boundary_layouts(w)
    rng = np.random.default_rng(2024)
    left = Ll.unpack(rng.standard_normal(Ll.size))
    right = Rl.unpack(rng.standard_normal(Rl.size))
    ots = oracle_twosite(w.mpo[w.site], w.mpo[w.site + 1], w.model.phys, w.model.phys)
    p = w.psi_host
    ket = R.MPSTensor(p.phys_i, p.left_i, p.right_i, p.data.copy(), R.LEFT_PAIRED)
    ref = R.site_hamil_lbtm(ket, left, right, ots)
    return w, left, right, ref


@pytest.mark.parametrize("form", ["fp64", "bf16x3", "bf16x2"])
def test_fullsize_sigma_matches_oracle(fullsize, form):
    from qcmaquis_gb300 import native as N
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine
    w, left, right, ref = fullsize
    prec = {"fp64": N.PREC_FP64, "bf16x3": N.PREC_BF16X3, "bf16x2": N.PREC_BF16X2}[form]
    eng = Engine("cuda:0", precision=prec)
    x = DeviceMPSTensor.from_host(w.psi_host)
    Lb, Rb = DeviceBoundary.from_host(left), DeviceBoundary.from_host(right)
    got = eng.site_hamil2(x, Lb, Rb, w.ts_mpo).data.cpu().numpy()
    torch.cuda.synchronize()
    want = x.layout.pack(ref.data)
    err = float(np.linalg.norm(got - want) / np.linalg.norm(want))
    print(f"full-size sigma {form}: relative error {err:.3e}")
    assert np.all(np.isfinite(got))
    assert err <= TOL[form], (form, err)
