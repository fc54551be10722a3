"""Dynamic range of the BF16 split forms.

The three (two) BF16 slices of an FP32 operand share FP32's 8-bit exponent, so a
split represents values of any magnitude down to about 1e-38 without per-block
scaling.  Checked directly: scaling the ket by 2^-100 or 1e-30, or the left
boundary by 2^-60 and the right one by 2^+60 (sigma unchanged), leaves the
BF16x3 / BF16x2 sigma's relative error against the FP64 sigma within the
full-size bars (5e-6 / 2e-5) and within a factor 1.5 of the unscaled error."""
import numpy as np
import pytest
import torch

from test_oracle import _random_site_problem

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("form,bar", [("bf16x3", 5e-6), ("bf16x2", 2e-5)])
def test_split_forms_need_no_per_block_scaling(form, bar):
    from qcmaquis_gb300 import native as N
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine
    psi, left, right, ts, _ = _random_site_problem(L=8, N=8, site=3, m=24)
    prec = {"bf16x3": N.PREC_BF16X3, "bf16x2": N.PREC_BF16X2}[form]
    x = DeviceMPSTensor.from_host(psi.copy().make_left_paired())

    def boundaries(sl, sr):
        Lb, Rb = DeviceBoundary.from_host(left), DeviceBoundary.from_host(right)
        Lb.data.mul_(sl)
        Rb.data.mul_(sr)
        return Lb, Rb

    def err(sk, sl, sr):
        Lb, Rb = boundaries(sl, sr)
        xs = x.like(x.data * sk)
        want = Engine("cuda:0", precision=N.PREC_FP64).site_hamil2(xs, Lb, Rb, ts).data
        got = Engine("cuda:0", precision=prec).site_hamil2(xs, Lb, Rb, ts).data
        assert torch.all(torch.isfinite(got))
        return float(torch.linalg.norm(got - want) / torch.linalg.norm(want))

    base = err(1.0, 1.0, 1.0)
    assert base <= bar
    for sk, sl, sr in ((2.0 ** -100, 1.0, 1.0), (1e-30, 1.0, 1.0), (1.0, 2.0 ** -60, 2.0 ** 60)):
        e = err(sk, sl, sr)
        assert e <= bar and e <= 1.5 * base + 1e-7, (form, sk, sl, sr, e, base)
