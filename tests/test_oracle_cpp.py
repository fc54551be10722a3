"""The C++/OpenMP oracle sigma (``oracle/sigma_ref.cpp``, the timed CPU baseline)
against the numpy oracle's ``site_hamil_lbtm`` on the same inputs, with and
without Hermitian partners, with the host BLAS and with the oracle's own loop
nest: relative 2-norm difference <= 1e-12 (FP64 sums in a different order)."""
import numpy as np
import pytest

from oracle import cpu_sigma as CS
from oracle import dmrg_ref as R

from test_oracle import _random_site_problem


def _inputs(psi, left, right, ots):
    psi = psi.copy().make_left_paired()
    keys, shapes = psi.data.keys, [b.shape for b in psi.data.blocks]
    offs = np.cumsum([0] + [r * c for r, c in shapes])[:-1]
    a = {}
    a.update(CS.index_arrays(psi.phys_i, "phys"))
    a.update(CS.index_arrays(psi.left_i, "left"))
    a.update(CS.index_arrays(psi.right_i, "right"))
    a.update(CS.block_arrays(keys, shapes, offs, "psi"))
    la, _ = CS.boundary_arrays([(bm.keys, [b.shape for b in bm.blocks]) for bm in left], "L")
    ra, _ = CS.boundary_arrays([(bm.keys, [b.shape for b in bm.blocks]) for bm in right], "R")
    a.update(la)
    a.update(ra)
    a.update(CS.flatten_mpo(ots))
    flat = lambda bms: np.concatenate([np.ravel(b, order="F") for bm in bms for b in bm.blocks] + [np.zeros(1)])
    return CS.SigmaInputs(a), np.concatenate([np.ravel(b, order="F") for b in psi.data.blocks]), flat(left), \
        flat(right), psi


@pytest.mark.parametrize("herm", [True, False])
@pytest.mark.parametrize("site,m", [(2, 16), (1, 24), (0, 8)])
@pytest.mark.parametrize("use_blas", [True, False])
def test_cpp_oracle_sigma_matches_numpy_oracle(herm, site, m, use_blas):
    psi, left, right, ts, ots = _random_site_problem(site=site, m=m, herm=herm)
    inp, x, Ld, Rd, psil = _inputs(psi, left, right, ots)
    got, work = CS.sigma(inp, x, Ld, Rd, hermitian=herm, threads=4, use_blas=use_blas)
    R.FLOPS.reset()
    ref = R.site_hamil_lbtm(psil, left, right, ots, is_hermitian=herm).make_left_paired()
    want = np.concatenate([np.ravel(ref.data.blocks[ref.data.find_block(*k)], order="F") for k in psil.data.keys])
    assert np.linalg.norm(got - want) <= 1e-12 * np.linalg.norm(want)
    assert work[0] == pytest.approx(R.FLOPS.gemm_flops, rel=1e-12)
    assert work[1] == pytest.approx(R.FLOPS.axpy_flops, rel=1e-12)


def test_cpp_oracle_reports_errors():
    psi, left, right, ts, ots = _random_site_problem(site=2, m=8)
    inp, x, Ld, Rd, _ = _inputs(psi, left, right, ots)
    inp.a["psi.rows"][0] += 1   # a ket block that no longer matches sigma's
    with pytest.raises(RuntimeError):
        CS.sigma(inp, np.zeros(inp.psi_size + 100), Ld, Rd)
