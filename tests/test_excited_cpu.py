"""The excited-state pieces of the device path (``qcmaquis_gb300.excited``: overlap
boundaries and constraint vectors) against the oracle's ``overlap_left_step`` /
``overlap_right_step`` / ``site_ortho_boundaries``.  They run here on CPU tensors,
their block products (native plans) executed by the task-table interpreter, to
check their index and layout logic without a GPU."""
import numpy as np
import pytest
import torch

from qcmaquis_gb300.engine import DeviceMPSTensor
from qcmaquis_gb300.excited import OverlapBoundaries
from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model import QCModel
from qcmaquis_gb300.mpo import make_mpo
from qcmaquis_gb300 import native as N

from oracle import dmrg_ref as R
from oracle.sweep import OverlapBoundaries as RefOverlap, SweepParams, initial_state
from plan_interp import patch_cpu_plans


def _dbm_dict(d):
    return {k: b.detach().cpu().numpy() for k, b in zip(d.keys, d.blocks)}


def _bm_dict(b):
    return {k: v for k, v in zip(b.keys, b.blocks)}


@pytest.mark.parametrize("seeds", [(11, 12), (3, 8)])
def test_overlap_boundaries_and_vectors_match_oracle(seeds, monkeypatch):
    patch_cpu_plans(monkeypatch)
    L, Ne = 6, 6
    model = QCModel(L, synthetic_integral_map(L, seed=3), Ne)
    mpo = make_mpo(model)
    psi = initial_state(model, mpo, SweepParams(init_bond_dimension=12, seed=seeds[0]), Ne, 0)
    phi = initial_state(model, mpo, SweepParams(init_bond_dimension=9, seed=seeds[1]), Ne, 0)
    ref = RefOverlap(psi, [phi])
    dev = lambda t: DeviceMPSTensor.from_host(t.copy().make_left_paired(), device="cpu")
    got = OverlapBoundaries([dev(t) for t in psi], [[dev(t) for t in phi]], (Ne, 0))
    for i in range(1, L):
        a, b = _dbm_dict(got.right[0][i]), _bm_dict(ref.right[0][i])
        assert a.keys() == b.keys()
        for k in a:
            assert np.allclose(a[k], b[k], rtol=0, atol=1e-13)
    for i in range(1, 4):
        ref.update_left(i)
        got.update_left(i)
        a, b = _dbm_dict(got.left[0][i]), _bm_dict(ref.left[0][i])
        assert a.keys() == b.keys()
        for k in a:
            assert np.allclose(a[k], b[k], rtol=0, atol=1e-13)
    # the constraint vector of the pair (2, 3), in the pair's own layout
    site = 2
    theta_ref = R.make_two_site_mps(psi[site], psi[site + 1])
    v_ref = ref.vectors(site, theta_ref)[0]
    # the two-site tensor itself is a native plan (GPU); it equals the oracle's
    # (tests/test_mps_plans_cpu.py), so the oracle's stands in for it here
    import qcmaquis_gb300.excited as X

    def host_theta(a, b):
        ha = R.MPSTensor(a.phys_i, a.left_i, a.right_i, a.to_block_matrix(), R.LEFT_PAIRED)
        hb = R.MPSTensor(b.phys_i, b.left_i, b.right_i, b.to_block_matrix(), R.LEFT_PAIRED)
        return dev(R.make_two_site_mps(ha, hb))
    monkeypatch.setattr(X, "make_two_site_mps", host_theta)
    theta = dev(theta_ref)
    v = got.vectors(site, theta)[0].numpy()
    lay = N.Layout.of(v_ref.copy().make_left_paired().data)
    assert list(lay.keys) == list(theta.layout.keys)
    want = lay.pack(v_ref.data)
    assert np.linalg.norm(v - want) <= 1e-12 * max(np.linalg.norm(want), 1e-300)
    assert np.linalg.norm(want) > 0
