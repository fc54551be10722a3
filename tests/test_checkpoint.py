"""MPS checkpoints (``mp_tensors/mps.hpp:312-365``, ``sim/sim.hpp:197-211``): the
file format round-trips bit for bit, damaged files are refused, and a run
resumed from a checkpoint gives the sweep energies of the uninterrupted run."""
import os

import numpy as np
import pytest

from qcmaquis_gb300 import checkpoint as CK
from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model import QCModel
from qcmaquis_gb300.mpo import make_mpo

from oracle.sweep import SweepParams, initial_state


def _mps(L=6, Ne=6, m=12):
    model = QCModel(L, synthetic_integral_map(L, seed=3), Ne)
    return model, initial_state(model, make_mpo(model), SweepParams(init_bond_dimension=m, seed=11), Ne, 0)


def test_round_trip_is_bit_exact(tmp_path):
    _, mps = _mps()
    d = str(tmp_path / "chk")
    CK.save(d, mps, status={"sweep": 3}, parameters={"max_bond_dimension": 12})
    sites, status, params = CK.load(d)
    assert status == {"sweep": 3} and params["max_bond_dimension"] == 12
    assert len(sites) == len(mps)
    for (phys, left, right, bm), t in zip(sites, mps):
        h = t.copy().make_left_paired()
        assert phys.data == h.phys_i.data and left.data == h.left_i.data and right.data == h.right_i.data
        assert bm.keys == h.data.keys
        for a, b in zip(bm.blocks, h.data.blocks):
            assert a.shape == b.shape and np.array_equal(a, b)
    assert not any(n.endswith(".new") for n in os.listdir(d))


def test_shorter_save_removes_stale_sites(tmp_path):
    _, mps = _mps()
    d = str(tmp_path / "chk")
    CK.save(d, mps)
    CK.save(d, mps[:4])
    assert len(CK.load(d)[0]) == 4


def test_damaged_files_are_refused(tmp_path):
    _, mps = _mps()
    d = str(tmp_path / "chk")
    CK.save(d, mps)
    p = os.path.join(d, "mps2")
    raw = open(p, "rb").read()
    open(p, "wb").write(raw[:-8])
    with pytest.raises(ValueError):
        CK.load(d)
    open(p, "wb").write(b"XXXX" + raw[4:])
    with pytest.raises(ValueError):
        CK.load(d)
    with pytest.raises(FileNotFoundError):
        CK.load(str(tmp_path / "nothing"))


@pytest.mark.gpu
def test_resumed_run_matches_the_uninterrupted_run(tmp_path):
    from qcmaquis_gb300 import sweep as G
    L, Ne, m = 6, 6, 24
    model = QCModel(L, synthetic_integral_map(L, seed=3), Ne)
    mpo = make_mpo(model)
    full, _ = G.run_dmrg(model, mpo, G.SweepParams(nsweeps=3, max_bond_dimension=m), nelec=Ne)
    d = str(tmp_path / "chk")
    first, _ = G.run_dmrg(model, mpo, G.SweepParams(nsweeps=1, max_bond_dimension=m), nelec=Ne, checkpoint=d)
    sites, status, _ = CK.load(d)
    assert status["sweep"] == 1
    rest, _ = G.run_dmrg(model, mpo, G.SweepParams(nsweeps=3, max_bond_dimension=m), nelec=Ne,
                         mps=CK.to_device(sites), start_sweep=status["sweep"])
    got = first.sweep_energy + rest.sweep_energy
    assert np.max(np.abs(np.array(got) - np.array(full.sweep_energy))) < 1e-11
