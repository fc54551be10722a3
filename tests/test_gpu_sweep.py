"""GPU two-site sweeps against the oracle: per-microiteration and per-sweep
energies to 1e-10 Eh, truncated weights to 1e-8 relative (absolute 1e-14
floor), starting from the identical initial MPS."""
import json
import os

import numpy as np
import pytest

from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model import QCModel
from qcmaquis_gb300.mpo import make_mpo

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
E_TOL = 1e-10
TW_REL = 1e-8
TW_ABS = 1e-14


def _gpu_sweep(L, N, m, nsweeps, seed_ints, twoS=0):
    from qcmaquis_gb300 import sweep as G
    model = QCModel(L, synthetic_integral_map(L, seed=seed_ints), N)
    mpo = make_mpo(model)
    rec, _ = G.run_dmrg(model, mpo, G.SweepParams(nsweeps=nsweeps, max_bond_dimension=m), nelec=N, twoS=twoS)
    return model, mpo, rec


def _check(gpu, ref_energies, ref_sweep, ref_tw):
    assert np.max(np.abs(np.array(gpu.energies) - np.array(ref_energies))) < E_TOL
    assert np.max(np.abs(np.array(gpu.sweep_energy) - np.array(ref_sweep))) < E_TOL
    tw_g, tw_r = np.array(gpu.truncated_weight), np.array(ref_tw)
    assert np.all(np.abs(tw_g - tw_r) <= TW_REL * np.abs(tw_r) + TW_ABS)


def test_gpu_sweep_matches_oracle_L6():
    from oracle.sweep import SweepParams, run_dmrg
    L, N, m = 6, 6, 24
    model, mpo, gpu = _gpu_sweep(L, N, m, 2, seed_ints=3)
    ref, _ = run_dmrg(model, mpo, SweepParams(nsweeps=2, max_bond_dimension=m), nelec=N)
    _check(gpu, ref.energies, ref.sweep_energy, ref.truncated_weight)
    assert gpu.bond_dimension == ref.bond_dimension


def test_gpu_sweep_golden_lih(golden):
    from conftest import integral_map
    from qcmaquis_gb300 import sweep as G
    g = golden["lih"]
    model = QCModel(g["L"], integral_map(g["integrals"]), g["nelec"])
    mpo = make_mpo(model)
    rec, _ = G.run_dmrg(model, mpo, G.SweepParams(nsweeps=2, max_bond_dimension=100), nelec=g["nelec"])
    assert abs(rec.sweep_energy[-1] - g["energy"]) < 1e-9 * abs(g["energy"])


def test_gpu_sweep_matches_oracle_config0():
    """Plain two-site DMRG, L=8 N=8 S=0, m=64, 6 sweeps (oracle values committed)."""
    with open(os.path.join(HERE, "golden", "oracle_L8_m64.json")) as f:
        ref = json.load(f)
    from qcmaquis_gb300 import sweep as G
    model = QCModel(8, synthetic_integral_map(8, seed=0, diag_range=(-2.0, -0.5)), 8)
    gpu, _ = G.run_dmrg(model, make_mpo(model), G.SweepParams(nsweeps=6, max_bond_dimension=64), nelec=8)
    _check(gpu, ref["energies"], ref["sweep_energy"], ref["tw"])


def test_mixed_precision_sweep_energy_close_to_fp64():
    """BF16x3 tensor-core sigma vectors inside the sweep: final energy within
    1e-6 Eh of the FP64 sweep (L=8, N=8, m=64, 6 sweeps)."""
    from qcmaquis_gb300 import sweep as G
    with open(os.path.join(HERE, "golden", "oracle_L8_m64.json")) as f:
        ref = json.load(f)
    model = QCModel(8, synthetic_integral_map(8, seed=0, diag_range=(-2.0, -0.5)), 8)
    gpu, _ = G.run_dmrg(model, make_mpo(model), G.SweepParams(nsweeps=6, max_bond_dimension=64), nelec=8,
                        precision=2)
    assert abs(gpu.sweep_energy[-1] - ref["sweep_energy"][-1]) < 1e-6


def test_mixed_precision_boundaries_sweep_energy_close_to_fp64():
    """BF16x3 sigma vectors and BF16x3 boundary updates (boundaries stored in
    FP64): final energy within 1e-6 Eh of the FP64 sweep (L=8, N=8, m=64, 6 sweeps)."""
    from qcmaquis_gb300 import sweep as G
    with open(os.path.join(HERE, "golden", "oracle_L8_m64.json")) as f:
        ref = json.load(f)
    model = QCModel(8, synthetic_integral_map(8, seed=0, diag_range=(-2.0, -0.5)), 8)
    gpu, _ = G.run_dmrg(model, make_mpo(model), G.SweepParams(nsweeps=6, max_bond_dimension=64), nelec=8,
                        precision=2, boundary_precision=2)
    assert abs(gpu.sweep_energy[-1] - ref["sweep_energy"][-1]) < 1e-6


def test_gpu_single_site_sweep_matches_oracle():
    """Single-site sweeps (density-matrix prediction with the reference's noise
    schedule): per-microiteration and per-sweep energies to 1e-10 Eh of the oracle's."""
    from oracle.sweep import SweepParams as OP, run_dmrg_single_site as oracle_ss
    from qcmaquis_gb300 import sweep as G
    L, N, m = 6, 6, 24
    model = QCModel(L, synthetic_integral_map(L, seed=3), N)
    mpo = make_mpo(model)
    gpu, _ = G.run_dmrg_single_site(model, mpo, G.SweepParams(nsweeps=3, max_bond_dimension=m), nelec=N)
    ref, _ = oracle_ss(model, mpo, OP(nsweeps=3, max_bond_dimension=m), nelec=N)
    assert np.max(np.abs(np.array(gpu.energies) - np.array(ref.energies))) < E_TOL
    assert np.max(np.abs(np.array(gpu.sweep_energy) - np.array(ref.sweep_energy))) < E_TOL
    # the bond dimension can differ by density-matrix eigenvalues at rounding level
    # (~1e-17) that fall on either side of the cut; the kept weight cannot
    tw_g, tw_r = np.array(gpu.truncated_weight), np.array(ref.truncated_weight)
    assert np.all(np.abs(tw_g - tw_r) <= TW_REL * np.abs(tw_r) + TW_ABS)


def test_gpu_sweep_with_plan_caches_is_unchanged():
    """``run_dmrg(plan_cache=n)`` reuses sigma and boundary-step plans whose layouts
    recur; the plans are the same tables, so every energy equals the uncached one."""
    from qcmaquis_gb300 import sweep as G
    L, Ne = 6, 6
    model = QCModel(L, synthetic_integral_map(L, seed=3), Ne)
    mpo = make_mpo(model)
    p = G.SweepParams(nsweeps=4, max_bond_dimension=24)
    plain, _ = G.run_dmrg(model, mpo, p, nelec=Ne)
    cached, _ = G.run_dmrg(model, mpo, p, nelec=Ne, plan_cache=64)
    assert cached.boundary_plan_hits > 0 and cached.plan_hits > 0
    assert np.max(np.abs(np.array(cached.energies) - np.array(plain.energies))) < 1e-12
    assert np.max(np.abs(np.array(cached.sweep_energy) - np.array(plain.sweep_energy))) < 1e-12
