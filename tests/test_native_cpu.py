"""The C-ABI library on the CPU: it loads, exports every declared symbol, and
its plan builder produces the reference layouts and sums (checked by
interpreting the exported task tables against the oracle)."""
import os
import re

import numpy as np
import pytest

from qcmaquis_gb300 import native as N
from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model import QCModel
from qcmaquis_gb300.mpo import make_mpo

from oracle import dmrg_ref as R
from oracle.sweep import SweepParams, initial_state
from plan_interp import run_plan
from test_oracle import _random_site_problem, _zero_site_problem

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_library_exports_every_declared_symbol():
    hdr = open(os.path.join(ROOT, "include", "qcm_gb300.h")).read()
    names = set(re.findall(r"\b(qcm_[a-z0-9_]+)\s*\(", hdr))
    assert len(names) >= 15
    lib = N.lib()
    for n in sorted(names):
        assert hasattr(lib, n), n


def test_invalid_layout_is_rejected():
    psi, left, right, ts, ots = _random_site_problem()
    psi = psi.copy().make_left_paired()
    lay = N.Layout.of(psi.data)
    bad = N.Layout(list(reversed(lay.keys)), list(reversed(lay.shapes)))
    with pytest.raises(RuntimeError, match="DualIndex order"):
        N.plan_sigma(psi.phys_i, psi.left_i, psi.right_i, bad, N.BoundaryLayout.of(left),
                     N.BoundaryLayout.of(right), N.FMpo(ts))


@pytest.mark.parametrize("herm", [True, False])
@pytest.mark.parametrize("site,m", [(1, 8), (2, 16), (3, 12)])
def test_sigma_plan_matches_oracle(herm, site, m):
    psi, left, right, ts, ots = _random_site_problem(site=site, m=m, herm=herm)
    psi = psi.copy().make_left_paired()
    lay = N.Layout.of(psi.data)
    Ll, Rl = N.BoundaryLayout.of(left), N.BoundaryLayout.of(right)
    p = N.plan_sigma(psi.phys_i, psi.left_i, psi.right_i, lay, Ll, Rl, N.FMpo(ts), herm)
    # scratch starts as NaN: a read of scratch that no stage wrote shows in sigma
    bufs = [lay.pack(psi.data), Ll.pack(left), Rl.pack(right), np.zeros(p.out_elems)] + \
        [np.full(max(s, 1), np.nan) for s in p.scratch]
    run_plan(p, bufs)
    ref = lay.pack(R.site_hamil2(psi, left, right, ots, is_hermitian=herm).data)
    assert np.linalg.norm(bufs[3] - ref) <= 1e-13 * np.linalg.norm(ref)


@pytest.mark.parametrize("L,m,site,herm", [(12, 400, 5, True), (8, 200, 3, False)])
def test_sigma_image_tables_match_oracle(L, m, site, herm):
    """The BF16x3 image executor's tables and addressing (emulated in FP64,
    stale shared-memory rows as NaN) reproduce the oracle's sigma; at L=12,
    m=400 blocks span several 128-row tiles and 32-wide K-chunks.  The
    executor keeps segment coefficients in FP32, hence the 1e-7 bound."""
    psi, left, right, ts, ots = _random_site_problem(L=L, N=L, m=m, site=site, herm=herm)
    psi = psi.copy().make_left_paired()
    lay = N.Layout.of(psi.data)
    Ll, Rl = N.BoundaryLayout.of(left), N.BoundaryLayout.of(right)
    p = N.plan_sigma(psi.phys_i, psi.left_i, psi.right_i, lay, Ll, Rl, N.FMpo(ts), herm)
    assert p.image_bytes > 0
    tiles = [len(p.stage_images(i)["tiles"]) for i, k in enumerate(p.stage_kinds()) if k == "gemm"]
    assert all(t > 0 for t in tiles)
    bufs = [lay.pack(psi.data), Ll.pack(left), Rl.pack(right), np.zeros(p.out_elems)] + \
        [np.full(max(s, 1), np.nan) for s in p.scratch]
    run_plan(p, bufs, images=True)
    ref = lay.pack(R.site_hamil2(psi, left, right, ots, is_hermitian=herm).data)
    assert np.linalg.norm(bufs[3] - ref) <= 1e-7 * np.linalg.norm(ref)


@pytest.mark.parametrize("herm", [True, False])
def test_boundary_image_tables_match_oracle(herm):
    """The BF16x3 image tables of the boundary-update plans (emulated in FP64,
    scratch starting as NaN) reproduce the oracle's boundaries."""
    L, Ne = 8, 8
    m = QCModel(L, synthetic_integral_map(L, seed=3), Ne)
    mpo = make_mpo(m)
    mps = initial_state(m, mpo, SweepParams(init_bond_dimension=64, seed=11), Ne, 0)
    left = R.left_boundary(mps[0])
    for i in range(4):
        A = mps[i].copy().make_left_paired()
        lay, Ll = N.Layout.of(A.data), N.BoundaryLayout.of(left)
        p = N.plan_boundary_left(A.phys_i, A.left_i, A.right_i, lay, Ll, N.FMpo(mpo[i]), herm)
        ol = p.out_layout()
        bufs = [lay.pack(A.data), Ll.pack(left), None, np.zeros(max(p.out_elems, 1))] + \
            [np.full(max(s, 1), np.nan) for s in p.scratch]
        run_plan(p, bufs, images=True)
        ref = ol.pack(R.overlap_mpo_left_step(mps[i], mps[i], left, mpo[i], herm))
        assert np.linalg.norm(bufs[3][:ol.size] - ref) <= 1e-7 * max(np.linalg.norm(ref), 1e-300)
        left = R.overlap_mpo_left_step(mps[i], mps[i], left, mpo[i], herm)
    right = R.right_boundary(mps[L - 1])
    for i in range(L - 1, 3, -1):
        A = mps[i].copy().make_left_paired()
        lay, Rl = N.Layout.of(A.data), N.BoundaryLayout.of(right)
        p = N.plan_boundary_right(A.phys_i, A.left_i, A.right_i, lay, Rl, N.FMpo(mpo[i]), herm)
        ol = p.out_layout()
        bufs = [lay.pack(A.data), None, Rl.pack(right), np.zeros(max(p.out_elems, 1))] + \
            [np.full(max(s, 1), np.nan) for s in p.scratch]
        run_plan(p, bufs, images=True)
        ref = ol.pack(R.overlap_mpo_right_step(mps[i], mps[i], right, mpo[i], herm))
        assert np.linalg.norm(bufs[3][:ol.size] - ref) <= 1e-7 * max(np.linalg.norm(ref), 1e-300)
        right = R.overlap_mpo_right_step(mps[i], mps[i], right, mpo[i], herm)


@pytest.mark.parametrize("herm", [True, False])
def test_boundary_plans_match_oracle_layout_and_values(herm):
    L, Ne = 6, 6
    m = QCModel(L, synthetic_integral_map(L, seed=3), Ne)
    mpo = make_mpo(m)
    mps = initial_state(m, mpo, SweepParams(init_bond_dimension=16, seed=11), Ne, 0)
    left = R.left_boundary(mps[0])
    for i in range(3):
        A = mps[i].copy().make_left_paired()
        lay, Ll = N.Layout.of(A.data), N.BoundaryLayout.of(left)
        p = N.plan_boundary_left(A.phys_i, A.left_i, A.right_i, lay, Ll, N.FMpo(mpo[i]), herm)
        ol = p.out_layout()
        bufs = [lay.pack(A.data), Ll.pack(left), None, np.zeros(max(p.out_elems, 1))] + \
            [np.zeros(max(s, 1)) for s in p.scratch]
        run_plan(p, bufs)
        ref = R.overlap_mpo_left_step(mps[i], mps[i], left, mpo[i], herm)
        got = ol.unpack(bufs[3])
        assert [g.keys for g in got] == [r.keys for r in ref]
        assert np.allclose(ol.pack(ref), bufs[3][:ol.size], rtol=0, atol=1e-13)
        left = ref
    right = R.right_boundary(mps[L - 1])
    for i in range(L - 1, 2, -1):
        A = mps[i].copy().make_left_paired()
        lay, Rl = N.Layout.of(A.data), N.BoundaryLayout.of(right)
        p = N.plan_boundary_right(A.phys_i, A.left_i, A.right_i, lay, Rl, N.FMpo(mpo[i]), herm)
        ol = p.out_layout()
        bufs = [lay.pack(A.data), None, Rl.pack(right), np.zeros(max(p.out_elems, 1))] + \
            [np.zeros(max(s, 1)) for s in p.scratch]
        run_plan(p, bufs)
        ref = R.overlap_mpo_right_step(mps[i], mps[i], right, mpo[i], herm)
        got = ol.unpack(bufs[3])
        assert [g.keys for g in got] == [r.keys for r in ref]
        assert np.allclose(ol.pack(ref), bufs[3][:ol.size], rtol=0, atol=1e-13)
        right = ref


@pytest.mark.parametrize("herm", [True, False])
@pytest.mark.parametrize("bond", [0, 2, 4])
@pytest.mark.parametrize("images", [False, True])
def test_zero_site_plan_matches_oracle(herm, bond, images):
    """qcm_plan_zerosite against the oracle's zerosite_hamil; images=True runs the
    BF16x3 image tables (FP64 values in slice 0)."""
    _, Cm, left, right, mpo = _zero_site_problem(bond=bond, herm=herm)
    lay, Ll, Rl = N.Layout.of(Cm), N.BoundaryLayout.of(left), N.BoundaryLayout.of(right)
    p = N.plan_zerosite(lay, Ll, Rl, N.FMpo(mpo[bond]), N.FMpo(mpo[bond + 1]), herm)
    assert [st[0] for st in p.stages()][:2] == ["gemm", "gemm"]
    bufs = [lay.pack(Cm), Ll.pack(left), Rl.pack(right), np.full(p.out_elems, np.nan)] + \
        [np.full(max(s, 1), np.nan) for s in p.scratch]
    run_plan(p, bufs, images=images)
    ref = lay.pack(R.zerosite_hamil(Cm, left, right, mpo[bond], mpo[bond + 1], is_hermitian=herm))
    assert np.linalg.norm(bufs[3] - ref) <= (1e-7 if images else 1e-13) * np.linalg.norm(ref)



@pytest.mark.parametrize("site,m", [(2, 8), (3, 12)])
def test_diagonal_plan_matches_oracle(site, m):
    """qcm_plan_diagonal against the oracle's diagonal_hamiltonian (full boundaries)."""
    psi, left, right, ts, ots = _random_site_problem(site=site, m=m, herm=False)
    psi = psi.copy().make_left_paired()
    lay, Ll, Rl = N.Layout.of(psi.data), N.BoundaryLayout.of(left), N.BoundaryLayout.of(right)
    p = N.plan_diagonal(psi.phys_i, psi.left_i, psi.right_i, lay, Ll, Rl, N.FMpo(ts))
    assert [st[0] for st in p.stages()][:3] == ["axpy", "zero", "gemm"]
    bufs = [lay.pack(psi.data), Ll.pack(left), Rl.pack(right), np.full(p.out_elems, np.nan)] + \
        [np.full(max(s, 1), np.nan) for s in p.scratch]
    run_plan(p, bufs)
    ref = lay.pack(R.diagonal_hamiltonian(left, right, ots, psi))
    assert np.linalg.norm(bufs[3] - ref) <= 1e-13 * np.linalg.norm(ref)


def test_zero_site_plan_rejects_mismatched_bond():
    _, Cm, left, right, mpo = _zero_site_problem(bond=2)
    lay, Ll, Rl = N.Layout.of(Cm), N.BoundaryLayout.of(left), N.BoundaryLayout.of(right)
    with pytest.raises(RuntimeError, match="qcm_plan_zerosite"):
        N.plan_zerosite(lay, Ll, Rl, N.FMpo(mpo[1]), N.FMpo(mpo[3]))


def test_plan_work_counters_match_oracle():
    psi, left, right, ts, ots = _random_site_problem()
    psi = psi.copy().make_left_paired()
    lay = N.Layout.of(psi.data)
    p = N.plan_sigma(psi.phys_i, psi.left_i, psi.right_i, lay, N.BoundaryLayout.of(left),
                     N.BoundaryLayout.of(right), N.FMpo(ts))
    R.FLOPS.reset()
    R.site_hamil_lbtm(psi, left, right, ots)
    # the plan computes every T row eagerly, as the oracle does; the sums match
    assert p.gemm_flops == R.FLOPS.gemm_flops
    assert p.axpy_flops <= R.FLOPS.axpy_flops


def test_cpp_layer_builds_a_plan(tmp_path):
    """The header-only C++ layer compiles with g++, links the library and builds a plan."""
    import subprocess
    exe = tmp_path / "capi_example"
    src = os.path.join(ROOT, "tests", "capi_example.cpp")
    libdir = os.path.join(ROOT, "qcmaquis_gb300")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I" + os.path.join(ROOT, "include"), src, "-o", str(exe),
                        "-L" + libdir, "-lqcm_gb300", "-Wl,-rpath," + libdir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "out=4" in out.stdout


@pytest.mark.parametrize("prog", ["capi_microiteration", "capi_engine"])
def test_cpp_microiteration_host_compiles(tmp_path, prog):
    """The C++ hosts that run a whole microiteration through the C ABI
    (tests/capi_microiteration.cpp) and through the reference-facing C++ classes
    (tests/capi_engine.cpp, include/qcm_gb300_engine.hpp) compile and link (the
    GPU tests run them)."""
    import subprocess
    exe = tmp_path / prog
    libdir = os.path.join(ROOT, "qcmaquis_gb300")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-I" + os.path.join(ROOT, "include"), "-I" + cuda + "/include",
                        os.path.join(ROOT, "tests", prog + ".cpp"), "-o", str(exe), "-L" + libdir,
                        "-lqcm_gb300", "-Wl,-rpath," + libdir, "-L" + cuda + "/lib64", "-lcudart"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


_FMPO_ARRAYS = ("left_spin", "right_spin", "left_herm", "right_herm", "left_phase", "right_phase", "col_ptr",
                "row_of", "term_ptr", "term_op", "term_scale", "op_spin", "op_blk_ptr", "blk_q", "blk_ent_ptr",
                "ent", "ent_coeff")


@pytest.mark.parametrize("L,nelec,seed", [(6, 6, 3), (8, 6, 5)])
def test_native_twosite_mpo_equals_python_builder(L, nelec, seed):
    """qcm_mpo_twosite_* (the native two-site builder) reproduces the flattened
    make_twosite_mpo tensor of every site pair array for array, bit for bit."""
    from qcmaquis_gb300.mpo import make_twosite_mpo
    model = QCModel(L, synthetic_integral_map(L, seed=seed), nelec)
    mpo = make_mpo(model)
    flat = [N.FMpo(w) for w in mpo]
    for p in range(L - 1):
        ref = N.FMpo(make_twosite_mpo(mpo[p], mpo[p + 1], model.phys, model.phys))
        got = N.make_twosite_fmpo(flat[p], flat[p + 1], model.phys)
        for k in _FMPO_ARRAYS:
            a, b = getattr(ref, k), getattr(got, k)
            assert a.shape == b.shape and np.array_equal(a, b), (p, k)
        assert got.n_ops == ref.n_ops and got.term_key == ref.term_key


def test_native_twosite_mpo_rejects_unshared_bond():
    model = QCModel(6, synthetic_integral_map(6, seed=3), 6)
    mpo = make_mpo(model)
    with pytest.raises(RuntimeError, match="do not share a bond"):
        N.make_twosite_fmpo(N.FMpo(mpo[0]), N.FMpo(mpo[2]), model.phys)


@pytest.mark.parametrize("name", ["h2", "lih"])
def test_native_twosite_mpo_on_the_golden_systems(golden, name):
    """The native two-site builder on the reference's H2 (L=2, one pair) and LiH
    (L=4) systems equals the Python builder array for array."""
    from conftest import integral_map
    from qcmaquis_gb300.mpo import make_twosite_mpo
    g = golden[name]
    model = QCModel(g["L"], integral_map(g["integrals"]), g["nelec"])
    mpo = make_mpo(model)
    for p in range(g["L"] - 1):
        ref = N.FMpo(make_twosite_mpo(mpo[p], mpo[p + 1], model.phys, model.phys))
        got = N.make_twosite_fmpo(N.FMpo(mpo[p]), N.FMpo(mpo[p + 1]), model.phys)
        for k in _FMPO_ARRAYS:
            assert np.array_equal(getattr(ref, k), getattr(got, k)), (p, k)


def test_native_twosite_mpo_with_native_kronecker_products():
    """qcm_mpo_twosite (the SU(2) op_kron in native code as well): the same tensor
    structure as the Python builder, coefficients equal to within 1e-15 of the
    tensor's largest (the Wigner symbols are long-double sums there, exact
    rationals in the Python restatement)."""
    from qcmaquis_gb300.mpo import make_twosite_mpo
    L, nelec = 8, 6
    model = QCModel(L, synthetic_integral_map(L, seed=5), nelec)
    mpo = make_mpo(model)
    flat = [N.FMpo(w) for w in mpo]
    for p in range(L - 1):
        ref = N.FMpo(make_twosite_mpo(mpo[p], mpo[p + 1], model.phys, model.phys))
        got = N.make_twosite_fmpo(flat[p], flat[p + 1], model.phys, native_kron=True)
        for k in _FMPO_ARRAYS:
            if k == "ent_coeff":
                continue
            assert np.array_equal(getattr(ref, k), getattr(got, k)), (p, k)
        assert got.term_key == ref.term_key
        assert np.max(np.abs(got.ent_coeff - ref.ent_coeff)) <= 1e-15 * np.max(np.abs(ref.ent_coeff))
