"""One two-site microiteration driven by a C++ host through the C ABI only
(``tests/capi_microiteration.cpp``: ``qcm_plan_two_site``, ``qcm_plan_sigma`` +
``qcm_jcd_solve``, ``qcm_split``, ``qcm_plan_boundary_left`` +
``qcm_boundary_step``), and the same microiteration written against the
reference-facing C++ classes over that ABI (``tests/capi_engine.cpp``:
``TwoSiteTensor``, ``SiteProblem``, ``solve_ietl_jcd``, ``split_mps_l2r``,
``Engine::overlap_mpo_left_step`` of ``include/qcm_gb300_engine.hpp``), against
the oracle's microiteration on the same inputs:

* LiH (the reference's ``dmrg/tests/test2.cpp`` system) at its converged state:
  the eigenvalue plus the core energy reproduces the reference's golden energy;
* a random L=6 singlet truncated to Mmax=8: eigenvalue and iteration count of the
  oracle's Jacobi-Davidson, bond dimension and truncated weight of its split.

Gauge-invariant comparisons: energies to 1e-10 Eh, truncated weight to 1e-8
relative, the two-site product A'B' of the new site tensors to 1e-10 (up to the
eigenvector's overall sign, which the eigensolver does not fix), the new
left boundary's layout exactly and its per-block Frobenius norms to 1e-10
relative (its blocks are A'^T L A' products, so an orthogonal gauge of the new
bond changes their entries but not their norms)."""
import os
import struct
import subprocess

import numpy as np
import pytest

from qcmaquis_gb300 import native as N
from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model import QCModel
from qcmaquis_gb300.mpo import make_mpo, make_ts_cache_mpo
from oracle import dmrg_ref as R
from oracle.sweep import SweepParams, initial_state, run_dmrg
from oracle.ts_mpo import make_twosite_mpo as oracle_twosite

from conftest import ROOT, integral_map

pytestmark = pytest.mark.gpu

_FM = ("left_spin", "right_spin", "left_herm", "right_herm", "left_phase", "right_phase", "col_ptr", "row_of",
       "term_ptr", "term_op", "term_scale", "op_spin", "op_blk_ptr", "blk_q", "blk_ent_ptr", "ent", "ent_coeff")


def _put(f, name, arr):
    a = np.ascontiguousarray(arr)
    t = {np.dtype(np.int32): b"i", np.dtype(np.int64): b"l", np.dtype(np.float64): b"d"}[a.dtype]
    f.write(name.encode().ljust(32, b"\0") + t + struct.pack("<q", a.size) + a.tobytes())


def _read(path):
    out = {}
    with open(path, "rb") as f:
        while True:
            head = f.read(41)
            if len(head) < 41:
                break
            name = head[:32].rstrip(b"\0").decode()
            t, n = head[32:33], struct.unpack("<q", head[33:41])[0]
            dt = {b"i": np.int32, b"l": np.int64, b"d": np.float64}[t]
            out[name] = np.frombuffer(f.read(n * np.dtype(dt).itemsize), dtype=dt)
    return out


def _index(f, name, idx):
    _put(f, name + ".q", np.array([x for c, _ in idx for x in c] or [0], dtype=np.int32))
    _put(f, name + ".size", np.array([s for _, s in idx], dtype=np.int64))


def _tensor(f, name, t):
    t = t.copy().make_left_paired()
    lay = N.Layout.of(t.data)
    _put(f, name + ".q", lay.q)
    _put(f, name + ".rows", np.array([s[0] for s in lay.shapes], dtype=np.int64))
    _put(f, name + ".cols", np.array([s[1] for s in lay.shapes], dtype=np.int64))
    _put(f, name + ".off", np.array(lay.offsets, dtype=np.int64))
    _put(f, name + ".data", lay.pack(t.data))
    _index(f, name + ".left", t.left_i)
    _index(f, name + ".right", t.right_i)


def _boundary(f, name, b):
    lay = N.BoundaryLayout.of(b)
    _put(f, name + ".blk_ptr", lay.ptr)
    for k in ("q", "rows", "cols", "off"):
        _put(f, name + "." + k, getattr(lay, k))
    _put(f, name + ".data", lay.pack(b))


def _mpo(f, name, fm):
    _put(f, name + ".dims", np.array([fm.mpo.row_dim, fm.mpo.col_dim, fm.n_ops], dtype=np.int32))
    for k in _FM:
        _put(f, name + "." + k, getattr(fm, k))


@pytest.fixture(scope="module", params=["capi_microiteration", "capi_engine"])
def host_exe(request, tmp_path_factory):
    """The host program: the raw C ABI (capi_microiteration.cpp) or the
    reference-facing C++ classes over it (capi_engine.cpp, qcm_gb300_engine.hpp)."""
    exe = tmp_path_factory.mktemp("capi") / request.param
    libdir = os.path.join(ROOT, "qcmaquis_gb300")
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-I" + os.path.join(ROOT, "include"), "-I" + cuda + "/include",
                        os.path.join(ROOT, "tests", request.param + ".cpp"), "-o", str(exe), "-L" + libdir,
                        "-lqcm_gb300", "-Wl,-rpath," + libdir, "-L" + cuda + "/lib64", "-lcudart",
                        "-Wl,-rpath," + cuda + "/lib64"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def _problem(case, golden):
    if case == "lih":
        g = golden["lih"]
        model = QCModel(g["L"], integral_map(g["integrals"]), g["nelec"])
        mpo = make_mpo(model)
        _, mps = run_dmrg(model, mpo, SweepParams(nsweeps=2, max_bond_dimension=100), nelec=g["nelec"])
        site, Mmax, nelec = 1, 100, g["nelec"]
    else:
        model = QCModel(6, synthetic_integral_map(6, seed=3), 6)
        mpo = make_mpo(model)
        mps = initial_state(model, mpo, SweepParams(init_bond_dimension=16, seed=11), 6, 0)
        site, Mmax, nelec = 2, 8, 6
    L = model.L
    left = R.left_boundary(mps[0])
    for i in range(site):
        t = R.left_normalize_and_return(mps[i])
        R.multiply_from_left(mps[i + 1], t)
        left = R.overlap_mpo_left_step(mps[i], mps[i], left, mpo[i])
    right = R.right_boundary(mps[L - 1])
    for i in range(L - 1, site + 1, -1):
        right = R.overlap_mpo_right_step(mps[i], mps[i], right, mpo[i])
    return model, mpo, mps, site, left, right, Mmax


@pytest.mark.parametrize("case", ["lih", "random6"])
def test_cpp_host_runs_a_microiteration(case, golden, host_exe, tmp_path):
    model, mpo, mps, site, left, right, Mmax = _problem(case, golden)
    tol, maxiter, cutoff = 1e-10, 10, 1e-16
    ts = make_ts_cache_mpo(mpo, model.phys)[site]
    inp, outp = tmp_path / "in.bin", tmp_path / "out.bin"
    with open(inp, "wb") as f:
        _index(f, "phys", model.phys)
        _tensor(f, "A", mps[site])
        _tensor(f, "B", mps[site + 1])
        _boundary(f, "L", left)
        _boundary(f, "R", right)
        _mpo(f, "ts", N.FMpo(ts))
        _mpo(f, "W", N.FMpo(mpo[site]))
        for k, v in (("tol", tol), ("maxiter", maxiter), ("Mmax", Mmax), ("cutoff", cutoff)):
            _put(f, k, np.array([float(v)]))
    r = subprocess.run([str(host_exe), str(inp), str(outp)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    got = _read(outp)
    energy, tw, tf, sev, bond = got["scalars"]
    # the oracle's microiteration on the same inputs
    ots = oracle_twosite(mpo[site], mpo[site + 1], model.phys, model.phys)
    psi = R.make_two_site_mps(mps[site], mps[site + 1])
    theta, u, iters = R.jcd_solve(lambda x: R.site_hamil2(x, left, right, ots), psi, tol, maxiter)
    u.make_left_paired()
    A0, B0 = mps[site], mps[site + 1]
    _, tst = R.unreduce_left(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, u.data)
    A, B, tr = R.split_mps(tst, A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, Mmax, cutoff, True)
    newL = R.overlap_mpo_left_step(A, A, left, mpo[site])
    assert abs(energy - theta) <= 1e-10, (energy, theta)
    assert int(got["iters"][0]) == iters
    assert int(bond) == tr.bond_dimension
    assert abs(tw - tr.truncated_weight) <= 1e-8 * tr.truncated_weight + 1e-15
    if case == "lih":
        assert abs(energy + mpo.core_energy - golden["lih"]["energy"]) < 1e-9
    # gauge-invariant checks of the new tensors and boundary
    lay = N.BoundaryLayout.of(newL)
    assert list(got["L2.blk_ptr"]) == list(lay.ptr)
    assert np.array_equal(got["L2.q"], lay.q[:len(got["L2.q"])])
    assert np.array_equal(got["L2.rows"], lay.rows[:len(got["L2.rows"])])
    assert np.array_equal(got["L2.cols"], lay.cols[:len(got["L2.cols"])])
    data = got["L2.data"]
    for k, ((lc, rc), (rr, cc), off) in enumerate(zip(lay.keys, lay.shapes, got["L2.off"])):
        b = int(np.searchsorted(lay.ptr, k, side="right") - 1)
        want = np.linalg.norm(newL[b].blocks[newL[b].find_block(lc, rc)])
        have = np.linalg.norm(data[int(off):int(off) + rr * cc])
        assert abs(have - want) <= 1e-10 * max(want, 1.0), (k, have, want)
    theta_ref = R.two_site_theta(A, B)
    # A'B' from the host's tensors
    from oracle.qn import BlockMatrix as OBM
    def unpack(prefix):
        q, rows, cols, data = got[prefix + ".q"], got[prefix + ".rows"], got[prefix + ".cols"], got[prefix + ".data"]
        bm, o = OBM(), 0
        for k in range(len(rows)):
            r_, c_ = int(rows[k]), int(cols[k])
            bm.insert_block(data[o:o + r_ * c_].reshape((c_, r_)).T.copy(), (int(q[4 * k]), int(q[4 * k + 1])),
                            (int(q[4 * k + 2]), int(q[4 * k + 3])))
            o += r_ * c_
        return bm
    A2 = R.MPSTensor(A.phys_i, A.left_i, A.right_i, unpack("A2"), R.LEFT_PAIRED)
    B2 = R.MPSTensor(B.phys_i, B.left_i, B.right_i, unpack("B2"), R.LEFT_PAIRED)
    th = R.two_site_theta(A2, B2)
    scale = theta_ref.norm()
    # an eigenvector is defined up to its sign: fix it by the overlap of the two products
    ovl = sum(float(np.sum(b * th.blocks[th.find_block(*k)])) for k, b in zip(theta_ref.keys, theta_ref.blocks)
              if th.find_block(*k) < th.n_blocks())
    sgn = 1.0 if ovl >= 0 else -1.0
    for key in set(theta_ref.keys) | set(th.keys):
        pa, pb = th.find_block(*key), theta_ref.find_block(*key)
        xa = th.blocks[pa] if pa < th.n_blocks() else 0.0
        xb = theta_ref.blocks[pb] if pb < theta_ref.n_blocks() else 0.0
        assert np.linalg.norm(np.asarray(xa) - sgn * np.asarray(xb)) <= 1e-10 * scale, key
