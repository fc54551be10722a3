"""The density-matrix (heev) truncation of the two-site step
(``TwoSiteTensor::predict_split_l2r/r2l``, ``twositetensor.hpp:184-297``;
``heev_truncate``, ``block_matrix_algorithms.h:388-440``) and the bra-free
boundary contractions that feed its perturbation
(``left/right_boundary_tensor_mpo``, ``move_boundary.hpp:66-126``).

The reference's tests hold no golden vectors for this path, so the oracle is
pinned through its relations to the pinned paths: without noise the eigenvector
cut keeps the same subspace as the SVD cut (eigenvalues = squared singular
values, truncated fraction = SVD truncated weight), and contracting the
bra-free boundary with the bra gives the boundary step.  The plan builder's
tensor-MPO plans are checked against the oracle through the task-table
interpreter; the GPU cases (marked) check the device path against the oracle."""
import numpy as np
import pytest

from qcmaquis_gb300 import native as N
from qcmaquis_gb300.block_matrix import BlockMatrix
from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model import QCModel
from qcmaquis_gb300.mpo import make_mpo
from qcmaquis_gb300.symmetry import adjoin, index_product

from oracle import dmrg_ref as R
from oracle.sweep import SweepParams, initial_state
from plan_interp import run_plan


def _pair_problem(L=6, Ne=6, m=16, site=2, seed=3):
    """Two-site problem at (site, site+1) with the single-site MPO tensors:
    (two-site tensor, A0, B0, left boundary, right boundary, mpo)."""
    model = QCModel(L, synthetic_integral_map(L, seed=seed), Ne)
    mpo = make_mpo(model)
    mps = initial_state(model, mpo, SweepParams(init_bond_dimension=m, seed=11), Ne, 0)
    left = R.left_boundary(mps[0])
    for i in range(site):
        t = R.left_normalize_and_return(mps[i])
        R.multiply_from_left(mps[i + 1], t)
        left = R.overlap_mpo_left_step(mps[i], mps[i], left, mpo[i])
    right = R.right_boundary(mps[L - 1])
    for i in range(L - 1, site + 1, -1):
        right = R.overlap_mpo_right_step(mps[i], mps[i], right, mpo[i])
    psi = R.make_two_site_mps(mps[site], mps[site + 1])
    return model, mpo, mps, psi, left, right


def _tst(psi, A0, B0):
    u = psi.copy().make_left_paired()
    _, tst = R.unreduce_left(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, u.data)
    return tst


def _theta(A, B):
    return R.two_site_theta(A, B)


def _block_pairs(a: BlockMatrix, b: BlockMatrix):
    """(key, block of a, block of b) over the union of keys; a missing block is zeros."""
    for k in sorted(set(a.keys) | set(b.keys), reverse=True):
        pa, pb = a.find_block(*k), b.find_block(*k)
        xa = a.blocks[pa] if pa < a.n_blocks() else None
        xb = b.blocks[pb] if pb < b.n_blocks() else None
        yield k, (np.zeros_like(xb) if xa is None else xa), (np.zeros_like(xa) if xb is None else xb)


def _bm_close(a: BlockMatrix, b: BlockMatrix, tol):
    """Same blocks (missing blocks count as zeros) within tol * max norm."""
    scale = max(a.norm(), b.norm(), 1e-300)
    for k, xa, xb in _block_pairs(a, b):
        assert xa.shape == xb.shape, k
        assert np.linalg.norm(xa - xb) <= tol * scale, k


@pytest.mark.parametrize("l2r", [True, False])
def test_oracle_heev_without_noise_keeps_the_svd_subspace(l2r):
    model, mpo, mps, psi, left, right = _pair_problem()
    A0, B0 = mps[2], mps[3]
    tst = _tst(psi, A0, B0)
    Mmax = 10
    As, Bs, ts = R.split_mps(tst, A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, Mmax, 1e-16, l2r)
    Ah, Bh, th = R.predict_split_mps(tst, A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, Mmax, 1e-16, l2r,
                                     alpha=0.0, boundary=None)
    assert th.bond_dimension == ts.bond_dimension
    # the eigenvalue cut: fraction of discarded eigenvalues = SVD truncated weight
    assert abs(th.truncated_fraction - ts.truncated_weight) <= 1e-9 * ts.truncated_weight + 1e-15
    assert th.truncated_weight == th.truncated_fraction
    _bm_close(_theta(Ah, Bh), _theta(As, Bs), 1e-10)


def test_oracle_boundary_tensor_mpo_contracts_to_the_boundary_steps():
    """sum over the bra of left/right_boundary_tensor_mpo = overlap_mpo_left/right_step."""
    model, mpo, mps, psi, left, right = _pair_problem()
    A = mps[2].copy().make_left_paired()
    half = R.left_boundary_tensor_mpo(A, left, mpo[2])
    # the boundaries hold no blocks at the Hermitian-skipped bonds: compare the others
    ref = R.overlap_mpo_left_step(A, A, left, mpo[2])
    assert len(half) == mpo[2].col_dim
    for b2 in range(mpo[2].col_dim):
        if mpo[2].herm.right_skip(b2):
            continue
        got = R.su2_gemm(half[b2].transpose(), A.data, mpo[2].right_spin(b2).get())
        _bm_close(got, ref[b2], 1e-12)
    B = mps[3].copy()
    half = R.right_boundary_tensor_mpo(B, right, mpo[3])
    refr = R.overlap_mpo_right_step(B, B, right, mpo[3])
    Brp = B.copy().make_right_paired()
    assert len(half) == mpo[3].row_dim
    for b1 in range(mpo[3].row_dim):
        if mpo[3].herm.left_skip(b1):
            continue
        got = R.su2_gemm(half[b1], Brp.data.transpose(), mpo[3].left_spin(b1).get())
        _bm_close(got, refr[b1], 1e-12)


@pytest.mark.parametrize("l2r", [True, False])
def test_oracle_heev_with_noise_is_an_orthonormal_projection(l2r):
    model, mpo, mps, psi, left, right = _pair_problem()
    A0, B0 = mps[2], mps[3]
    tst = _tst(psi, A0, B0)
    both = R._reshape_left_to_both(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, tst)
    bnd, w = (left, mpo[2]) if l2r else (right, mpo[3])
    A, B, tr = R.predict_split_mps(tst, A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, 10, 1e-16, l2r,
                                   alpha=1e-2, boundary=bnd, mpo=w)
    An, Bn, _ = R.predict_split_mps(tst, A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, 10, 1e-16, l2r,
                                    alpha=0.0, boundary=None)
    # the kept factor is orthonormal (left-normalised A going right, right-normalised B going left)
    iso = A.copy().make_left_paired().data if l2r else B.copy().make_right_paired().data
    for b in iso.blocks:
        g = b.T @ b if l2r else b @ b.T
        assert np.allclose(g, np.eye(g.shape[0]), atol=1e-12)
    # the kept two-site state is theta's orthogonal projection onto the kept subspace
    kept = _theta(A, B)
    cross = sum(float(np.vdot(xk, xt - xk)) for _, xk, xt in _block_pairs(kept, both))
    assert abs(cross) <= 1e-12 * both.norm() ** 2
    assert 0 < tr.bond_dimension <= 11
    # the noise moves the kept subspace away from the noiseless one
    diff = np.sqrt(sum(np.linalg.norm(x - y) ** 2 for _, x, y in _block_pairs(kept, _theta(An, Bn))))
    assert diff > 1e-8 * both.norm()


@pytest.mark.parametrize("side", ["left", "right"])
def test_tensor_mpo_plans_match_oracle(side):
    """qcm_plan_boundary_tensor_mpo on the two-site tensor seen as one site, as the
    heev perturbation uses it, through the task-table interpreter."""
    model, mpo, mps, psi, left, right = _pair_problem()
    A0, B0 = mps[2], mps[3]
    tst = _tst(psi, A0, B0)
    both = R._reshape_left_to_both(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, tst)
    if side == "left":
        tmp = R.MPSTensor.from_block(A0.phys_i, A0.left_i, index_product(adjoin(B0.phys_i), B0.right_i), both,
                                     R.LEFT_PAIRED)
        ref = R.left_boundary_tensor_mpo(tmp, left, mpo[2])
        bnd, w = left, mpo[2]
    else:
        tmp = R.MPSTensor.from_block(B0.phys_i, index_product(A0.phys_i, A0.left_i), B0.right_i, both,
                                     R.RIGHT_PAIRED)
        ref = R.right_boundary_tensor_mpo(tmp, right, mpo[3])
        bnd, w = right, mpo[3]
    t = tmp.copy().make_left_paired()
    lay, Bl = N.Layout.of(t.data), N.BoundaryLayout.of(bnd)
    p = N.plan_boundary_tensor_mpo(t.phys_i, t.left_i, t.right_i, lay, Bl, N.FMpo(w), side, True)
    ol = p.out_layout()
    assert ol.aux == len(ref)
    bufs = [lay.pack(t.data), Bl.pack(bnd) if side == "left" else None, Bl.pack(bnd) if side == "right" else None,
            np.full(max(p.out_elems, 1), np.nan)] + [np.full(max(s, 1), np.nan) for s in p.scratch]
    run_plan(p, bufs)
    got = ol.unpack(bufs[3])
    assert [g.keys for g in got] == [r.keys for r in ref]
    assert np.allclose(ol.pack(ref), bufs[3][:ol.size], rtol=0, atol=1e-13)


def test_tensor_mpo_plan_rejects_a_bad_side():
    lib = N.lib()
    import ctypes as C
    h = C.c_void_p()
    assert lib.qcm_plan_boundary_tensor_mpo(None, None, None, None, None, None, 2, 1, C.byref(h)) != 0
    assert "side" in lib.qcm_last_error().decode()


def _run_interp(p, slots):
    bufs = [slots.get(i) for i in range(3)] + [np.full(max(p.out_elems, 1), np.nan)]
    bufs += [np.full(max(x, 1), np.nan) for x in p.scratch] + [None]
    run_plan(p, bufs)
    return bufs[3]


def _both_and_half(l2r):
    """The two-site problem's both-paired theta and the bra-free boundary product h
    its perturbation reads (as predict_split_mps builds them)."""
    model, mpo, mps, psi, left, right = _pair_problem()
    A0, B0 = mps[2], mps[3]
    both = R._reshape_left_to_both(A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, _tst(psi, A0, B0))
    if l2r:
        tmp = R.MPSTensor.from_block(A0.phys_i, A0.left_i, index_product(adjoin(B0.phys_i), B0.right_i), both,
                                     R.LEFT_PAIRED)
        half = R.left_boundary_tensor_mpo(tmp, left, mpo[2])
    else:
        tmp = R.MPSTensor.from_block(B0.phys_i, index_product(A0.phys_i, A0.left_i), B0.right_i, both,
                                     R.RIGHT_PAIRED)
        half = R.right_boundary_tensor_mpo(tmp, right, mpo[3])
    return both, half


@pytest.mark.parametrize("l2r", [True, False])
@pytest.mark.parametrize("alpha", [0.0, 1e-2])
def test_density_matrix_plan_matches_oracle(l2r, alpha):
    """qcm_plan_density_matrix = the oracle's rho with its noise term (predict_split_mps:
    theta theta^T or theta^T theta plus alpha h h^T on the blocks theta holds), layout
    block for block, values to 1e-13 relative, through the task-table interpreter."""
    both, half = _both_and_half(l2r)
    bt = both.transpose()
    ref = R.bm_gemm(both, bt) if l2r else R.bm_gemm(bt, both)
    for h in half:
        ht = h.transpose()
        tdm = R.bm_gemm(h, ht) if l2r else R.bm_gemm(ht, h)
        for (lc, rc), b in zip(tdm.keys, tdm.blocks):
            if both.find_block(lc, rc) == both.n_blocks():
                continue
            q = ref.find_block(lc, rc)
            if q == ref.n_blocks():
                ref.insert_block(alpha * b, lc, rc)
            else:
                ref.blocks[q] = ref.blocks[q] + alpha * b
    lay, hl = N.Layout.of(both), N.BoundaryLayout.of(half)
    p = N.plan_density_matrix(lay, l2r, hl, alpha)
    _, _, _, ol = N.out_tensor(p)
    assert list(ol.keys) == list(ref.keys)
    assert list(ol.shapes) == [b.shape for b in ref.blocks]
    got = _run_interp(p, {0: lay.pack(both), 2: hl.pack(half)})[:ol.size]
    want = ol.pack(ref)
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()
    if alpha:
        plain = N.plan_density_matrix(lay, l2r)
        # the noise adds products to the grouped GEMM (last column of an output: its segment end)
        assert plain.stages()[-1][1][-1][-1] < p.stages()[-1][1][-1][-1]


@pytest.mark.parametrize("ta,tb", [(False, False), (True, False), (False, True), (True, True)])
def test_block_gemm_plan_matches_oracle(ta, tb):
    """qcm_plan_block_gemm = bm_gemm of the (transposed where asked) operands."""
    both, _ = _both_and_half(True)
    bt = both.transpose()
    a = bt if ta else both       # op(A) = theta in every case
    b = both if tb else bt       # op(B) = theta^T
    ref = R.bm_gemm(both, bt)
    la, lb = N.Layout.of(a), N.Layout.of(b)
    p = N.plan_block_gemm(la, ta, lb, tb)
    _, _, _, ol = N.out_tensor(p)
    assert list(ol.keys) == list(ref.keys)
    got = _run_interp(p, {0: la.pack(a), 1: lb.pack(b)})[:ol.size]
    want = ol.pack(ref)
    assert np.abs(got - want).max() <= 1e-13 * np.abs(want).max()
    # a product with a factor of another shape: U^T theta for the heev cut's U
    U, _, _ = R.heev_truncate(ref, 1e-12, 6)
    lu = N.Layout.of(U)
    p = N.plan_block_gemm(lu, True, la if not ta else N.Layout.of(both), False)
    _, _, _, ol = N.out_tensor(p)
    ref2 = R.bm_gemm(U.transpose(), both)
    assert list(ol.keys) == list(ref2.keys)
    got = _run_interp(p, {0: lu.pack(U), 1: N.Layout.of(both).pack(both)})[:ol.size]
    assert np.abs(got - ol.pack(ref2)).max() <= 1e-13 * max(np.abs(ol.pack(ref2)).max(), 1e-300)


def test_block_gemm_plan_rejects_mismatched_inner_dimensions():
    both, _ = _both_and_half(True)
    lay = N.Layout.of(both)
    bad = N.Layout(lay.keys, [(r + 1, c) for r, c in lay.shapes])
    with pytest.raises(RuntimeError, match="inner dimensions"):
        N.plan_block_gemm(lay, False, bad, False)


@pytest.mark.parametrize("l2r", [True, False])
def test_heev_products_wiring_on_the_interpreter(l2r, monkeypatch):
    """The Python layer's density matrix and block products (mps_ops.density_matrix,
    mps_ops.gemm with transpose flags) on CPU tensors, their plans executed by the
    task-table interpreter in place of the device: slots, layouts and offsets as
    the GPU path passes them, values equal to the oracle's."""
    import types
    import torch
    from qcmaquis_gb300 import mps_ops as O
    from plan_interp import patch_cpu_plans
    patch_cpu_plans(monkeypatch)
    both, half = _both_and_half(l2r)
    lay, hl = N.Layout.of(both), N.BoundaryLayout.of(half)
    M = O._flat_dbm(lay, torch.from_numpy(lay.pack(both)))
    h = types.SimpleNamespace(layout=hl, data=torch.from_numpy(hl.pack(half)))
    alpha = 1e-2
    dm = O.density_matrix(M, l2r, h, alpha)
    bt = both.transpose()
    ref = R.bm_gemm(both, bt) if l2r else R.bm_gemm(bt, both)
    for hb in half:
        tdm = R.bm_gemm(hb, hb.transpose()) if l2r else R.bm_gemm(hb.transpose(), hb)
        for (lc, rc), b in zip(tdm.keys, tdm.blocks):
            if both.find_block(lc, rc) == both.n_blocks():
                continue
            q = ref.find_block(lc, rc)
            if q == ref.n_blocks():
                ref.insert_block(alpha * b, lc, rc)
            else:
                ref.blocks[q] = ref.blocks[q] + alpha * b
    assert dm.keys == ref.keys
    for a, b in zip(dm.blocks, ref.blocks):
        assert np.abs(a.numpy() - b).max() <= 1e-13 * np.abs(b).max()
    # the heev cut's factor products: U^T theta (l2r), theta U (r2l), U as the first
    # kk columns of each block of a packed factor buffer (as the batched SVD leaves it)
    U, _, _ = R.heev_truncate(ref, 1e-12, 6)
    keys, shapes, offs, flat, o = [], [], [], [], 0
    for (lc, rc), b in zip(U.keys, U.blocks):
        r, kk = b.shape
        full = np.concatenate([b, np.full((r, 2), np.nan)], axis=1)   # columns past kk never read
        keys.append((lc, rc)); shapes.append((r, kk)); offs.append(o)
        flat.append(np.ravel(full, order="F")); o += full.size
    Ud = O._flat_dbm(N.Layout(keys, shapes, offs), torch.from_numpy(np.concatenate(flat)))
    got = O.gemm(Ud, M, ta=True) if l2r else O.gemm(M, Ud)
    want = R.bm_gemm(U.transpose(), both) if l2r else R.bm_gemm(both, U)
    assert got.keys == want.keys
    for a, b in zip(got.blocks, want.blocks):
        assert np.abs(a.numpy() - b).max() <= 1e-13 * max(np.abs(b).max(), 1e-300)


def test_block_plans_on_empty_and_unmatched_inputs():
    """Empty operands and operands whose inner charges never agree give empty
    products (no blocks, nothing to run); a perturbation block outside theta's
    charges is not added."""
    empty = N.Layout([], [])
    for p in (N.plan_block_gemm(empty, False, empty, True), N.plan_density_matrix(empty, True),
              N.plan_density_matrix(empty, False)):
        _, _, _, lay = N.out_tensor(p)
        assert lay.keys == [] and p.out_elems == 0
    a = N.Layout([((2, 0), (1, 1))], [(3, 2)])
    b = N.Layout([((0, 0), (1, 1))], [(2, 4)])     # op(B) = B: inner charge (0, 0) never meets (1, 1)
    _, _, _, lay = N.out_tensor(N.plan_block_gemm(a, False, b, False))
    assert lay.keys == []
    _, _, _, lay = N.out_tensor(N.plan_block_gemm(a, True, b, True))   # (1,1)x(2,0) . (1,1)x(0,0): inner (2,0) vs (1,1)
    assert lay.keys == []
    # a half boundary whose only pair lands on charges theta does not hold adds nothing
    theta = N.Layout([((2, 0), (2, 0))], [(3, 3)])
    half = N.BoundaryLayout([N.Layout([((4, 0), (1, 1))], [(2, 5)])])
    p = N.plan_density_matrix(theta, True, half, 0.5)
    _, _, _, lay = N.out_tensor(p)
    assert lay.keys == [((2, 0), (2, 0))]
    x = np.arange(9.0)
    got = _run_interp(p, {0: x, 2: np.ones(10)})[:9].reshape(3, 3, order="F")
    X = x.reshape(3, 3, order="F")
    assert np.allclose(got, X @ X.T, rtol=0, atol=1e-13)


# ------------------------------------------------------------------ GPU
def _host_theta(A, B):
    """Two-site product of device tensors, on the host."""
    a = R.MPSTensor(A.phys_i, A.left_i, A.right_i, A.to_block_matrix(), R.LEFT_PAIRED)
    b = R.MPSTensor(B.phys_i, B.left_i, B.right_i, B.to_block_matrix(), R.LEFT_PAIRED)
    return R.two_site_theta(a, b)


@pytest.mark.gpu
@pytest.mark.parametrize("l2r", [True, False])
@pytest.mark.parametrize("alpha", [0.0, 1e-2])
def test_gpu_heev_split_matches_oracle(l2r, alpha):
    from qcmaquis_gb300 import mps_ops as O
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine
    model, mpo, mps, psi, left, right = _pair_problem(m=24)
    A0, B0 = mps[2], mps[3]
    tst = _tst(psi, A0, B0)
    bnd, w = (left, mpo[2]) if l2r else (right, mpo[3])
    Ar, Br, tr = R.predict_split_mps(tst, A0.phys_i, B0.phys_i, A0.left_i, B0.right_i, 12, 1e-16, l2r,
                                     alpha=alpha, boundary=bnd, mpo=w)
    eng = Engine("cuda:0")
    dA0 = DeviceMPSTensor.from_host(A0.copy().make_left_paired())
    dB0 = DeviceMPSTensor.from_host(B0.copy().make_left_paired())
    u = DeviceMPSTensor.from_host(psi.copy().make_left_paired())
    A, B, tg = O.split(u, dA0, dB0, 12, 1e-16, l2r, truncation="heev", alpha=alpha, engine=eng,
                       boundary=DeviceBoundary.from_host(bnd), mpo=w)
    assert tg.bond_dimension == tr.bond_dimension
    assert abs(tg.truncated_fraction - tr.truncated_fraction) <= 1e-8 * tr.truncated_fraction + 1e-14
    assert abs(tg.smallest_ev - tr.smallest_ev) <= 1e-8 * tr.smallest_ev + 1e-16
    _bm_close(_host_theta(A, B), R.two_site_theta(Ar, Br), 1e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("side", ["left", "right"])
def test_gpu_boundary_tensor_mpo_matches_oracle(side):
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine
    model, mpo, mps, psi, left, right = _pair_problem()
    t = mps[2] if side == "left" else mps[3]
    bnd, w = (left, mpo[2]) if side == "left" else (right, mpo[3])
    ref = (R.left_boundary_tensor_mpo if side == "left" else R.right_boundary_tensor_mpo)(t, bnd, w)
    eng = Engine("cuda:0")
    got = eng.boundary_tensor_mpo(DeviceMPSTensor.from_host(t.copy().make_left_paired()),
                                  DeviceBoundary.from_host(bnd), w, side)
    lay = got.layout
    assert np.allclose(lay.pack(ref), got.data.cpu().numpy()[:lay.size], rtol=0, atol=1e-13)


@pytest.mark.gpu
def test_gpu_heev_sweep_matches_oracle():
    """Two heev sweeps with the reference's noise schedule (alpha 1e-2 in the
    growth sweeps): per-sweep energies to 1e-10 Eh of the oracle's."""
    from qcmaquis_gb300 import sweep as G
    from oracle.sweep import SweepParams as OP, run_dmrg as oracle_dmrg
    L, Ne, m = 6, 6, 24
    model = QCModel(L, synthetic_integral_map(L, seed=3), Ne)
    mpo = make_mpo(model)
    gpu, _ = G.run_dmrg(model, mpo, G.SweepParams(nsweeps=2, max_bond_dimension=m, twosite_truncation="heev"),
                        nelec=Ne)
    ref, _ = oracle_dmrg(model, mpo, OP(nsweeps=2, max_bond_dimension=m, twosite_truncation="heev"), nelec=Ne)
    assert np.max(np.abs(np.array(gpu.energies) - np.array(ref.energies))) < 1e-10
    assert np.max(np.abs(np.array(gpu.sweep_energy) - np.array(ref.sweep_energy))) < 1e-10
    assert gpu.bond_dimension == ref.bond_dimension
