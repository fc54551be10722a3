"""The batched FP64 one-sided Jacobi SVD (``qcm_svd_*``) and the device truncation cut
(``qcm_truncation_cut``) against numpy's LAPACK and the oracle's ``svd_truncate`` /
``heev_truncate`` cut (``block_matrix_algorithms.h:163-333, 387-440``).

Tolerances: singular values within 1e-13 of the largest singular value of their
block (and 1e-12 relative for values above 1e-6 of it); U S Vt reproduces the
block to 1e-13 of its norm; U and Vt orthonormal to 1e-12; the cut's keep
counts and bond dimension exact, its weights within 1e-10 relative (absolute
1e-28 / 1e-14 for weights made only of rounding-level values)."""
import numpy as np
import pytest
import torch

from oracle import dmrg_ref as R
from oracle.qn import BlockMatrix

pytestmark = pytest.mark.gpu

SHAPES = [(7, 7), (12, 5), (5, 12), (1, 9), (9, 1), (1, 1), (0, 4), (64, 63), (63, 64), (130, 130), (460, 451)]


def _blocks(seed=0, grade=10.0):
    rng = np.random.default_rng(seed)
    out = []
    for r, c in SHAPES:
        a = rng.standard_normal((r, c))
        if min(r, c) > 1:
            a = a @ np.diag(np.logspace(0, -grade, c))
        out.append(a)
    return out


def _run(blocks, panel_width=None):
    from qcmaquis_gb300 import native as N
    offs = np.cumsum([0] + [b.size for b in blocks])
    flat = np.concatenate([np.ravel(b, order="F") for b in blocks] + [np.zeros(1)])
    src = torch.tensor(flat, dtype=torch.float64, device="cuda")
    svd = N.BatchedSVD([b.shape for b in blocks], offs[:-1], panel_width=panel_width)
    svd.run(src, torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return svd


def _check_svd(svd, blocks):
    for k, a in enumerate(blocks):
        r, c = a.shape
        if min(r, c) == 0:
            continue
        U, S, Vt = svd.u(k).cpu().numpy(), svd.s(k).cpu().numpy(), svd.vt(k).cpu().numpy()
        ref = np.linalg.svd(a, compute_uv=False)
        s0 = ref[0]
        assert np.all(np.diff(S) <= 0), k
        assert np.max(np.abs(S - ref)) <= 1e-13 * s0, (k, np.max(np.abs(S - ref)) / s0)
        big = ref > 1e-6 * s0
        assert np.max(np.abs(S[big] - ref[big]) / ref[big]) <= 1e-12, k
        assert np.linalg.norm(U @ np.diag(S) @ Vt - a) <= 1e-13 * np.linalg.norm(a), k
        nz = S > 1e-13 * s0
        assert np.allclose(U[:, nz].T @ U[:, nz], np.eye(int(nz.sum())), atol=1e-12), k
        assert np.allclose(Vt[nz] @ Vt[nz].T, np.eye(int(nz.sum())), atol=1e-12), k



@pytest.mark.parametrize("bw", [0, 2, 4, 8, 16])
def test_every_panel_width_matches_lapack(bw):
    """The panel rounds (bw columns per panel, each panel pair swept in shared memory)
    and the single-column rounds (bw = 0) give the same factorisation: graded,
    rank-deficient and tall / wide blocks, column counts that are not multiples of
    the panel width, one batch."""
    rng = np.random.default_rng(5)
    blocks = _blocks(seed=2)
    if bw == 16:
        # two 16-column panels of W and V of a 460 x 451 block exceed shared memory
        blocks = [a if a.shape != (460, 451) else rng.standard_normal((230, 180)) for a in blocks]
    # exactly rank 3 and rank 40 blocks (the rest of the spectrum is rounding)
    blocks.append(rng.standard_normal((50, 3)) @ rng.standard_normal((3, 37)))
    blocks.append(rng.standard_normal((200, 40)) @ rng.standard_normal((40, 90)))
    svd = _run(blocks, panel_width=bw)
    assert svd.panel_width() == bw
    assert 1 <= svd.sweeps() <= 40
    _check_svd(svd, blocks)


def test_default_panel_width_is_the_widest_that_fits():
    from qcmaquis_gb300 import native as N
    assert N.BatchedSVD([(200, 150), (5, 3)], [0, 200 * 150]).panel_width() == 16
    assert N.BatchedSVD([(460, 451), (5, 3)], [0, 460 * 451]).panel_width() == 8
    assert N.BatchedSVD([(1200, 40)], [0]).panel_width() == 8
    assert N.BatchedSVD([(5000, 30)], [0]).panel_width() == 0
    assert N.BatchedSVD([(20000, 3)], [0]).panel_width() == 0


def test_batched_svd_matches_lapack():
    blocks = _blocks()
    svd = _run(blocks)
    assert 1 <= svd.sweeps() <= 40
    for k, a in enumerate(blocks):
        r, c = a.shape
        kk = min(r, c)
        if kk == 0:
            continue
        U, S, Vt = svd.u(k).cpu().numpy(), svd.s(k).cpu().numpy(), svd.vt(k).cpu().numpy()
        ref = np.linalg.svd(a, compute_uv=False)
        s0 = ref[0]
        assert np.all(np.diff(S) <= 0), k
        assert np.max(np.abs(S - ref)) <= 1e-13 * s0, (k, np.max(np.abs(S - ref)) / s0)
        big = ref > 1e-6 * s0
        assert np.max(np.abs(S[big] - ref[big]) / ref[big]) <= 1e-12, k
        assert np.linalg.norm(U @ np.diag(S) @ Vt - a) <= 1e-13 * np.linalg.norm(a), k
        nz = S > 1e-13 * s0
        assert np.allclose(U[:, nz].T @ U[:, nz], np.eye(int(nz.sum())), atol=1e-12), k
        assert np.allclose(Vt[nz] @ Vt[nz].T, np.eye(int(nz.sum())), atol=1e-12), k


def test_batched_svd_is_repeatable():
    blocks = _blocks(seed=3)
    a, b = _run(blocks), _run(blocks)
    assert torch.equal(a.S, b.S) and torch.equal(a.U, b.U) and torch.equal(a.Vt, b.Vt)


@pytest.mark.parametrize("Mmax,cutoff", [(20, 1e-16), (400, 1e-8), (5, 1e-3), (10_000, 1e-16)])
def test_device_cut_matches_oracle_svd_truncate(Mmax, cutoff):
    blocks = [b for b in _blocks(seed=1, grade=14.0) if min(b.shape) > 0]
    svd = _run(blocks)
    keep, tr = svd.cut(Mmax, cutoff, 0, torch.cuda.current_stream().cuda_stream)
    M = BlockMatrix()
    for k, b in enumerate(blocks):
        M.insert_block(b, (k, 0), (k, 0))
    _, _, _, ref = R.svd_truncate(M, cutoff, Mmax)
    # the oracle lists blocks in DualIndex (descending key) order
    assert int(tr.bond_dimension) == ref.bond_dimension
    assert sum(int(x) for x in keep) == ref.bond_dimension
    # discarded values at the rounding level (below 1e-16 s0) are known only to about
    # 1e-16 s0 in absolute terms, so their weight (~1e-32) and fraction (~1e-16) are
    # compared absolutely there
    assert abs(tr.truncated_weight - ref.truncated_weight) <= 1e-10 * ref.truncated_weight + 1e-28
    assert abs(tr.truncated_fraction - ref.truncated_fraction) <= 1e-10 * ref.truncated_fraction + 1e-14
    assert abs(tr.smallest_ev - ref.smallest_ev) <= 1e-12 * ref.smallest_ev + 1e-300


def test_device_cut_on_density_matrix_eigenvalues():
    rng = np.random.default_rng(4)
    thetas = [rng.standard_normal((n, n + 3)) @ np.diag(np.logspace(0, -6, n + 3)) for n in (30, 17, 44)]
    rhos = [t @ t.T for t in thetas]
    svd = _run(rhos)
    keep, tr = svd.cut(40, 1e-12, 1, torch.cuda.current_stream().cuda_stream)
    M = BlockMatrix()
    for k, b in enumerate(rhos):
        M.insert_block(b, (k, 0), (k, 0))
    Uref, _, ref = R.heev_truncate(M, 1e-12, 40)
    assert int(tr.bond_dimension) == ref.bond_dimension
    assert tr.truncated_weight == tr.truncated_fraction
    assert abs(tr.truncated_fraction - ref.truncated_fraction) <= 1e-9 * ref.truncated_fraction
    for k, rho in enumerate(rhos):
        w = np.sort(np.linalg.eigvalsh(rho))[::-1]
        assert np.max(np.abs(svd.s(k).cpu().numpy() - w)) <= 1e-13 * w[0]
