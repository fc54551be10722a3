"""Batching: one merged plan for several independent sigma problems
(``qcm_plan_merge``).  Its task tables are the problems' tables moved to each
problem's slice of shared buffers, so running it gives every problem's sigma
exactly as its own plan does -- checked here through the task-table interpreter
(FP64 tables and BF16x3 image tables) and on the GPU against separate runs."""
import numpy as np
import pytest

from qcmaquis_gb300 import native as N

from oracle import dmrg_ref as R
from plan_interp import run_plan
from test_oracle import _random_site_problem


def _problems():
    out = []
    for (L, Ne, m, site, seed) in [(6, 6, 16, 2, 3), (6, 6, 12, 1, 4), (5, 4, 10, 1, 5)]:
        psi, left, right, ts, ots = _random_site_problem(L=L, N=Ne, m=m, site=site, seed=seed)
        psi = psi.copy().make_left_paired()
        lay, Ll, Rl = N.Layout.of(psi.data), N.BoundaryLayout.of(left), N.BoundaryLayout.of(right)
        p = N.plan_sigma(psi.phys_i, psi.left_i, psi.right_i, lay, Ll, Rl, N.FMpo(ts), True)
        out.append((psi, left, right, ots, lay, Ll, Rl, p))
    return out


def _merged(probs):
    offs, ket, lft, rgt, outn = [], 0, 0, 0, 0
    for psi, left, right, ts, lay, Ll, Rl, p in probs:
        offs.append((ket, lft, rgt, outn))
        ket += max(lay.size, 1)
        lft += max(Ll.size, 1)
        rgt += max(Rl.size, 1)
        outn += max(p.out_elems, 1)
    return N.plan_merge([pr[-1] for pr in probs], offs), offs, (ket, lft, rgt, outn)


@pytest.mark.parametrize("images", [False, True])
def test_merged_plan_gives_every_problems_sigma(images):
    probs = _problems()
    mp, offs, (nk, nl, nr, no) = _merged(probs)
    ket, lb, rb = np.zeros(nk), np.zeros(nl), np.zeros(nr)
    for (psi, left, right, ts, lay, Ll, Rl, p), (ko, lo, ro, oo) in zip(probs, offs):
        ket[ko:ko + lay.size] = lay.pack(psi.data)
        lb[lo:lo + Ll.size] = Ll.pack(left)
        rb[ro:ro + Rl.size] = Rl.pack(right)
    bufs = [ket, lb, rb, np.full(max(no, 1), np.nan)] + [np.full(max(s, 1), np.nan) for s in mp.scratch]
    run_plan(mp, bufs, images=images)
    assert mp.image_bytes >= max(pr[-1].image_bytes for pr in probs)
    for (psi, left, right, ts, lay, Ll, Rl, p), (ko, lo, ro, oo) in zip(probs, offs):
        own = [lay.pack(psi.data), Ll.pack(left), Rl.pack(right), np.full(max(p.out_elems, 1), np.nan)] + \
            [np.full(max(s, 1), np.nan) for s in p.scratch]
        run_plan(p, own, images=images)
        got = bufs[3][oo:oo + p.out_elems]
        assert np.array_equal(got, own[3][:p.out_elems])
        ref = lay.pack(R.site_hamil2(psi, left, right, ts).data)
        assert np.linalg.norm(got - ref) <= (2e-5 if images else 1e-12) * np.linalg.norm(ref)


def test_only_sigma_plans_merge():
    probs = _problems()
    psi, left, right, ts, lay, Ll, Rl, p = probs[0]
    from qcmaquis_gb300.mpo import make_mpo
    bl = N.plan_boundary_left(psi.phys_i, psi.left_i, psi.right_i, lay, Ll, N.FMpo(ts))
    with pytest.raises(RuntimeError):
        N.plan_merge([p, bl], [(0, 0, 0, 0), (0, 0, 0, 0)])


# ------------------------------------------------------------------ GPU
def _device_problems(engine):
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor
    out = []
    for psi, left, right, ts, lay, Ll, Rl, p in _problems():
        out.append((DeviceMPSTensor.from_host(psi), DeviceBoundary.from_host(left), DeviceBoundary.from_host(right),
                    ts))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("prec", [N.PREC_FP64, N.PREC_BF16X3])
def test_gpu_batched_sigma_equals_separate_runs(prec):
    import torch
    from qcmaquis_gb300.batch import BatchedSigma
    from qcmaquis_gb300.engine import Engine
    eng = Engine("cuda:0", precision=prec)
    probs = _device_problems(eng)
    bs = BatchedSigma(eng, probs)
    got = bs.unpack(bs.apply(bs.pack([p[0].data for p in probs])))
    for (ket, L, R, ts), g in zip(probs, got):
        want = eng.site_hamil2(ket, L, R, ts).data
        assert torch.linalg.norm(g - want).item() <= 1e-12 * torch.linalg.norm(want).item()
    # the captured graph replays the same sigma
    bs.capture()
    x = bs.pack([p[0].data for p in probs])
    assert torch.equal(bs.apply_graph(x), bs.apply(x))


@pytest.mark.gpu
def test_gpu_batched_davidson_equals_separate_solves():
    from qcmaquis_gb300.batch import BatchedSigma, solve_jcd_batched
    from qcmaquis_gb300.engine import Engine, SiteProblem
    from qcmaquis_gb300.jd import solve_ietl_jcd
    eng = Engine("cuda:0")
    probs = _device_problems(eng)
    bs = BatchedSigma(eng, probs)
    theta, u, iters = solve_jcd_batched(bs, bs.pack([p[0].data for p in probs]), tol=1e-8, maxiter=8)
    for k, (ket, L, R, ts) in enumerate(probs):
        th, uk, it = solve_ietl_jcd(SiteProblem(eng, L, R, ts), ket, 1e-8, 8)
        assert abs(theta[k] - th) < 1e-10
        assert iters[k] == it
        a, b = bs.unpack(u)[k], uk.data
        assert abs(abs(float((a @ b).item())) - float((a @ a).item()) ** 0.5 * float((b @ b).item()) ** 0.5) < 1e-8
