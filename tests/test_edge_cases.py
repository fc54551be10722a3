"""Edge cases of the plan builder and executors: the smallest problems (one
orbital pair, 1x1 blocks), sigma of a zero vector, oversized blocks, null and
out-of-range arguments, and a problem run through every precision form.

The CPU cases check the plan builder and the C ABI's argument checks; the GPU
cases (marked) run the executors on the same inputs."""
import ctypes as C

import numpy as np
import pytest

from qcmaquis_gb300 import native as N

from oracle import dmrg_ref as R
from plan_interp import run_plan
from test_oracle import _random_site_problem


def _plan(psi, left, right, ts, herm=True):
    psi = psi.copy().make_left_paired()
    lay = N.Layout.of(psi.data)
    Ll, Rl = N.BoundaryLayout.of(left), N.BoundaryLayout.of(right)
    return psi, lay, Ll, Rl, N.plan_sigma(psi.phys_i, psi.left_i, psi.right_i, lay, Ll, Rl, N.FMpo(ts), herm)


def test_smallest_problem_plan_matches_oracle():
    """L=2, N=2 (the H2 case of the reference's tests): every block is tiny."""
    psi, left, right, ts, ots = _random_site_problem(L=2, N=2, m=4, site=0)
    psi, lay, Ll, Rl, p = _plan(psi, left, right, ts)
    bufs = [lay.pack(psi.data), Ll.pack(left), Rl.pack(right), np.zeros(p.out_elems)] + \
        [np.full(max(s, 1), np.nan) for s in p.scratch]
    run_plan(p, bufs, images=True)
    ref = lay.pack(R.site_hamil2(psi, left, right, ots).data)
    assert np.linalg.norm(bufs[3] - ref) <= 1e-7 * np.linalg.norm(ref)


def test_sigma_of_zero_vector_is_zero():
    psi, left, right, ts, ots = _random_site_problem(m=16)
    psi, lay, Ll, Rl, p = _plan(psi, left, right, ts)
    bufs = [np.zeros(lay.size), Ll.pack(left), Rl.pack(right), np.full(p.out_elems, np.nan)] + \
        [np.full(max(s, 1), np.nan) for s in p.scratch]
    run_plan(p, bufs)
    assert np.all(bufs[3] == 0.0)


def test_oversized_block_is_rejected():
    """Blocks of 2^31 elements or more are refused (the executors use 32-bit in-block offsets)."""
    psi, left, right, ts, ots = _random_site_problem(m=8)
    psi = psi.copy().make_left_paired()
    lay = N.Layout.of(psi.data)
    shapes = list(lay.shapes)
    shapes[0] = (1 << 16, 1 << 15)
    big = N.Layout(lay.keys, shapes)
    with pytest.raises(RuntimeError):
        N.plan_sigma(psi.phys_i, psi.left_i, psi.right_i, big, N.BoundaryLayout.of(left),
                     N.BoundaryLayout.of(right), N.FMpo(ts))


def test_null_and_out_of_range_arguments_are_rejected():
    lib = N.lib()
    assert lib.qcm_plan_sigma(None, None, None, None, None, None, None, 1, None) == -1
    assert lib.qcm_plan_sizes(None, None, None) == -1
    psi, left, right, ts, ots = _random_site_problem(m=8)
    _, _, _, _, p = _plan(psi, left, right, ts)
    cnt = np.zeros(4, dtype=np.int64)
    rc = lib.qcm_plan_stage_images(p.h, 99, cnt.ctypes.data_as(C.POINTER(C.c_int64)), None, None, None, None, None)
    assert rc == -5
    assert "range" in lib.qcm_last_error().decode()
    # more vectors than the allocation-free dot product holds
    out = C.c_double()
    rc = lib.qcm_multi_dot_noalloc(None, 33, None, 0, C.byref(out), None)
    assert rc in (-1, -5)


@pytest.mark.gpu
@pytest.mark.parametrize("L,N_,m,site", [(2, 2, 4, 0), (6, 6, 16, 2)])
def test_small_problems_every_precision_on_gpu(L, N_, m, site):
    """Tiny blocks through the FP64, TF32, BF16x3 (images) and BF16x3 (in-kernel split) executors."""
    import torch
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine
    psi, left, right, ts, ots = _random_site_problem(L=L, N=N_, m=m, site=site)
    psi = psi.copy().make_left_paired()
    ref = N.Layout.of(psi.data).pack(R.site_hamil2(psi, left, right, ots).data)
    eng = Engine("cuda:0")
    x, Lb, Rb = DeviceMPSTensor.from_host(psi), DeviceBoundary.from_host(left), DeviceBoundary.from_host(right)
    nref = np.linalg.norm(ref)
    for prec, images, tol in [(N.PREC_FP64, True, 1e-12), (N.PREC_TF32, True, 5e-3),
                              (N.PREC_BF16X3, True, 2e-5), (N.PREC_BF16X3, False, 2e-5)]:
        eng.use_images = images
        got = eng.site_hamil2(x, Lb, Rb, ts, precision=prec).data.cpu().numpy()
        assert np.linalg.norm(got - ref) <= tol * nref, (prec, images)


@pytest.mark.gpu
def test_zero_vector_on_gpu():
    import torch
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine
    psi, left, right, ts, ots = _random_site_problem(m=16)
    psi = psi.copy().make_left_paired()
    x = DeviceMPSTensor.from_host(psi)
    x.data.zero_()
    eng = Engine("cuda:0")
    for prec in (N.PREC_FP64, N.PREC_BF16X3):
        got = eng.site_hamil2(x, DeviceBoundary.from_host(left), DeviceBoundary.from_host(right), ts,
                              precision=prec).data
        assert torch.count_nonzero(got).item() == 0


def test_plan_cache_key_is_the_layout_content():
    """Sigma plans are cached by the content of their indices and layouts: equal
    content gives one key, any change of a block gives another."""
    from qcmaquis_gb300.engine import _digest
    psi, left, right, ts, ots = _random_site_problem(m=8)
    psi = psi.copy().make_left_paired()
    a, b = N.Layout.of(psi.data), N.Layout.of(psi.data)
    assert a is not b and _digest(psi.phys_i, a) == _digest(psi.phys_i, b)
    shapes = list(a.shapes)
    shapes[0] = (shapes[0][0] + 1, shapes[0][1])
    assert _digest(psi.phys_i, a) != _digest(psi.phys_i, N.Layout(a.keys, shapes))
    La, Lb = N.BoundaryLayout.of(left), N.BoundaryLayout.of(left)
    assert _digest(La) == _digest(Lb) != _digest(N.BoundaryLayout.of(right))


def test_plan_shape_options_keep_sigma_and_change_the_plan():
    """Plan-shape options (the autotuner's knobs) change the split-K and dense-group
    tables, never the sigma; the shape key ignores block values and offsets."""
    from qcmaquis_gb300.autotune import shape_key
    psi, left, right, ts, ots = _random_site_problem(L=6, N=6, m=24, site=2)
    psi = psi.copy().make_left_paired()
    lay, Ll, Rl = N.Layout.of(psi.data), N.BoundaryLayout.of(left), N.BoundaryLayout.of(right)
    ref = lay.pack(R.site_hamil2(psi, left, right, ots).data)
    outs = []
    for sk, dm in [(0, 0), (2, 8), (4, 16)]:
        p = N.plan_sigma(psi.phys_i, psi.left_i, psi.right_i, lay, Ll, Rl, N.FMpo(ts), True,
                         split_k_segs=sk, dense_min_terms=dm)
        bufs = [lay.pack(psi.data), Ll.pack(left), Rl.pack(right), np.full(p.out_elems, np.nan)] + \
            [np.full(max(s, 1), np.nan) for s in p.scratch]
        run_plan(p, bufs, images=True)
        assert np.linalg.norm(bufs[3] - ref) <= 1e-7 * np.linalg.norm(ref)
        st = p.stages()
        outs.append((len(p.stage_images(4)["tiles"]), len(st[6][1]) if len(st) > 6 else 0))
    # lower thresholds: more dense-group tiles and more split-K outputs
    assert outs[1][0] > outs[0][0] and outs[1][1] > outs[0][1]
    with pytest.raises(RuntimeError):
        N.plan_sigma(psi.phys_i, psi.left_i, psi.right_i, lay, Ll, Rl, N.FMpo(ts), True, split_k_segs=1)
    assert shape_key(lay, Ll, Rl, ts, 2) == shape_key(N.Layout.of(psi.data), Ll, Rl, ts, 2)
    assert shape_key(lay, Ll, Rl, ts, 2) != shape_key(lay, Ll, Rl, ts, 0)


def test_tile_width_and_k1_schedule_options_keep_sigma():
    """The autotuner's tile-shape and schedule knobs: no tile wider than n_tile_max (so
    at least as many tiles), the K1 A-resident schedule reorders K1's tiles, the sigma is unchanged
    (image tables interpreted on the CPU); invalid values are refused."""
    psi, left, right, ts, ots = _random_site_problem(L=6, N=6, m=64, site=2)
    psi = psi.copy().make_left_paired()
    lay, Ll, Rl = N.Layout.of(psi.data), N.BoundaryLayout.of(left), N.BoundaryLayout.of(right)
    ref = lay.pack(R.site_hamil2(psi, left, right, ots).data)
    tiles = {}
    for ntm, k1s in [(0, 0), (32, 0), (16, 0), (0, 1)]:
        p = N.plan_sigma(psi.phys_i, psi.left_i, psi.right_i, lay, Ll, Rl, N.FMpo(ts), True,
                         n_tile_max=ntm, k1_schedule=k1s)
        bufs = [lay.pack(psi.data), Ll.pack(left), Rl.pack(right), np.full(p.out_elems, np.nan)] + \
            [np.full(max(s, 1), np.nan) for s in p.scratch]
        run_plan(p, bufs, images=True)
        assert np.linalg.norm(bufs[3] - ref) <= 1e-7 * np.linalg.norm(ref)
        tabs = [p.stage_images(i)["tiles"] for i, k in enumerate(p.stage_kinds()) if k == "gemm"]
        tiles[(ntm, k1s)] = sum(len(t) for t in tabs)
        # every tile at most n_tile_max wide (column 3 of a tile: its N width)
        assert max(int(t[3]) for tab in tabs for t in tab) <= (ntm or 128)
    assert tiles[(16, 0)] >= tiles[(32, 0)] >= tiles[(0, 0)]
    assert tiles[(0, 1)] == tiles[(0, 0)]
    for bad in ({"n_tile_max": 24}, {"n_tile_max": 256}, {"k1_schedule": 2}):
        with pytest.raises(RuntimeError):
            N.plan_sigma(psi.phys_i, psi.left_i, psi.right_i, lay, Ll, Rl, N.FMpo(ts), True, **bad)


@pytest.mark.gpu
def test_autotuned_engine_gives_the_same_sigma(tmp_path):
    import torch
    from qcmaquis_gb300.autotune import Autotuner
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine
    psi, left, right, ts, ots = _random_site_problem(L=6, N=6, m=24, site=2)
    psi = psi.copy().make_left_paired()
    x, Lb, Rb = DeviceMPSTensor.from_host(psi), DeviceBoundary.from_host(left), DeviceBoundary.from_host(right)
    a = Engine("cuda:0", precision=N.PREC_BF16X3)
    b = Engine("cuda:0", precision=N.PREC_BF16X3)
    b.autotuner = Autotuner(path=str(tmp_path / "tune.json"), candidates=[(4, 16), (32, 64)], reps=2)
    # the tile-width and K1-schedule candidates are measured too (tensor-core forms)
    sa = a.site_hamil2(x, Lb, Rb, ts).data
    sb = b.site_hamil2(x, Lb, Rb, ts).data
    assert torch.linalg.norm(sa - sb).item() <= 1e-5 * torch.linalg.norm(sa).item()
    assert len(Autotuner(path=str(tmp_path / "tune.json")).table) == 1


@pytest.mark.gpu
def test_bf16x2_form_on_gpu():
    import torch
    from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine
    psi, left, right, ts, ots = _random_site_problem(L=6, N=6, m=24, site=2)
    psi = psi.copy().make_left_paired()
    ref = N.Layout.of(psi.data).pack(R.site_hamil2(psi, left, right, ots).data)
    x, Lb, Rb = DeviceMPSTensor.from_host(psi), DeviceBoundary.from_host(left), DeviceBoundary.from_host(right)
    err = {}
    for prec in (N.PREC_BF16X2, N.PREC_BF16X3):
        got = Engine("cuda:0", precision=prec).site_hamil2(x, Lb, Rb, ts).data.cpu().numpy()
        err[prec] = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    # the three products with i + j <= 1: two-slice accuracy, looser than BF16x3
    assert err[N.PREC_BF16X2] < 1e-4 and err[N.PREC_BF16X2] > err[N.PREC_BF16X3]
