"""Host-side interpreter of exported plan task tables (test infrastructure).

Executes the ZERO / AXPY / GEMM / DOT stages of a native plan with numpy so the
plan builder can be checked against the oracle without a GPU.  It is a
checker of the task tables, not an execution path of the library.
"""
import numpy as np


def _view(buf, off, ld, rows, cols):
    # column-major (rows x cols) view with leading dimension ld
    return np.lib.stride_tricks.as_strided(buf[off:], shape=(rows, cols), strides=(8, 8 * ld))


def run_plan(plan, bufs, images=False, nprod=6):
    """images=True runs the GEMM stages through the BF16x3 image-executor tables
    (nprod=3: the BF16x2 form's three slice products)."""
    for si, st in enumerate(plan.stages()):
        heavy = set()
        if images and st[0] in ("gemm", "axpy"):
            tab = plan.stage_images(si)
            if len(tab["tiles"]):
                run_gemm_images(tab, bufs, plan.image_bytes, nprod)
                if st[0] == "gemm":
                    continue
                heavy = set(int(x) for x in tab["coltab"][0::2])   # outputs the dense groups wrote
        if st[0] == "zero":
            zbuf, zlen = st[1], st[2]
            bufs[zbuf][:zlen] = 0.0
        elif st[0] == "dot":
            # per-term dots against the output-adjoint tiles, then sums per MPO term
            od, td, w, tt, gbuf, ntt = st[1:]
            g = np.zeros(len(td))
            for o in od:
                dst_buf, dst_off, ldd, rows, cols, tb, te = [int(x) for x in o]
                Y = _view(bufs[dst_buf], dst_off, ldd, rows, cols)
                for t in range(tb, te):
                    sb, so, lds = [int(x) for x in td[t]]
                    g[t] = float(np.sum(_view(bufs[sb], so, lds, rows, cols) * Y))
            bufs[gbuf][:len(g)] = g
            out = np.zeros(ntt)
            np.add.at(out, tt, w * g)
            bufs[3][:ntt] = out
        elif st[0] == "axpy":
            od, td, ta = st[1], st[2], st[3]
            for o in od:
                dst_buf, dst_off, ldd, rows, cols, tb, te = [int(x) for x in o]
                if dst_off in heavy:
                    continue
                acc = np.zeros((rows, cols))
                for t in range(tb, te):
                    sb, so, lds = [int(x) for x in td[t]]
                    acc += ta[t] * _view(bufs[sb], so, lds, rows, cols)
                _view(bufs[dst_buf], dst_off, ldd, rows, cols)[:, :] = acc
        else:
            od, sd, sa = st[1], st[2], st[3]
            for o in od:
                cb, co, ldc, M, N, sb_, se = [int(x) for x in o]
                acc = np.zeros((M, N))
                for s in range(sb_, se):
                    ab, ta, ao, lda, bb, tb, bo, ldb, K = [int(x) for x in sd[s]]
                    A = _view(bufs[ab], ao, lda, K, M).T if ta else _view(bufs[ab], ao, lda, M, K)
                    B = _view(bufs[bb], bo, ldb, N, K).T if tb else _view(bufs[bb], bo, ldb, K, N)
                    acc += sa[s] * (A @ B)
                _view(bufs[cb], co, ldc, M, N)[:, :] = acc


def _bf16_slots(raw):
    """Decode an image byte array into one float per 2-byte BF16 slot."""
    u = np.frombuffer(raw.tobytes(), dtype=np.uint16).astype(np.uint32) << 16
    return u.view(np.float32).astype(np.float64)


PAIRS = [(0, 0), (0, 1), (1, 0), (0, 2), (1, 1), (2, 0)]   # the six BF16 slice products


def run_gemm_images(tab, bufs, image_bytes, nprod=6):
    """Execute the image-executor tables of one stage the way the kernels
    address them.  Per-call images are built with the FP64 value in slice 0
    and zero slices 1 and 2; constant images (coefficient matrices) hold the
    plan's real BF16 slices.  For every output tile each K-chunk's row groups
    are copied into a 128-row "shared memory" tile (rows the copy does not
    reach are NaN, as a stale shared-memory row would be garbage), the six
    slice products are summed, the segment is scaled by its coefficient and
    the tile's valid region is stored.  A check of the tables and of the
    kernels' index arithmetic, not an execution path."""
    img = np.zeros(image_bytes // 2)   # one slot per 2-byte element position
    cimg = _bf16_slots(tab["cimg"]) if len(tab["cimg"]) else np.zeros(1)

    def slot(img_off, G, c, s, r, k):
        return (img_off + ((c * 3 + s) * G + r // 8) * 512 + ((k % 32) // 8) * 128 + (r % 8) * 16 + (k % 8) * 2) // 2

    def panel_values(pn, r, k):
        src_off, img_off, src_buf, ld, R, K, kcontig, G = [int(x) for x in pn]
        ok = (r < R) & (k < K)
        if kcontig == 2:
            ix = tab["gather"][src_off + np.clip(k, 0, K - 1)] + r
        else:
            ix = src_off + np.where(kcontig, r * ld + k, r + k * ld)
        return np.where(ok, bufs[src_buf][np.where(ok, ix, 0)], 0.0)

    for pn in tab["panels"]:
        src_off, img_off, src_buf, ld, R, K, kcontig, G = [int(x) for x in pn]
        if img_off < 0:
            continue   # a panel no segment reads from an image
        kc = (K + 31) // 32
        r = np.arange(G * 8)[:, None]
        k = np.arange(kc * 32)[None, :]
        vals = panel_values(pn, r, k)
        assert img_off % 512 == 0 and img_off + kc * 3 * G * 512 <= image_bytes
        for s in range(3):
            img[slot(img_off, G, k // 32, s, r, k)] = vals if s == 0 else 0.0
    outs, segs, alpha = tab["outs"], tab["segs"], tab["alpha"]
    for (out, m0, n0, nt, sb, se) in tab["tiles"]:
        c_off, si, sj, c_buf, mrows, ncols, mode, rows, ctab, vrows = [int(x) for x in outs[out]]
        assert nt % 16 == 0 and 16 <= nt <= 128 and m0 % 128 == 0 and n0 % 8 == 0
        acc = np.zeros((128, nt))
        for s in range(sb, se):
            a_img, b_img, a_G, b_G, kc, flags, a_panel, a_c0 = [int(x) for x in segs[s]]
            bsrc = cimg if flags & 2 else img
            ngA, ngB = min(16, a_G - m0 // 8), min(nt // 8, b_G - n0 // 8)
            assert ngA > 0 and ngB > 0
            D = np.zeros((128, nt))
            kk = np.arange(32)[None, :]
            ra = np.arange(ngA * 8)[:, None]
            rb = np.arange(ngB * 8)[:, None]
            for c in range(kc):
                A = np.full((3, 128, 32), np.nan)
                B = np.full((3, nt, 32), np.nan)
                for sl in range(3):
                    A[sl, :ngA * 8] = img[slot(a_img, a_G, c, sl, m0 + ra, kk)]
                    B[sl, :ngB * 8] = bsrc[slot(b_img, b_G, c, sl, n0 + rb, kk)]
                for ia, ib in PAIRS[:nprod]:
                    D += A[ia] @ B[ib].T
            acc += alpha[s] * D
        i = np.arange(128)[:, None]
        j = np.arange(nt)[None, :]
        valid = (m0 + i < mrows) & (n0 + j < ncols)
        if mode == 1 and vrows > 0:
            # a pitch-`rows` run of which the first vrows rows of every column are stored
            valid &= (m0 + i) % rows < vrows
        assert np.all(np.isfinite(acc[valid]))
        if mode == 0:
            dst = c_off + (m0 + i) * si + (n0 + j) * sj
        else:
            e = m0 + i
            jj = ctab + np.minimum(n0 + j, ncols - 1)
            dst = tab["coltab"][2 * jj] + (e % rows) + (e // rows) * tab["coltab"][2 * jj + 1]
        bufs[c_buf][dst[valid]] = acc[valid]


def patch_cpu_plans(monkeypatch):
    """Run the MPS-level plans of ``qcmaquis_gb300.mps_ops`` on CPU tensors through
    this interpreter (no upload, no device): lets the Python layer's calls of the
    plans (their slots, layouts and offsets) be checked without a GPU."""
    from qcmaquis_gb300 import mps_ops as O
    from qcmaquis_gb300 import native as N

    def interp(plan, device, ket=None, left=None, out=None, s2=None, right=None):
        bufs = [None if t is None else t.numpy() for t in (ket, left, right, out)]
        bufs += [np.full(max(x, 1), np.nan) for x in plan.scratch] + [None]
        if s2 is not None:
            bufs[6] = s2.numpy()
        run_plan(plan, bufs)

    monkeypatch.setattr(O, "_run_fp64", interp)
    monkeypatch.setattr(N.Plan, "upload", lambda self: None)
