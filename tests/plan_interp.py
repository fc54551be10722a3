"""Host-side interpreter of exported plan task tables (test infrastructure).

Executes the ZERO / AXPY / GEMM stages of a native plan with numpy so the
plan builder can be checked against the oracle without a GPU.  It is a
checker of the task tables, not an execution path of the library.
"""
import numpy as np


def _view(buf, off, ld, rows, cols):
    # column-major (rows x cols) view with leading dimension ld
    return np.lib.stride_tricks.as_strided(buf[off:], shape=(rows, cols), strides=(8, 8 * ld))


def run_plan(plan, bufs):
    for st in plan.stages():
        if st[0] == "zero":
            zbuf, zlen = st[1], st[2]
            bufs[zbuf][:zlen] = 0.0
        elif st[0] == "axpy":
            od, td, ta = st[1], st[2], st[3]
            for o in od:
                dst_buf, dst_off, ldd, rows, cols, tb, te = [int(x) for x in o]
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
