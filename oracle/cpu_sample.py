"""Timed CPU sample of the oracle's sigma vector at the benchmark's full size
(test infrastructure: used only as the CPU baseline of the benchmark).

The oracle restates the reference's lbtm sigma vector
(``ct/non-abelian/site_hamil.hpp:57-147``): all boundary x MPS products
(``boundary_times_mps.hpp:163-209``), then for every right MPO bond index b2
the operator application (``lbtm_kernel``, ``micro_kernels.hpp:19-198``)
followed by the product with the right boundary (``gemm_trim``,
``gemm.hpp:178-204``).  Its FP64 block products run on numpy's BLAS with all
host threads; the operator application is a Python loop, as the reference's is
a scalar C++ loop over micro-axpys.

Boundaries of a bond dimension of 1024 cannot be built by the oracle in a
bounded CPU time, so the sample takes the boundary *layouts* of the benchmark
workload (from the plan builder's layout query, not timed) and fills them with
seeded random values: the work of one sigma does not depend on the values.
The sample evaluates every boundary x MPS product and then as many b2 columns
as fit in the time budget; its FLOP rate (oracle work counters / wall time) is
the baseline.
"""
from __future__ import annotations

import os
import time

import numpy as np

from . import dmrg_ref as R


def boundary_layouts(w):
    """Left boundary at the pair's left site and right boundary after it (layouts only)."""
    from qcmaquis_gb300 import native as N
    from qcmaquis_gb300.block_matrix import BlockMatrix
    from qcmaquis_gb300.symmetry import Index
    one = lambda c: BlockMatrix.from_indices(Index([(c, 1)]), Index([(c, 1)]), fill=1.0)
    Ll = N.BoundaryLayout.of([one((0, 0))])
    for i, t in enumerate(w.left_sites):
        Ll = N.plan_boundary_left(t.phys_i, t.left_i, t.right_i, N.Layout.of(t.data), Ll,
                                  N.FMpo(w.mpo[i])).out_layout()
    Rl = N.BoundaryLayout.of([one((w.nelec, 0))])
    for k in range(len(w.right_sites) - 1, -1, -1):
        t = w.right_sites[k]
        Rl = N.plan_boundary_right(t.phys_i, t.left_i, t.right_i, N.Layout.of(t.data), Rl,
                                   N.FMpo(w.mpo[w.site + 2 + k])).out_layout()
    return Ll, Rl


class SigmaSample:
    """The benchmark workload on the host (built once, not timed) and timed
    bounded samples of the oracle's sigma on it (see the module docstring)."""

    def __init__(self, L: int = 24, m: int = 1024, seed: int = 7):
        from qcmaquis_gb300.workloads import build_sigma_host
        t0 = time.time()
        self.L, self.m = L, m
        self.w = build_sigma_host(L=L, m=m)
        Ll, Rl = boundary_layouts(self.w)
        rng = np.random.default_rng(seed)
        self.left = Ll.unpack(rng.standard_normal(max(Ll.size, 1)))
        self.right = Rl.unpack(rng.standard_normal(max(Rl.size, 1)))
        self.setup_s = time.time() - t0

    def step(self, budget_s: float):
        """One sample: all boundary x MPS products, then b2 columns until the
        budget is spent.  Returns (flops, seconds, columns done)."""
        p = self.w.psi_host
        ket = R.MPSTensor(p.phys_i, p.left_i, p.right_i, p.data.copy(), R.LEFT_PAIRED)
        mpo = self.w.ts_mpo
        R.FLOPS.reset()
        t1 = time.time()
        # site_hamil_lbtm (ct/non-abelian/site_hamil.hpp:57-147), stopped after the budget
        phys = ket.phys_i
        out_left_i = R.index_product(phys, ket.left_i)
        rib = ket.right_i.copy()
        R.common_subset(out_left_i, rib)
        out_left_pb = R.ProductBasis(phys, ket.left_i)
        in_right_pb = R.ProductBasis(phys, ket.right_i, R.fuse_neg_first)
        ket.make_right_paired()
        T = R.boundary_mps_product(ket.data, self.left, mpo, ket.data.left_basis(), True)
        h = mpo.herm
        done = 0
        for b2 in range(mpo.col_dim):
            contr = R.lbtm_kernel(b2, T, mpo, ket.right_i, out_left_i, in_right_pb, out_left_pb)
            if h.right_skip(b2):
                Radj = self.right[h.right_conj(b2)].transpose()
                R.gemm_trim(contr, Radj, R.conjugate_phases(Radj, mpo, b2, False, True), False)
            else:
                R.gemm_trim(contr, self.right[b2], [1.0] * contr.n_blocks(), True)
            done += 1
            if time.time() - t1 > budget_s:
                break
        return R.FLOPS.gemm_flops + R.FLOPS.axpy_flops, time.time() - t1, done

    def describe(self, flops, dt, done, steps=1):
        return (f"numpy oracle sigma (lbtm), L={self.L} N={self.w.nelec} middle sites, m={self.m}: per step all "
                f"boundary x MPS products, then right MPO bond columns until the step budget ({done} of "
                f"{self.w.ts_mpo.col_dim} in the last step); {steps} step(s), {dt:.1f}s, {flops / 1e9:.1f} GFLOP; "
                f"boundary layouts of the workload with seeded random values (setup {self.setup_s:.0f}s, not "
                f"timed); BLAS threads = host cores")


def sigma_sample(L: int = 24, m: int = 1024, budget_s: float = 20.0, seed: int = 7):
    """One bounded sample as a cpu_baseline record."""
    s = SigmaSample(L, m, seed)
    flops, dt, done = s.step(budget_s)
    return {"value": flops / dt / 1e12, "unit": "TFLOP/s", "cores": os.cpu_count(), "kind": "port",
            "sample": s.describe(flops, dt, done)}


__all__ = ["SigmaSample", "sigma_sample", "boundary_layouts"]
