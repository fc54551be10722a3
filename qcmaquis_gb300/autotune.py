"""Autotuner of sigma-plan shapes, keyed on the block-size histogram.

Four plan-shape parameters of a sigma plan are measured instead of fixed:

- ``split_k_segs``: the largest number of block products summed into one K3
  output before the output is split into partial tiles;
- ``dense_min_terms``: the fewest K2 terms an output tile needs to join a dense
  tensor-core group;
- ``n_tile_max``: the widest N of a tensor-core tile (the tile shape of the
  image executor's block products; wider blocks are cut into balanced tiles);
- ``k1_schedule``: the block-to-CTA schedule of the K1 products (round robin,
  or contiguous cost-balanced ranges with each A tile resident in shared memory).

For a site problem the tuner builds the plan of every candidate, times ``reps``
sigma vectors of each with CUDA events (after a warm-up) and keeps the
fastest: first the (split_k_segs, dense_min_terms) grid, then, for the
tensor-core forms, the tile widths and the K1 schedule around the best pair.
The choice is stored under a key made of the problem's block-size histogram
(log2 buckets of the psi, left and right boundary blocks), the MPO bond
dimensions and the precision, so problems of the same shape -- the other sites
of a sweep once the bond dimensions have settled, the same system at a later
sweep, similar systems -- reuse it without measuring.  The table can be kept in
a JSON file.
"""
from __future__ import annotations

import hashlib
import json
import os
import time
from typing import Dict, Iterable, Optional, Tuple

import numpy as np
import torch

from . import native as N

CANDIDATES: Tuple[Tuple[int, int], ...] = tuple((sk, dm) for sk in (16, 32, 64) for dm in (32, 64, 128))
# tile widths and K1 schedules tried around the best (split_k_segs, dense_min_terms) pair
SHAPE_CANDIDATES: Tuple[Tuple[int, int], ...] = ((96, 0), (64, 0), (128, 1))
OPTION_KEYS = ("split_k_segs", "dense_min_terms", "n_tile_max", "k1_schedule")


def _histogram(rows: np.ndarray, cols: np.ndarray) -> list:
    e = np.maximum(rows.astype(np.int64) * cols.astype(np.int64), 1)
    b = np.floor(np.log2(e)).astype(np.int64)
    return np.bincount(b, minlength=40)[:40].tolist()


def shape_key(ket_layout, left_layout, right_layout, mpo, precision: int) -> str:
    """Digest of the problem's shape: block-size histograms, MPO bond dimensions, precision."""
    parts = {
        "psi": _histogram(ket_layout.rows, ket_layout.cols),
        "left": _histogram(left_layout.rows, left_layout.cols),
        "right": _histogram(right_layout.rows, right_layout.cols),
        "mpo": [int(mpo.row_dim), int(mpo.col_dim)],
        "precision": int(precision),
    }
    return hashlib.blake2b(json.dumps(parts, sort_keys=True).encode(), digest_size=12).hexdigest()


class Autotuner:
    """Measured plan-shape choices, keyed by ``shape_key``."""

    def __init__(self, path: Optional[str] = None, candidates: Iterable[Tuple[int, int]] = CANDIDATES,
                 reps: int = 3):
        self.path = path
        self.candidates = tuple(candidates)
        self.reps = reps
        self.table: Dict[str, dict] = {}
        if path and os.path.exists(path):
            with open(path) as f:
                self.table = json.load(f)

    def save(self):
        if self.path:
            tmp = self.path + ".new"
            with open(tmp, "w") as f:
                json.dump(self.table, f, indent=1)
            os.replace(tmp, self.path)

    def choice(self, engine, ket, L, R, mpo, precision: Optional[int] = None) -> Dict[str, int]:
        """The plan options (``plan_sigma`` keywords) for this problem, measured on first
        sight of its shape; options a stored entry lacks take their defaults (0)."""
        prec = engine.precision if precision is None else precision
        key = shape_key(ket.layout, L.layout, R.layout, mpo, prec)
        hit = self.table.get(key)
        if hit is None:
            hit = self.measure(engine, ket, L, R, mpo, prec)
            self.table[key] = hit
            self.save()
        return {k: int(hit.get(k, 0)) for k in OPTION_KEYS}

    def _time(self, engine, ket, L, R, f, prec, out, opts) -> Tuple[float, float]:
        t0 = time.time()
        p = N.plan_sigma(ket.phys_i, ket.left_i, ket.right_i, ket.layout, L.layout, R.layout, f, engine.hermitian,
                         **opts)
        p.upload()
        build = time.time() - t0
        engine.run(p, ket=ket.data, left=L, right=R, out=out, precision=prec)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(self.reps):
            engine.run(p, ket=ket.data, left=L, right=R, out=out, precision=prec)
        b.record()
        torch.cuda.synchronize()
        del p
        return a.elapsed_time(b) / self.reps, build

    def measure(self, engine, ket, L, R, mpo, prec: int) -> dict:
        f = engine.fmpo(mpo)
        out = torch.empty(max(ket.n, 1), dtype=torch.float64, device=engine.device)
        ms, build_s, opts_of = {}, {}, {}
        for sk, dm in self.candidates:
            o = {"split_k_segs": sk, "dense_min_terms": dm, "n_tile_max": 0, "k1_schedule": 0}
            name = f"{sk},{dm}"
            ms[name], build_s[name] = self._time(engine, ket, L, R, f, prec, out, o)
            opts_of[name] = o
        if prec in (N.PREC_BF16X3, N.PREC_BF16X2):
            base = dict(opts_of[min(ms, key=ms.get)])
            for ntm, k1s in SHAPE_CANDIDATES:
                o = dict(base, n_tile_max=ntm, k1_schedule=k1s)
                name = f"{o['split_k_segs']},{o['dense_min_terms']},n{ntm},s{k1s}"
                ms[name], build_s[name] = self._time(engine, ket, L, R, f, prec, out, o)
                opts_of[name] = o
        best = min(ms, key=ms.get)
        return dict(opts_of[best], ms=ms, plan_s=build_s)


__all__ = ["Autotuner", "shape_key", "CANDIDATES", "SHAPE_CANDIDATES", "OPTION_KEYS"]
