"""Autotuner of sigma-plan shapes, keyed on the block-size histogram.

Two plan-shape parameters of a sigma plan are measured instead of fixed:

- ``split_k_segs``: the largest number of block products summed into one K3
  output before the output is split into partial tiles;
- ``dense_min_terms``: the fewest K2 terms an output tile needs to join a dense
  tensor-core group.

For a site problem the tuner builds the plan of every candidate pair, times
``reps`` sigma vectors of each with CUDA events (after a warm-up) and keeps the
fastest.  The choice is stored under a key made of the problem's block-size
histogram (log2 buckets of the psi, left and right boundary blocks), the MPO
bond dimensions and the precision, so problems of the same shape -- the other
sites of a sweep once the bond dimensions have settled, the same system at a
later sweep, similar systems -- reuse it without measuring.  The table can be
kept in a JSON file.
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

    def choice(self, engine, ket, L, R, mpo, precision: Optional[int] = None) -> Tuple[int, int]:
        """(split_k_segs, dense_min_terms) for this problem, measured on first sight of its shape."""
        prec = engine.precision if precision is None else precision
        key = shape_key(ket.layout, L.layout, R.layout, mpo, prec)
        hit = self.table.get(key)
        if hit is None:
            hit = self.measure(engine, ket, L, R, mpo, prec)
            self.table[key] = hit
            self.save()
        return int(hit["split_k_segs"]), int(hit["dense_min_terms"])

    def measure(self, engine, ket, L, R, mpo, prec: int) -> dict:
        f = engine.fmpo(mpo)
        out = torch.empty(max(ket.n, 1), dtype=torch.float64, device=engine.device)
        ms, build_s = {}, {}
        for sk, dm in self.candidates:
            t0 = time.time()
            p = N.plan_sigma(ket.phys_i, ket.left_i, ket.right_i, ket.layout, L.layout, R.layout, f, engine.hermitian,
                             split_k_segs=sk, dense_min_terms=dm)
            p.upload()
            build_s[f"{sk},{dm}"] = time.time() - t0
            engine.run(p, ket=ket.data, left=L, right=R, out=out, precision=prec)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            for _ in range(self.reps):
                engine.run(p, ket=ket.data, left=L, right=R, out=out, precision=prec)
            b.record()
            torch.cuda.synchronize()
            ms[f"{sk},{dm}"] = a.elapsed_time(b) / self.reps
            del p
        best = min(ms, key=ms.get)
        sk, dm = (int(x) for x in best.split(","))
        return {"split_k_segs": sk, "dense_min_terms": dm, "ms": ms, "plan_s": build_s}


__all__ = ["Autotuner", "shape_key", "CANDIDATES"]
