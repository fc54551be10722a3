"""Host-side block-sparse matrix keyed by (row charge, column charge).

Restates the container semantics of ``block_matrix`` in
``dmrg/framework/dmrg/block_matrix/block_matrix.h:34-178`` /
``block_matrix.hpp:136-144, 401-420``: a list of dense blocks kept in
``DualIndex`` order (descending on ``(lc, rc)``), each block a dense matrix.
Blocks are numpy arrays; the column-major storage of ``alps::numeric::matrix``
(``dmrg/alps/src/alps/numeric/matrix/matrix.ipp:129``) is what the device
layout and the checkpoint format use, so :meth:`flat` emits Fortran order.

This container is used for the small site operators of the MPO builder, for
host copies of MPS tensors and boundaries, and as the data model of the CPU
oracle.  The GPU path keeps the same block order but stores all blocks of a
tensor in one flat device buffer.
"""
from __future__ import annotations

from typing import Iterable, List, Optional, Tuple

import numpy as np

from .symmetry import Charge, Index


class BlockMatrix:
    __slots__ = ("keys", "blocks")

    def __init__(self):
        self.keys: List[Tuple[Charge, Charge]] = []   # descending (lc, rc)
        self.blocks: List[np.ndarray] = []

    # -- construction ---------------------------------------------------
    @classmethod
    def from_indices(cls, rows: Index, cols: Index, fill=0.0) -> "BlockMatrix":
        """``block_matrix(Index rows, Index cols)``: pairs rows[k] with cols[k]."""
        bm = cls()
        assert len(rows) == len(cols)
        for (rc_, rs), (cc, cs) in zip(rows, cols):
            bm.keys.append((rc_, cc))
            bm.blocks.append(np.full((rs, cs), fill, dtype=np.float64))
        return bm

    def copy(self) -> "BlockMatrix":
        bm = BlockMatrix()
        bm.keys = list(self.keys)
        bm.blocks = [b.copy() for b in self.blocks]
        return bm

    # -- lookup -----------------------------------------------------------
    def n_blocks(self) -> int:
        return len(self.keys)

    def _lower_bound(self, key) -> int:
        lo, hi = 0, len(self.keys)
        while lo < hi:
            mid = (lo + hi) // 2
            if self.keys[mid] > key:
                lo = mid + 1
            else:
                hi = mid
        return lo

    def find_block(self, lc: Charge, rc: Charge) -> int:
        p = self._lower_bound((lc, rc))
        if p < len(self.keys) and self.keys[p] == (lc, rc):
            return p
        return len(self.keys)

    def has_block(self, lc: Charge, rc: Charge) -> bool:
        return self.find_block(lc, rc) < len(self.keys)

    def left_lower_bound(self, lc: Charge) -> int:
        """First block whose left charge is <= lc (``dual_index.h:157-167``)."""
        lo, hi = 0, len(self.keys)
        while lo < hi:
            mid = (lo + hi) // 2
            if self.keys[mid][0] > lc:
                lo = mid + 1
            else:
                hi = mid
        return lo

    def left_charge(self, k):
        return self.keys[k][0]

    def right_charge(self, k):
        return self.keys[k][1]

    def __getitem__(self, k) -> np.ndarray:
        return self.blocks[k]

    # -- mutation ---------------------------------------------------------
    def insert_block(self, mtx: np.ndarray, lc: Charge, rc: Charge) -> int:
        assert not self.has_block(lc, rc), (lc, rc)
        p = self._lower_bound((lc, rc))
        self.keys.insert(p, (lc, rc))
        self.blocks.insert(p, np.asarray(mtx, dtype=np.float64))
        return p

    def remove_block(self, k: int):
        del self.keys[k]
        del self.blocks[k]

    def match_and_add_block(self, mtx: np.ndarray, lc: Charge, rc: Charge):
        """``block_matrix::match_and_add_block`` (``block_matrix.hpp:401-430``)."""
        p = self.find_block(lc, rc)
        if p < len(self.keys):
            cur = self.blocks[p]
            if cur.shape == mtx.shape:
                self.blocks[p] = cur + mtx
            else:
                r = max(cur.shape[0], mtx.shape[0])
                c = max(cur.shape[1], mtx.shape[1])
                new = np.zeros((r, c))
                new[:cur.shape[0], :cur.shape[1]] += cur
                new[:mtx.shape[0], :mtx.shape[1]] += mtx
                self.blocks[p] = new
        else:
            self.insert_block(mtx.copy(), lc, rc)

    def iadd(self, other: "BlockMatrix") -> "BlockMatrix":
        """``operator+=``: add matching blocks, insert the rest."""
        for (lc, rc), b in zip(other.keys, other.blocks):
            p = self.find_block(lc, rc)
            if p < len(self.keys):
                self.blocks[p] = self.blocks[p] + b
            else:
                self.insert_block(b.copy(), lc, rc)
        return self

    def scale(self, s: float) -> "BlockMatrix":
        for k in range(len(self.blocks)):
            self.blocks[k] = self.blocks[k] * s
        return self

    # -- views ------------------------------------------------------------
    def left_basis(self) -> Index:
        return Index.from_sorted([(k[0], b.shape[0]) for k, b in zip(self.keys, self.blocks)])

    def right_basis(self) -> Index:
        return Index.from_sorted([(k[1], b.shape[1]) for k, b in zip(self.keys, self.blocks)])

    def basis(self):
        """List of (lc, rc, ls, rs) in block order."""
        return [(k[0], k[1], b.shape[0], b.shape[1]) for k, b in zip(self.keys, self.blocks)]

    def transpose(self) -> "BlockMatrix":
        """``transpose(block_matrix)``: swap charges, transpose blocks (re-sorted)."""
        bm = BlockMatrix()
        for (lc, rc), b in zip(self.keys, self.blocks):
            bm.insert_block(b.T.copy(), rc, lc)
        return bm

    def norm(self) -> float:
        return float(np.sqrt(sum(float(np.vdot(b, b)) for b in self.blocks)))

    def trace(self) -> float:
        return float(sum(np.trace(b) for b in self.blocks))

    def num_elements(self) -> int:
        return int(sum(b.size for b in self.blocks))

    def flat(self) -> np.ndarray:
        """All blocks concatenated, each in column-major order."""
        if not self.blocks:
            return np.zeros(0)
        return np.concatenate([np.asarray(b, order="F").ravel(order="F") for b in self.blocks])

    def __repr__(self):
        return "BlockMatrix(" + ", ".join(f"{k[0]}x{k[1]}:{b.shape}" for k, b in zip(self.keys, self.blocks)) + ")"


def gemm(A: BlockMatrix, B: BlockMatrix) -> BlockMatrix:
    """Charge-matched block product (``block_matrix_algorithms.h:47-80``)."""
    C = BlockMatrix()
    for k in range(A.n_blocks()):
        ar = A.right_charge(k)
        it = B.left_lower_bound(ar)
        while it < B.n_blocks() and B.keys[it][0] == ar:
            lc = A.left_charge(k)
            rc = B.keys[it][1]
            prod = A.blocks[k] @ B.blocks[it]
            p = C.find_block(lc, rc)
            if p < C.n_blocks():
                C.blocks[p] = C.blocks[p] + prod
            else:
                C.insert_block(prod, lc, rc)
            it += 1
    return C


__all__ = ["BlockMatrix", "gemm"]
