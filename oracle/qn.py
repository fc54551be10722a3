"""The oracle's own quantum-number indices and block-sparse matrices (test infrastructure).

Written from the reference, not from the product package, so that layout
comparisons between the native planner and the oracle compare two independent
implementations:

* charges of ``NU1Charge<2,int>`` (``bm/symmetry/nu1_tpl.h:152-236``): the
  pair (N, 2S), fused by component-wise addition, ordered lexicographically;
  ``SU2U1::spin`` is the second component (``bm/symmetry/su2u1.h:18-50``);
* ``Index`` (``bm/indexing_stable.hpp:82-260``): a vector of (charge, size)
  kept in descending charge order; ``insert`` puts a new entry before the first
  entry with a smaller charge (``destination``, ``:258-264``); ``position``
  returns the size of the index for a missing charge (``:117-127``);
* ``ProductBasis`` (``:305-351``): offset of every (a, b) pair inside the
  fused sector, accumulated in the iteration order of a then b;
* ``operator*`` (``:498-516``), ``adjoin`` (``:459-480``) and
  ``common_subset`` (``:534-547``);
* ``block_matrix`` (``bm/block_matrix.h:34-178``, ``bm/block_matrix.hpp``)
  with its ``DualIndex`` order (``bm/dual_index.h:39-60``: descending on the
  (left, right) charge pair), ``insert_block``, ``match_and_add_block``
  (``block_matrix.hpp:401-430``), ``operator+=`` and the charge-matched
  ``gemm`` (``bm/block_matrix_algorithms.h:47-80``).

Blocks are numpy arrays (row-major in memory; only their values matter here).
The objects expose the same member names as the reference's types
(``position``, ``size_of_block``, ``insert_block``, ``left_lower_bound`` ...),
so tensors built by either side can be handed to the other in tests.
"""
from __future__ import annotations

from typing import Iterable, List, Tuple

import numpy as np

Charge = Tuple[int, int]


def fuse(a: Charge, b: Charge) -> Charge:
    """``NU1Charge`` addition."""
    return (a[0] + b[0], a[1] + b[1])


def neg(a: Charge) -> Charge:
    return (-a[0], -a[1])


def fuse_neg_first(a: Charge, b: Charge) -> Charge:
    """The fusion of right-paired product bases: ``fuse(-a, b)``."""
    return fuse(neg(a), b)


def spin(c: Charge) -> int:
    return c[1]


def triangle(a: int, b: int, c: int) -> bool:
    """``SU2::triangle`` on doubled spins (``bm/symmetry/gsl_coupling.h:25-28``)."""
    return (a + b + c) % 2 == 0 and abs(a - b) <= c <= a + b


class Index:
    """``Index<SU2U1>``: entries [charge, size], descending in charge."""

    __slots__ = ("data",)

    def __init__(self, entries: Iterable = ()):
        self.data: List[list] = []
        for c, s in entries:
            self.insert((int(c[0]), int(c[1])), int(s))

    @classmethod
    def from_sorted(cls, entries):
        out = cls()
        out.data = [[(int(c[0]), int(c[1])), int(s)] for c, s in entries]
        return out

    def copy(self) -> "Index":
        return Index.from_sorted(self.data)

    def _destination(self, c: Charge) -> int:
        # first entry whose charge is smaller than c
        for k, (cc, _) in enumerate(self.data):
            if cc < c:
                return k
        return len(self.data)

    def insert(self, c: Charge, s: int) -> int:
        k = self._destination(c)
        self.data.insert(k, [c, s])
        return k

    def position(self, c: Charge) -> int:
        lo, hi = 0, len(self.data)
        while lo < hi:               # lower_bound under the descending order
            mid = (lo + hi) // 2
            if self.data[mid][0] > c:
                lo = mid + 1
            else:
                hi = mid
        if lo < len(self.data) and self.data[lo][0] == c:
            return lo
        return len(self.data)

    def has(self, c: Charge) -> bool:
        return self.position(c) < len(self.data)

    def size_of_block(self, c: Charge, missing_ok: bool = False) -> int:
        k = self.position(c)
        if k == len(self.data):
            if missing_ok:
                return 0
            raise KeyError(c)
        return self.data[k][1]

    def charges(self) -> List[Charge]:
        return [e[0] for e in self.data]

    def sizes(self) -> List[int]:
        return [e[1] for e in self.data]

    def sum_of_sizes(self) -> int:
        return sum(e[1] for e in self.data)

    def sort(self):
        self.data.sort(key=lambda e: e[0], reverse=True)

    def __len__(self):
        return len(self.data)

    def __getitem__(self, k):
        return self.data[k]

    def __iter__(self):
        return iter(self.data)

    def __eq__(self, other):
        try:
            return [(tuple(c), int(s)) for c, s in self] == [(tuple(c), int(s)) for c, s in other]
        except TypeError:
            return NotImplemented

    def __repr__(self):
        return "Index(" + ", ".join(f"{c}:{s}" for c, s in self.data) + ")"


def index_product(i1: Index, i2: Index) -> Index:
    """``operator*(Index, Index)``: fused charges, sizes multiplied and summed, sorted."""
    out = Index()
    for c1, s1 in i1:
        for c2, s2 in i2:
            pc = fuse(c1, c2)
            k = out.position(pc)
            if k < len(out):
                out.data[k][1] += s1 * s2
            else:
                out.insert(pc, s1 * s2)
    out.sort()
    return out


def adjoin(inp: Index) -> Index:
    """Negated charges in ascending order of the negated charge, each with its size."""
    old = [tuple(c) for c, _ in inp]
    sizes = [s for _, s in inp]
    out = Index()
    for c in sorted(neg(c) for c in old):
        out.insert(c, sizes[old.index(neg(c))])
    return out


def common_subset(a: Index, b: Index) -> Index:
    """Erase from a the charges b lacks, then from b the charges a lacks (in place)."""
    a.data = [e for e in a.data if b.has(tuple(e[0]))]
    b.data = [e for e in b.data if a.has(tuple(e[0]))]
    return a


class ProductBasis:
    """``ProductBasis``: offsets of charge pairs inside their fused sector."""

    __slots__ = ("_off", "_size")

    def __init__(self, a: Index, b: Index, f=fuse):
        self._off = {}
        self._size = {}
        for c1, s1 in a:
            for c2, s2 in b:
                pc = f(c1, c2)
                cur = self._size.setdefault(pc, 0)
                self._off[(tuple(c1), tuple(c2))] = cur
                self._size[pc] = cur + s1 * s2

    def __call__(self, a: Charge, b: Charge) -> int:
        return self._off[(tuple(a), tuple(b))]

    def size(self, pc: Charge) -> int:
        return self._size[tuple(pc)]


class BlockMatrix:
    """``block_matrix``: (left charge, right charge) keys in DualIndex order, dense blocks."""

    __slots__ = ("keys", "blocks")

    def __init__(self):
        self.keys: List[Tuple[Charge, Charge]] = []
        self.blocks: List[np.ndarray] = []

    @classmethod
    def from_indices(cls, rows: Index, cols: Index, fill: float = 0.0) -> "BlockMatrix":
        """``block_matrix(Index rows, Index cols)``: block k pairs rows[k] with cols[k]."""
        out = cls()
        if len(rows) != len(cols):
            raise ValueError("row and column indices differ in length")
        for (rc, rs), (cc, cs) in zip(rows, cols):
            out.keys.append((tuple(rc), tuple(cc)))
            out.blocks.append(np.full((rs, cs), fill, dtype=np.float64))
        return out

    def copy(self) -> "BlockMatrix":
        out = BlockMatrix()
        out.keys = list(self.keys)
        out.blocks = [b.copy() for b in self.blocks]
        return out

    def n_blocks(self) -> int:
        return len(self.keys)

    def _bound(self, pred) -> int:
        lo, hi = 0, len(self.keys)
        while lo < hi:
            mid = (lo + hi) // 2
            if pred(self.keys[mid]):
                lo = mid + 1
            else:
                hi = mid
        return lo

    def find_block(self, lc: Charge, rc: Charge) -> int:
        key = (tuple(lc), tuple(rc))
        k = self._bound(lambda x: x > key)
        if k < len(self.keys) and self.keys[k] == key:
            return k
        return len(self.keys)

    def has_block(self, lc: Charge, rc: Charge) -> bool:
        return self.find_block(lc, rc) < len(self.keys)

    def left_lower_bound(self, lc: Charge) -> int:
        """First block whose left charge is not greater than lc (``dual_index.h:157-167``)."""
        lc = tuple(lc)
        return self._bound(lambda x: x[0] > lc)

    def left_charge(self, k):
        return self.keys[k][0]

    def right_charge(self, k):
        return self.keys[k][1]

    def __getitem__(self, k) -> np.ndarray:
        return self.blocks[k]

    def insert_block(self, mtx, lc: Charge, rc: Charge) -> int:
        key = (tuple(lc), tuple(rc))
        if self.has_block(*key):
            raise ValueError(f"block {key} already present")
        k = self._bound(lambda x: x > key)
        self.keys.insert(k, key)
        self.blocks.insert(k, np.asarray(mtx, dtype=np.float64))
        return k

    def remove_block(self, k: int):
        del self.keys[k]
        del self.blocks[k]

    def match_and_add_block(self, mtx, lc: Charge, rc: Charge):
        """Add to the block (grown to the larger shape) or insert a copy."""
        k = self.find_block(lc, rc)
        if k == len(self.keys):
            self.insert_block(np.array(mtx, dtype=np.float64), lc, rc)
            return
        cur = self.blocks[k]
        if cur.shape == mtx.shape:
            self.blocks[k] = cur + mtx
            return
        grown = np.zeros((max(cur.shape[0], mtx.shape[0]), max(cur.shape[1], mtx.shape[1])))
        grown[:cur.shape[0], :cur.shape[1]] += cur
        grown[:mtx.shape[0], :mtx.shape[1]] += mtx
        self.blocks[k] = grown

    def iadd(self, other) -> "BlockMatrix":
        """``operator+=``: matching blocks added, the others inserted."""
        for (lc, rc), b in zip(other.keys, other.blocks):
            k = self.find_block(lc, rc)
            if k < len(self.keys):
                self.blocks[k] = self.blocks[k] + b
            else:
                self.insert_block(np.array(b), lc, rc)
        return self

    def scale(self, s: float) -> "BlockMatrix":
        self.blocks = [b * s for b in self.blocks]
        return self

    def left_basis(self) -> Index:
        return Index.from_sorted([(k[0], b.shape[0]) for k, b in zip(self.keys, self.blocks)])

    def right_basis(self) -> Index:
        return Index.from_sorted([(k[1], b.shape[1]) for k, b in zip(self.keys, self.blocks)])

    def basis(self):
        return [(k[0], k[1], b.shape[0], b.shape[1]) for k, b in zip(self.keys, self.blocks)]

    def transpose(self) -> "BlockMatrix":
        out = BlockMatrix()
        for (lc, rc), b in zip(self.keys, self.blocks):
            out.insert_block(b.T.copy(), rc, lc)
        return out

    def norm(self) -> float:
        return float(np.sqrt(sum(float(np.sum(b * b)) for b in self.blocks)))

    def trace(self) -> float:
        return float(sum(np.trace(b) for b in self.blocks))

    def num_elements(self) -> int:
        return int(sum(b.size for b in self.blocks))

    def flat(self) -> np.ndarray:
        """Blocks concatenated in block order, each column-major."""
        if not self.blocks:
            return np.zeros(0)
        return np.concatenate([np.ravel(b, order="F") for b in self.blocks])

    def __repr__(self):
        return "BlockMatrix(" + ", ".join(f"{k[0]}x{k[1]}:{b.shape}" for k, b in zip(self.keys, self.blocks)) + ")"


def bm_gemm(A, B) -> BlockMatrix:
    """Charge-matched product: every A block (lc, x) times every B block (x, rc)."""
    C = BlockMatrix()
    for (lc, x), a in zip(A.keys, A.blocks):
        k = B.left_lower_bound(x)
        while k < B.n_blocks() and B.keys[k][0] == x:
            prod = a @ B.blocks[k]
            rc = B.keys[k][1]
            p = C.find_block(lc, rc)
            if p < C.n_blocks():
                C.blocks[p] = C.blocks[p] + prod
            else:
                C.insert_block(prod, lc, rc)
            k += 1
    return C


__all__ = ["Charge", "fuse", "neg", "fuse_neg_first", "spin", "triangle", "Index", "index_product", "adjoin",
           "common_subset", "ProductBasis", "BlockMatrix", "bm_gemm"]
