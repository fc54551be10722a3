"""SU2U1 quantum numbers and the block-index bookkeeping built on them.

A charge is the pair ``(N, 2S)`` (particle number, twice the spin), fused by
plain addition and ordered lexicographically, as ``NU1Charge<2,int>`` is in
``dmrg/framework/dmrg/block_matrix/symmetry/su2u1.h:18-50`` and
``nu1_tpl.h:152-170``.  The physical basis of a spatial orbital holds the
pseudo-charge ``(1,-1)`` beside ``(1,1)``: fusing with it lowers the coupled
spin, which is how the abelian fuse rule enumerates both SU(2) coupling
branches (``models/chem/su2u1/model.hpp:26-41``).

``Index`` is a list of ``(charge, size)`` kept sorted in *descending* charge
order (``block_matrix/indexing_stable.hpp:82-160``); ``ProductBasis`` assigns
the offset of each ``(a, b)`` pair inside its fused sector in the iteration
order of ``a`` then ``b`` (``indexing_stable.hpp:305-351``).  Block lists
(``DualIndex``) are sorted descending on ``(lc, rc)`` (``dual_index.h:39-60``).
These orders fix the memory layout of every block-sparse tensor, so they are
reproduced exactly.
"""
from __future__ import annotations

import bisect
from typing import Callable, Dict, Iterable, List, Tuple

Charge = Tuple[int, int]

IDENTITY: Charge = (0, 0)


def fuse(a: Charge, b: Charge) -> Charge:
    return (a[0] + b[0], a[1] + b[1])


def neg(a: Charge) -> Charge:
    return (-a[0], -a[1])


def fuse_neg_first(a: Charge, b: Charge) -> Charge:
    """``fuse(-a, b)``: the fusion rule of right-paired product bases."""
    return (b[0] - a[0], b[1] - a[1])


def spin(c: Charge) -> int:
    return c[1]


def particle_number(c: Charge) -> int:
    return c[0]


def triangle(a: int, b: int, c: int) -> bool:
    """SU(2) triangle rule on doubled spins (``gsl_coupling.h:25-28``)."""
    return ((a + b + c) % 2 == 0) and abs(a - b) <= c <= a + b


class Index:
    """Sorted (descending) list of ``(charge, size)`` sectors."""

    __slots__ = ("data",)

    def __init__(self, entries: Iterable[Tuple[Charge, int]] = ()):
        self.data: List[List] = []
        for c, s in entries:
            self.insert(tuple(c), int(s))

    # -- construction -------------------------------------------------
    @classmethod
    def from_sorted(cls, entries):
        idx = cls()
        idx.data = [[tuple(c), int(s)] for c, s in entries]
        return idx

    def copy(self) -> "Index":
        return Index.from_sorted(self.data)

    def insert(self, c: Charge, s: int) -> int:
        # destination = first entry with charge < c  (indexing_stable.hpp:275-282)
        pos = 0
        n = len(self.data)
        while pos < n and not (self.data[pos][0] < c):
            pos += 1
        self.data.insert(pos, [c, s])
        return pos

    # -- queries ------------------------------------------------------
    def position(self, c: Charge) -> int:
        for i, (cc, _) in enumerate(self.data):
            if cc == c:
                return i
        return len(self.data)

    def has(self, c: Charge) -> bool:
        return self.position(c) < len(self.data)

    def size_of_block(self, c: Charge, missing_ok: bool = False) -> int:
        p = self.position(c)
        if p == len(self.data):
            if missing_ok:
                return 0
            raise KeyError(c)
        return self.data[p][1]

    def charges(self) -> List[Charge]:
        return [c for c, _ in self.data]

    def sizes(self) -> List[int]:
        return [s for _, s in self.data]

    def sum_of_sizes(self) -> int:
        return sum(s for _, s in self.data)

    def __len__(self):
        return len(self.data)

    def __getitem__(self, i):
        return self.data[i]

    def __iter__(self):
        return iter(self.data)

    def __eq__(self, other):
        if not isinstance(other, Index):
            return NotImplemented
        return [tuple(x) for x in self.data] == [tuple(x) for x in other.data]

    def __repr__(self):
        return "Index(" + ", ".join(f"{c}:{s}" for c, s in self.data) + ")"

    def sort(self):
        self.data.sort(key=lambda e: e[0], reverse=True)


def index_product(i1: Index, i2: Index) -> Index:
    """``operator*`` of two indices (``indexing_stable.hpp:498-516``)."""
    ret = Index()
    for c1, s1 in i1:
        for c2, s2 in i2:
            pc = fuse(c1, c2)
            p = ret.position(pc)
            if p < len(ret):
                ret.data[p][1] += s1 * s2
            else:
                ret.insert(pc, s1 * s2)
    ret.sort()
    return ret


def adjoin(inp: Index) -> Index:
    """Negated charges, sorted (``indexing_stable.hpp:459-480``)."""
    sizes = {c: s for c, s in inp}
    ret = Index()
    for c in sorted(neg(c) for c, _ in inp):
        ret.insert(c, sizes[neg(c)])
    return ret


def common_subset(a: Index, b: Index) -> Index:
    """Drop from ``a`` the charges absent from ``b`` and vice versa, in place."""
    bset = {c for c, _ in b}
    a.data = [e for e in a.data if e[0] in bset]
    aset = {c for c, _ in a}
    b.data = [e for e in b.data if e[0] in aset]
    return a


class ProductBasis:
    """Offsets of ``(a, b)`` charge pairs inside their fused sector."""

    __slots__ = ("keys", "sizes")

    def __init__(self, a: Index, b: Index, f: Callable[[Charge, Charge], Charge] = fuse):
        self.keys: Dict[Tuple[Charge, Charge], int] = {}
        self.sizes: Dict[Charge, int] = {}
        for c1, s1 in a:
            for c2, s2 in b:
                pc = f(c1, c2)
                cur = self.sizes.get(pc, 0)
                self.keys[(c1, c2)] = cur
                self.sizes[pc] = cur + s1 * s2

    def __call__(self, a: Charge, b: Charge) -> int:
        return self.keys[(a, b)]

    def size(self, pc: Charge) -> int:
        return self.sizes[pc]


def dual_key(lc: Charge, rc: Charge):
    """Sort key that puts ``(lc, rc)`` block lists in DualIndex order."""
    return (lc, rc)


def sorted_block_position(keys: List[Tuple[Charge, Charge]], lc: Charge, rc: Charge) -> int:
    """Insertion position of ``(lc, rc)`` in a descending-sorted key list."""
    # keys sorted descending; bisect on negated order
    lo, hi = 0, len(keys)
    k = (lc, rc)
    while lo < hi:
        mid = (lo + hi) // 2
        if keys[mid] > k:
            lo = mid + 1
        else:
            hi = mid
    return lo


__all__ = [
    "Charge", "IDENTITY", "fuse", "neg", "fuse_neg_first", "spin", "particle_number",
    "triangle", "Index", "index_product", "adjoin", "common_subset", "ProductBasis",
    "sorted_block_position", "bisect",
]
