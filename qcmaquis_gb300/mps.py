"""Host-side MPS construction: allowed sectors, bond dimensions, canonical site tensors.

* ``allowed_sectors`` restates ``mp_tensors/mps_sectors.h:23-112`` (one site type).
* Bond dimensions: the reference initialiser caps every sector at the same
  ``Mmax`` (``mp_tensors/mps_initializers.h:62-70``); here the cap is chosen per
  bond ("water filling") so that the bond's total multiplet count is at most
  ``m`` -- a random state with the sector structure of a converged run at
  bond dimension ``m``.
* Site tensors follow the ``MPSTensor`` constructor (``mp_tensors/mpstensor.hpp:25-60``):
  block-diagonal left-paired blocks over ``common_subset(phys*left, right)``.
* Canonicalisation uses per-block QR / LQ (``block_matrix_algorithms.h:442-492``).

These helpers prepare inputs (the initial state and the benchmark
workloads); the contractions themselves run on the GPU.
"""
from __future__ import annotations

from typing import List, Tuple

import numpy as np

from .block_matrix import BlockMatrix
from .symmetry import (Index, ProductBasis, adjoin, common_subset, fuse, fuse_neg_first, index_product, neg,
                       spin)


class HostMPSTensor:
    """Site tensor on the host, always stored left-paired."""

    def __init__(self, phys: Index, left_i: Index, right_i: Index, data: BlockMatrix):
        self.phys_i = phys
        self.left_i = left_i
        self.right_i = right_i
        self.data = data

    def norm(self) -> float:
        return self.data.norm()


def allowed_sectors(L: int, phys: Index, right_end, Mmax: int, abelian: bool = False) -> List[Index]:
    """``allowed_sectors``; ``abelian`` (TwoU1) drops the SU(2) test that a sector's
    spin is not negative (``ChargeDetailClass::physical``)."""
    physc = phys.copy()
    physc.sort()
    cmax, cmin = physc[0][0], physc[len(physc) - 1][0]
    if cmin > cmax:
        cmax, cmin = cmin, cmax
    maxt = (L * cmax[0], L * cmax[1])
    mint = (L * cmin[0], L * cmin[1])
    left = [None] * (L + 1)
    right = [None] * (L + 1)
    left[0] = Index([((0, 0), 1)])
    right[L] = Index([(right_end, 1)])
    cmaxi, cmini = maxt, mint
    for i in range(1, L + 1):
        li = index_product(phys, left[i - 1])
        cmaxi = fuse(cmaxi, neg(cmax))
        cmini = fuse(cmini, neg(cmin))
        li.data = [[c, min(Mmax, s)] for c, s in li
                   if not (fuse(c, cmaxi) < right_end) and not (fuse(c, cmini) > right_end)
                   and (abelian or spin(c) >= 0)]
        left[i] = li
    cmaxi, cmini = maxt, mint
    for i in range(L - 1, -1, -1):
        ri = index_product(adjoin(phys), right[i + 1])
        cmaxi = fuse(cmaxi, neg(cmax))
        cmini = fuse(cmini, neg(cmin))
        ri.data = [[c, min(Mmax, s)] for c, s in ri
                   if not (fuse(c, neg(cmaxi)) > (0, 0)) and not (fuse(c, neg(cmini)) < (0, 0))
                   and (abelian or spin(c) >= 0)]
        right[i] = ri
        common_subset(left[i], right[i])
    out = []
    for i in range(L + 1):
        a, b = left[i].copy(), right[i].copy()
        common_subset(a, b)
        a.data = [[c, min(Mmax, left[i].size_of_block(c), right[i].size_of_block(c))] for c, _ in a]
        out.append(a)
    return out


def waterfill(idx: Index, m: int) -> Index:
    """Largest uniform per-sector cap with total size <= m (at least 1 state per sector kept if possible)."""
    sizes = [s for _, s in idx]
    if sum(sizes) <= m:
        return idx.copy()
    lo, hi = 0, max(sizes)
    while lo < hi:
        mid = (lo + hi + 1) // 2
        if sum(min(mid, s) for s in sizes) <= m:
            lo = mid
        else:
            hi = mid - 1
    cap = max(lo, 1)
    out = Index.from_sorted([(c, min(cap, s)) for c, s in idx])
    return out


def profile_fill(idx: Index, m: int, n_expect: float, sigma_n: float = 1.5, sigma_s: float = 1.0) -> Index:
    """Distribute m multiplets over the sectors of ``idx`` with a Gaussian profile.

    Weight of sector (N, 2S): exp(-(N - n_expect)^2 / (2 sigma_n^2)) * exp(-S^2 / (2 sigma_s^2)),
    i.e. the particle-number and spin distribution of a block of a
    ground state; each sector is capped by its allowed size and the remainder
    is handed out in weight order.  Sectors that receive nothing are dropped.
    """
    if idx.sum_of_sizes() <= m:
        return idx.copy()
    w = np.array([np.exp(-(c[0] - n_expect) ** 2 / (2 * sigma_n ** 2)) * np.exp(-(0.5 * c[1]) ** 2 / (2 * sigma_s ** 2))
                  for c, _ in idx])
    cap = np.array([s for _, s in idx])
    alloc = np.minimum(np.floor(m * w / w.sum()).astype(np.int64), cap)
    order = np.argsort(-w, kind="stable")
    left = m - int(alloc.sum())
    while left > 0:
        moved = False
        for k in order:
            if left == 0:
                break
            if alloc[k] < cap[k] and w[k] > 1e-12:
                alloc[k] += 1
                left -= 1
                moved = True
        if not moved:
            break
    return Index.from_sorted([(c, int(a)) for (c, _), a in zip(idx, alloc) if a > 0])


def bond_indices(L: int, phys: Index, right_end, m: int, profile: bool = True) -> List[Index]:
    full = allowed_sectors(L, phys, right_end, 1 << 40)
    if not profile:
        return [waterfill(x, m) for x in full]
    return [profile_fill(x, m, right_end[0] * i / L) for i, x in enumerate(full)]


def _lp_layout(phys: Index, left_i: Index, right_i: Index):
    lb = index_product(phys, left_i)
    rb = right_i.copy()
    common_subset(lb, rb)
    return lb, rb


def random_tensor(phys: Index, left_i: Index, right_i: Index, rng: np.random.Generator) -> HostMPSTensor:
    lb, rb = _lp_layout(phys, left_i, right_i)
    bm = BlockMatrix.from_indices(lb, rb)
    for k in range(bm.n_blocks()):
        bm.blocks[k] = rng.random(bm.blocks[k].shape) - 0.5
    li = left_i.copy()
    common_subset(li, index_product(adjoin(phys), rb))
    t = HostMPSTensor(phys, li, rb, bm)
    t.data.scale(1.0 / t.norm())
    return t


def reshape_l2r(phys: Index, left_i: Index, right_i: Index, m1: BlockMatrix) -> BlockMatrix:
    """``reshape_left_to_right_new`` (``mp_tensors/reshapes.h:178-221``)."""
    m2 = BlockMatrix()
    in_left = ProductBasis(phys, left_i)
    out_right = ProductBasis(phys, right_i, fuse_neg_first)
    for blk in range(m1.n_blocks()):
        r = right_i.position(m1.right_charge(blk))
        if r == len(right_i):
            continue
        in_r = right_i[r][0]
        for ps, sd in phys:
            l = left_i.position(fuse(m1.left_charge(blk), neg(ps)))
            if l == len(left_i):
                continue
            ol, orr = left_i[l][0], fuse(neg(ps), in_r)
            if not m2.has_block(ol, orr):
                m2.insert_block(np.zeros((left_i[l][1], out_right.size(orr))), ol, orr)
            ob = m2.blocks[m2.find_block(ol, orr)]
            ilo, oro = in_left(ps, ol), out_right(ps, in_r)
            ld, rd = left_i[l][1], right_i[r][1]
            for ss in range(sd):
                ob[:ld, oro + ss * rd:oro + (ss + 1) * rd] = m1.blocks[blk][ilo + ss * ld:ilo + (ss + 1) * ld, :rd]
    return m2


def reshape_r2l(phys: Index, left_i: Index, right_i: Index, m1: BlockMatrix) -> BlockMatrix:
    """``reshape_right_to_left_new`` (``mp_tensors/reshapes.h:290-338``)."""
    m2 = BlockMatrix()
    in_right = ProductBasis(phys, right_i, fuse_neg_first)
    out_left = ProductBasis(phys, left_i)
    for blk in range(m1.n_blocks()):
        l = left_i.position(m1.left_charge(blk))
        if l == len(left_i):
            continue
        in_l = left_i[l][0]
        for ps, sd in phys:
            r = right_i.position(fuse(m1.right_charge(blk), ps))
            if r == len(right_i):
                continue
            ol, orr = fuse(ps, in_l), right_i[r][0]
            if not m2.has_block(ol, orr):
                m2.insert_block(np.zeros((out_left.size(ol), right_i[r][1])), ol, orr)
            ob = m2.blocks[m2.find_block(ol, orr)]
            iro, olo = in_right(ps, orr), out_left(ps, in_l)
            ld, rd = left_i[l][1], right_i[r][1]
            for ss in range(sd):
                ob[olo + ss * ld:olo + (ss + 1) * ld, :rd] = m1.blocks[blk][:ld, iro + ss * rd:iro + (ss + 1) * rd]
    return m2


def left_canonical_chain(phys: Index, bonds: List[Index], upto: int, rng) -> Tuple[List[HostMPSTensor], Index]:
    """Random left-normalised tensors for sites 0..upto-1; returns them and the reached bond index."""
    out = []
    left = bonds[0]
    for i in range(upto):
        t = random_tensor(phys, left, bonds[i + 1], rng)
        Q = BlockMatrix()
        for (lc, rc), b in zip(t.data.keys, t.data.blocks):
            q, _ = np.linalg.qr(b, mode="reduced")
            Q.insert_block(q, lc, rc)
        t.data = Q
        t.right_i = Q.right_basis()
        out.append(t)
        left = t.right_i
    return out, left


def right_canonical_chain(phys: Index, bonds: List[Index], L: int, downto: int, rng):
    """Random right-normalised tensors for sites downto..L-1 (returned in site order) and the reached bond."""
    out = []
    right = bonds[L]
    for i in range(L - 1, downto - 1, -1):
        t = random_tensor(phys, bonds[i], right, rng)
        rp = reshape_l2r(phys, t.left_i, t.right_i, t.data)
        Qb = BlockMatrix()
        for (lc, rc), b in zip(rp.keys, rp.blocks):
            q, _ = np.linalg.qr(b.T, mode="reduced")
            Qb.insert_block(q.T, lc, rc)
        new_left = Qb.left_basis()
        t.left_i = new_left
        t.data = reshape_r2l(phys, new_left, t.right_i, Qb)
        out.append(t)
        right = new_left
    out.reverse()
    return out, right


def two_site_random(phys2: Index, left_i: Index, right_i: Index, rng) -> HostMPSTensor:
    """A random normalised two-site (SU2-reduced) tensor in left-paired layout."""
    return random_tensor(phys2, left_i, right_i, rng)


__all__ = ["HostMPSTensor", "allowed_sectors", "waterfill", "bond_indices", "random_tensor", "reshape_l2r",
           "reshape_r2l", "left_canonical_chain", "right_canonical_chain", "two_site_random"]
