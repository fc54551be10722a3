"""Excited states: optimisation orthogonal to other states, on the GPU.

The reference optimises an excited state with the states below it as
constraints (``n_ortho_states`` / ``ortho_states``,
``sba/SweepBasedEnergyMinimization.h:52-67``): per constraint state phi_n it
keeps MPO-free overlap boundaries <psi|phi_n> to the left and right of the
optimised pair (``sba/OverlapPropagator.h``, ``common::overlap_left_step`` /
``overlap_right_step``, ``ct/common/move_boundary.hpp:20-62``), forms at every
microiteration phi_n's projection onto the pair's variational space
(``site_ortho_boundaries``, ``ct/abelian/special.hpp:16-43``), and the
Jacobi-Davidson solver keeps its basis orthogonal to those vectors
(``ietl_jacobi_davidson.h:28-49``, ``jacobi.h:378, 393, 432``).

The overlap boundaries are single block matrices (no MPO bond) of the
bond-dimension size; their products run as per-block device GEMMs.
"""
from __future__ import annotations

from typing import List, Sequence

import torch

from .engine import DeviceMPSTensor
from .mps_ops import DBM, as_dbm, block_views, gemm, make_two_site_mps, reshape_l2r, reshape_r2l
from .symmetry import Index, ProductBasis, fuse, neg


def _ones(c, device) -> DBM:
    d = DBM()
    d.insert(torch.ones((1, 1), dtype=torch.float64, device=device), c, c)
    return d


def overlap_left_step(bra: DeviceMPSTensor, ket: DeviceMPSTensor, left: DBM) -> DBM:
    """``common::overlap_left_step`` with ``SU2::gemm`` (``ct/common/move_boundary.hpp:20-40``):
    blocks keyed (bra charge, ket charge)."""
    ket_rp = reshape_l2r(ket.phys_i, ket.left_i, ket.right_i, as_dbm(ket))
    t1 = gemm(left, ket_rp)
    t3 = reshape_r2l(ket.phys_i, bra.left_i, ket.right_i, t1)
    return gemm(as_dbm(bra), t3, ta=True)


def overlap_right_step(bra: DeviceMPSTensor, ket: DeviceMPSTensor, right: DBM) -> DBM:
    """``common::overlap_right_step`` (``ct/common/move_boundary.hpp:45-62``)."""
    t1 = gemm(as_dbm(ket), right, tb=True)
    t3 = reshape_l2r(ket.phys_i, ket.left_i, bra.right_i, t1)
    bra_rp = reshape_l2r(bra.phys_i, bra.left_i, bra.right_i, as_dbm(bra))
    return gemm(bra_rp, t3, tb=True)


def _pad_left(phys: Index, in_left_i: Index, in_right_i: Index, psi: DeviceMPSTensor, m1: DBM) -> torch.Tensor:
    """``reshape_and_pad_left`` (``mp_tensors/reshapes.h:228-278``) into a zeroed copy of
    psi's left-paired layout; returns the flat vector."""
    flat = torch.zeros_like(psi.data)
    out = block_views(psi.layout, flat)
    in_left = ProductBasis(phys, in_left_i)
    out_left = ProductBasis(phys, psi.left_i)
    for (lc, rc), blk in zip(m1.keys, m1.blocks):
        if not in_right_i.has(rc):
            continue
        nr = in_right_i[in_right_i.position(rc)][1]
        for pc, pd in phys:
            l_in = fuse(lc, neg(pc))
            if not in_left_i.has(l_in) or not psi.left_i.has(l_in):
                continue
            k = out.find(lc, rc)
            if k == len(out.keys):
                continue
            ldim = in_left_i[in_left_i.position(l_in)][1]
            io, oo = in_left(pc, l_in), out_left(pc, l_in)
            out.blocks[k][oo:oo + pd * ldim, :nr] = blk[io:io + pd * ldim, :nr]
    return flat


def site_ortho_boundaries(psi: DeviceMPSTensor, theta: DeviceMPSTensor, o_left: DBM, o_right: DBM) -> torch.Tensor:
    """``site_ortho_boundaries`` (``ct/abelian/special.hpp:16-43``): ``theta`` (a
    constraint state's two-site tensor) through the overlap boundaries, in psi's layout."""
    t = gemm(o_left, reshape_l2r(theta.phys_i, theta.left_i, theta.right_i, as_dbm(theta)))
    li = o_left.left_basis()
    t2 = reshape_r2l(psi.phys_i, li, theta.right_i, t)
    t3 = gemm(t2, o_right, tb=True)
    return _pad_left(psi.phys_i, li, o_right.left_basis(), psi, t3)


class OverlapBoundaries:
    """``OverlapPropagator`` on the device: per constraint state n the left and right
    overlap boundaries of the current MPS (bra) with that state (ket), started at
    site 0 with every right boundary built."""

    def __init__(self, mps: List[DeviceMPSTensor], others: Sequence[List[DeviceMPSTensor]], right_end):
        L = len(mps)
        dev = mps[0].data.device
        self.mps, self.others = mps, list(others)
        self.left = [[None] * (L + 1) for _ in self.others]
        self.right = [[None] * (L + 1) for _ in self.others]
        for n in range(len(self.others)):
            self.left[n][0] = _ones((0, 0), dev)
            self.right[n][L] = _ones(tuple(right_end), dev)
            for i in range(L - 1, 0, -1):
                self.update_right(i, n)

    def update_left(self, i: int, only=None):
        for n in (range(len(self.others)) if only is None else [only]):
            self.left[n][i] = overlap_left_step(self.mps[i - 1], self.others[n][i - 1], self.left[n][i - 1])

    def update_right(self, i: int, only=None):
        for n in (range(len(self.others)) if only is None else [only]):
            self.right[n][i] = overlap_right_step(self.mps[i], self.others[n][i], self.right[n][i + 1])

    def vectors(self, site: int, psi: DeviceMPSTensor) -> List[torch.Tensor]:
        """The constraint vectors of the two-site problem at (site, site + 1), flat in psi's layout."""
        out = []
        for n, phi in enumerate(self.others):
            theta = make_two_site_mps(phi[site], phi[site + 1])
            out.append(site_ortho_boundaries(psi, theta, self.left[n][site], self.right[n][site + 2]))
        return out


__all__ = ["overlap_left_step", "overlap_right_step", "site_ortho_boundaries", "OverlapBoundaries"]
