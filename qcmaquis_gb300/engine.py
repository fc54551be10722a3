"""GPU engine mirroring the reference's ``contraction::Engine`` surface.

``Engine.site_hamil2`` / ``overlap_mpo_left_step`` / ``overlap_mpo_right_step``
take the same roles as ``contraction::Engine<Matrix, OtherMatrix, SU2U1>``
(``dmrg/framework/dmrg/mp_tensors/contractions/non-abelian/engine.hpp:104-207``)
and ``SiteProblem`` / ``ietl::mult`` (``mp_tensors/siteproblem.h:22-53``,
``optimize/ietl_lanczos_solver.h:108-115``).  Tensors live on the GPU as one
flat FP64 buffer per tensor with a host-side block layout; every contraction
goes through a native plan of ``libqcm_gb300.so`` (no CPU path).
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, List, Optional, Tuple

import numpy as np
import time

import torch

from . import native as N
from .symmetry import Index


def _require_cuda():
    if not torch.cuda.is_available():
        raise RuntimeError("qcmaquis_gb300 engine needs a CUDA device (sm_103a); there is no CPU path")


@dataclass
class DeviceMPSTensor:
    """An MPS tensor in left-paired layout on the device (``MPSTensor``)."""
    phys_i: Index
    left_i: Index
    right_i: Index
    layout: N.Layout
    data: torch.Tensor  # float64, flat

    @classmethod
    def from_host(cls, t, device="cuda"):
        """From an MPSTensor-like object with ``phys_i/left_i/right_i`` and a left-paired ``data``."""
        lay = N.Layout.of(t.data)
        flat = torch.from_numpy(lay.pack(t.data)).to(device)
        return cls(t.phys_i, t.left_i, t.right_i, lay, flat)

    def to_block_matrix(self):
        return self.layout.unpack(self.data.detach().cpu().numpy())

    def like(self, data: torch.Tensor) -> "DeviceMPSTensor":
        return DeviceMPSTensor(self.phys_i, self.left_i, self.right_i, self.layout, data)

    @property
    def n(self) -> int:
        return int(self.data.numel())


@dataclass
class DeviceBlockMatrix:
    """A block matrix (the bond matrix of a zero-site problem) in one device arena."""
    layout: N.Layout
    data: torch.Tensor  # float64, flat

    @classmethod
    def from_host(cls, bm, device="cuda"):
        lay = N.Layout.of(bm)
        return cls(lay, torch.from_numpy(lay.pack(bm)).to(device))

    def to_host(self):
        return self.layout.unpack(self.data.detach().cpu().numpy())

    def like(self, data: torch.Tensor) -> "DeviceBlockMatrix":
        return DeviceBlockMatrix(self.layout, data)

    @property
    def n(self) -> int:
        return int(self.data.numel())


@dataclass
class DeviceBoundary:
    """A boundary (one block matrix per MPO bond index) in one device arena."""
    layout: N.BoundaryLayout
    data: torch.Tensor

    @classmethod
    def from_host(cls, boundary, device="cuda"):
        lay = N.BoundaryLayout.of(boundary)
        flat = torch.from_numpy(lay.pack(boundary) if lay.size else np.zeros(1)).to(device)
        return cls(lay, flat)

    def to_host(self):
        return self.layout.unpack(self.data.detach().cpu().numpy())

    def f32(self) -> torch.Tensor:
        """FP32 shadow of the arena for the mixed-precision forms (made once, then cached)."""
        sh = getattr(self, "_f32", None)
        if sh is None or sh.numel() != self.data.numel():
            sh = self.data.float()
            self._f32 = sh
        return sh


def _digest(*parts) -> bytes:
    """Content digest of indices and layouts (cached on layout objects)."""
    import hashlib
    h = hashlib.blake2b(digest_size=20)
    for x in parts:
        d = getattr(x, "_qcm_digest", None)
        if d is None:
            g = hashlib.blake2b(digest_size=20)
            if not hasattr(x, "q"):   # a quantum-number index (list of [charge, size])
                g.update(repr(x.data).encode())
            else:
                for a in (x.q, x.rows, x.cols, x.off, getattr(x, "ptr", None)):
                    if a is not None:
                        g.update(np.ascontiguousarray(a).tobytes())
                        g.update(b"|")
            d = g.digest()
            try:
                x._qcm_digest = d
            except AttributeError:   # Index has __slots__
                pass
        h.update(d)
    return h.digest()


def _ptr(t: Optional[torch.Tensor]) -> int:
    return 0 if t is None else int(t.data_ptr())


class Workspace:
    """Grow-only scratch buffers: the three plan scratch slots and the operand-image slot."""

    def __init__(self, device):
        self.device = device
        self.bufs = [None, None, None, None]

    def get(self, sizes):
        out = []
        for i, s in enumerate(sizes):
            s = max(int(s), 1)
            b = self.bufs[i]
            if b is None or b.numel() < s:
                self.bufs[i] = None
                b = torch.empty(s, dtype=torch.float64, device=self.device)
                self.bufs[i] = b
            out.append(b)
        return out


class Engine:
    """Plan cache + execution of the SU2U1 contractions on one GPU."""

    def __init__(self, device="cuda", precision: int = N.PREC_FP64, hermitian: bool = True,
                 use_images: bool = True):
        _require_cuda()
        N.lib()
        self.device = torch.device(device)
        self.precision = precision
        self.hermitian = hermitian
        # BF16x3 form: feed the tensor cores from pre-split operand images
        self.use_images = use_images
        self.ws = Workspace(self.device)
        self.plan_seconds = 0.0   # host time spent building and uploading plans
        self._plans: Dict[tuple, N.Plan] = {}
        self.plan_cache_size = 2     # sigma plans kept (least recently used dropped first)
        self.autotuner = None        # autotune.Autotuner: measured plan shapes per problem shape
        self.plan_hits = 0
        # boundary-step plans kept, keyed like the sigma plans (0: none, the default)
        self.boundary_plan_cache_size = 0
        self.boundary_plan_hits = 0
        self._bplans: Dict[tuple, N.Plan] = {}
        self._mpo_cache: Dict[int, N.FMpo] = {}
        self.launches = 0

    # -- helpers ---------------------------------------------------------
    def context(self) -> N.Context:
        """The engine's native context (``qcm_ctx``) on the current stream."""
        c = getattr(self, "_ctx", None)
        if c is None:
            with torch.cuda.device(self.device):
                c = self._ctx = N.Context(self._stream())
        else:
            c.set_stream(self._stream())
        return c

    def fmpo(self, mpo) -> N.FMpo:
        if isinstance(mpo, N.FMpo):     # already flattened (the native two-site builder)
            return mpo
        f = self._mpo_cache.get(id(mpo))
        if f is None or f.mpo is not mpo:
            f = N.FMpo(mpo)
            self._mpo_cache[id(mpo)] = f
        return f

    def _stream(self) -> int:
        return int(torch.cuda.current_stream(self.device).cuda_stream)

    def sigma_plan(self, ket: DeviceMPSTensor, L: DeviceBoundary, R: DeviceBoundary, mpo) -> N.Plan:
        # keyed by content: a later site problem with the same indices, layouts and MPO
        # tensor (frequent once the bond dimensions have settled) reuses the plan
        key = ("s", _digest(ket.phys_i, ket.left_i, ket.right_i, ket.layout), _digest(L.layout), _digest(R.layout),
               id(mpo), self.hermitian)
        p = self._plans.get(key)
        if p is not None:
            self._plans[key] = self._plans.pop(key)   # most recently used last
            self.plan_hits += 1
        if p is None:
            opts = {}
            if self.autotuner is not None:
                opts = self.autotuner.choice(self, ket, L, R, mpo)
            t0 = time.time()
            p = N.plan_sigma(ket.phys_i, ket.left_i, ket.right_i, ket.layout, L.layout, R.layout, self.fmpo(mpo),
                             self.hermitian, **opts)
            p.upload()
            self.plan_seconds += time.time() - t0
            p._keep = (mpo,)
            # keep the most recently used sigma plans (a plan's task tables can be hundreds of MB)
            while self._plans and len(self._plans) >= max(1, self.plan_cache_size):
                self._plans.pop(next(iter(self._plans)))
            self._plans[key] = p
        return p

    def run(self, plan: N.Plan, ket=None, left=None, right=None, out=None, precision=None, first=0, last=-1):
        """Run a plan.  ``left`` / ``right`` are DeviceBoundary objects or raw FP64 tensors;
        the mixed forms read FP32 boundary shadows and keep every intermediate in FP32."""
        prec = self.precision if precision is None else precision
        img_form = prec == N.PREC_BF16X3 or prec == N.PREC_BF16X2
        img_elems = (plan.image_bytes + 7) // 8 if (img_form and (self.use_images or prec == N.PREC_BF16X2)) else 0
        s0, s1, s2, img = self.ws.get(list(plan.scratch) + [img_elems])
        mask = 0
        lt = left.data if isinstance(left, DeviceBoundary) else left
        rt = right.data if isinstance(right, DeviceBoundary) else right
        if prec != N.PREC_FP64:
            mask = (1 << N.QCM_BUF_S0) | (1 << N.QCM_BUF_S1) | (1 << N.QCM_BUF_S2)
            if isinstance(left, DeviceBoundary):
                lt = left.f32()
                mask |= 1 << N.QCM_BUF_LEFT
            if isinstance(right, DeviceBoundary):
                rt = right.f32()
                mask |= 1 << N.QCM_BUF_RIGHT
        plan.run_typed([_ptr(ket), _ptr(lt), _ptr(rt), _ptr(out), _ptr(s0), _ptr(s1), _ptr(s2),
                        _ptr(img) if img_elems else 0], mask, prec, self._stream(), first, last)
        if first == 0 and last == -1:
            self.launches += plan.last_kernels()

    # -- Engine surface ----------------------------------------------------
    def site_hamil2(self, ket: DeviceMPSTensor, L: DeviceBoundary, R: DeviceBoundary, mpo,
                    out: Optional[torch.Tensor] = None, precision=None) -> DeviceMPSTensor:
        """sigma = H_eff ket (``Engine::site_hamil2``); result in the ket's layout."""
        p = self.sigma_plan(ket, L, R, mpo)
        if out is None:
            out = torch.empty(max(p.out_elems, 1), dtype=torch.float64, device=self.device)
        self.run(p, ket=ket.data, left=L, right=R, out=out, precision=precision)
        return ket.like(out)

    def diagonal_hamiltonian(self, ket: DeviceMPSTensor, L: DeviceBoundary, R: DeviceBoundary, mpo) -> DeviceMPSTensor:
        """The diagonal of H_eff in the ket's layout (``Engine::diagonal_hamiltonian``,
        ``non-abelian/engine.hpp:221-226`` -> ``h_diag.hpp:118-158``), in FP64.  Reads
        every L[b1] and R[b2]: the boundaries must be built with ``hermitian=False``."""
        t0 = time.time()
        p = N.plan_diagonal(ket.phys_i, ket.left_i, ket.right_i, ket.layout, L.layout, R.layout, self.fmpo(mpo))
        p.upload()
        self.plan_seconds += time.time() - t0
        out = torch.empty(max(p.out_elems, 1), dtype=torch.float64, device=self.device)
        self.run(p, ket=ket.data, left=L, right=R, out=out, precision=N.PREC_FP64)
        return ket.like(out)

    def zerosite_hamil2(self, bond: DeviceBlockMatrix, L: DeviceBoundary, R: DeviceBoundary, mpo_left, mpo_right,
                        out: Optional[torch.Tensor] = None, precision=None) -> DeviceBlockMatrix:
        """sigma = H_eff C for the bond matrix C between sites i and i+1
        (``Engine::zerosite_hamil2``, ``non-abelian/zero_site_hamil.hpp:36-79``);
        L = L[i+1], R = R[i+1], mpo_left = W[i], mpo_right = W[i+1]."""
        key = ("z", _digest(bond.layout), _digest(L.layout), _digest(R.layout), id(mpo_left), id(mpo_right),
               self.hermitian)
        p = self._plans.get(key)
        if p is None:
            t0 = time.time()
            p = N.plan_zerosite(bond.layout, L.layout, R.layout, self.fmpo(mpo_left), self.fmpo(mpo_right),
                                self.hermitian)
            p.upload()
            self.plan_seconds += time.time() - t0
            p._keep = (mpo_left, mpo_right)
            while self._plans and len(self._plans) >= max(1, self.plan_cache_size):
                self._plans.pop(next(iter(self._plans)))
            self._plans[key] = p
        else:
            self.plan_hits += 1
        if out is None:
            out = torch.empty(max(p.out_elems, 1), dtype=torch.float64, device=self.device)
        self.run(p, ket=bond.data, left=L, right=R, out=out, precision=precision)
        return bond.like(out)

    def _boundary_plan(self, side: str, mps: DeviceMPSTensor, B: DeviceBoundary, mpo) -> N.Plan:
        """A boundary-step plan, from the cache when ``boundary_plan_cache_size`` > 0 and a
        step with the same indices, layouts and MPO tensor was planned before."""
        key = (side, _digest(mps.phys_i, mps.left_i, mps.right_i, mps.layout), _digest(B.layout), id(mpo),
               self.hermitian)
        p = self._bplans.get(key) if self.boundary_plan_cache_size > 0 else None
        if p is not None:
            self._bplans[key] = self._bplans.pop(key)   # most recently used last
            self.boundary_plan_hits += 1
            return p
        t0 = time.time()
        build = N.plan_boundary_left if side == "left" else N.plan_boundary_right
        p = build(mps.phys_i, mps.left_i, mps.right_i, mps.layout, B.layout, self.fmpo(mpo), self.hermitian)
        p.upload()
        self.plan_seconds += time.time() - t0
        if self.boundary_plan_cache_size > 0:
            p._keep = (mpo,)
            while self._bplans and len(self._bplans) >= self.boundary_plan_cache_size:
                self._bplans.pop(next(iter(self._bplans)))
            self._bplans[key] = p
        return p

    def overlap_mpo_left_step(self, mps: DeviceMPSTensor, L: DeviceBoundary, mpo,
                              precision: int = N.PREC_FP64) -> DeviceBoundary:
        """L[i+1] from L[i], A[i], W[i] (``Engine::overlap_mpo_left_step``, bra = ket).
        The boundary is stored in FP64; ``precision`` selects the arithmetic of its
        block products (the mixed forms: FP32 intermediates, tensor-core products)."""
        p = self._boundary_plan("left", mps, L, mpo)
        lay = p.out_layout()
        out = torch.empty(max(p.out_elems, 1), dtype=torch.float64, device=self.device)
        self.run(p, ket=mps.data, left=L, out=out, precision=precision)
        return DeviceBoundary(lay, out)

    def overlap_mpo_right_step(self, mps: DeviceMPSTensor, R: DeviceBoundary, mpo,
                               precision: int = N.PREC_FP64) -> DeviceBoundary:
        """R[i] from R[i+1], B[i], W[i] (``Engine::overlap_mpo_right_step``, bra = ket);
        ``precision`` as for ``overlap_mpo_left_step``."""
        p = self._boundary_plan("right", mps, R, mpo)
        lay = p.out_layout()
        out = torch.empty(max(p.out_elems, 1), dtype=torch.float64, device=self.device)
        self.run(p, ket=mps.data, right=R, out=out, precision=precision)
        return DeviceBoundary(lay, out)

    def boundary_tensor_mpo(self, mps: DeviceMPSTensor, B: DeviceBoundary, mpo, side: str) -> DeviceBoundary:
        """``Engine::left_boundary_tensor_mpo`` (side "left", B = left boundary) or
        ``right_boundary_tensor_mpo`` (side "right", B = right boundary),
        ``non-abelian/engine.hpp:84-102``: the bra-free contraction, one block
        matrix per open MPO bond, in FP64."""
        t0 = time.time()
        p = N.plan_boundary_tensor_mpo(mps.phys_i, mps.left_i, mps.right_i, mps.layout, B.layout, self.fmpo(mpo),
                                       side, self.hermitian)
        p.upload()
        self.plan_seconds += time.time() - t0
        lay = p.out_layout()
        out = torch.empty(max(p.out_elems, 1), dtype=torch.float64, device=self.device)
        if side == "left":
            self.run(p, ket=mps.data, left=B, out=out, precision=N.PREC_FP64)
        else:
            self.run(p, ket=mps.data, right=B, out=out, precision=N.PREC_FP64)
        return DeviceBoundary(lay, out)


class SiteProblem:
    """``SiteProblem{left, right, mpo}`` with ``ietl::mult`` = ``apply``."""

    def __init__(self, engine: Engine, left: DeviceBoundary, right: DeviceBoundary, mpo):
        self.engine = engine
        self.left = left
        self.right = right
        self.mpo = mpo

    def apply(self, x: DeviceMPSTensor, out: Optional[torch.Tensor] = None) -> DeviceMPSTensor:
        return self.engine.site_hamil2(x, self.left, self.right, self.mpo, out=out)


class ZeroSiteProblem:
    """``ZeroSiteProblem{mpo_left, mpo_right, left, right}`` (``mp_tensors/zerositeproblem.h:25-56``):
    ``apply`` = ``zerosite_hamil2``, ``get_energy`` = <x|H x> / <x|x>."""

    def __init__(self, engine: Engine, mpo_left, mpo_right, left: DeviceBoundary, right: DeviceBoundary):
        self.engine = engine
        self.mpo_left = mpo_left
        self.mpo_right = mpo_right
        self.left = left
        self.right = right

    def apply(self, x: DeviceBlockMatrix, out: Optional[torch.Tensor] = None) -> DeviceBlockMatrix:
        return self.engine.zerosite_hamil2(x, self.left, self.right, self.mpo_left, self.mpo_right, out=out)

    def get_energy(self, x: DeviceBlockMatrix) -> float:
        from .jd import VecOps
        ops = getattr(self, "_ops", None) or VecOps(self.engine.device)
        self._ops = ops
        y = self.apply(x)
        return ops.dot(x.data, y.data) / ops.dot(x.data, x.data)


__all__ = ["Engine", "SiteProblem", "ZeroSiteProblem", "DeviceMPSTensor", "DeviceBlockMatrix", "DeviceBoundary"]
