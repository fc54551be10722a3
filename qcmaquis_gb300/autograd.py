"""The adjoint of the DMRG energy behind ``torch.autograd.Function``.

* ``IntegralEnergy``: E(t, V) = <Psi|H(t, V)|Psi> / <Psi|Psi> + E_core for a fixed
  MPS, as a function of the Hamiltonian's unique integrals (1-based
  ``integral_map`` keys, the format of the reference's FCIDUMP-style maps).  The
  backward pass is the hand-written adjoint (``gradient.energy_gradient``: one
  native energy-gradient plan per site, ``qcm_plan_energy_gradient``, chained
  from MPO term scales to integrals); E is linear in the integrals, so the
  forward pass reads the energy off the same plans.
* ``LocalEnergy``: the Rayleigh quotient <psi|H_eff|psi> / <psi|psi> of one site
  problem as a function of the site tensor psi (flat, in its layout); the
  backward pass is 2 (H_eff psi - E psi) / <psi|psi> from one sigma vector.

Both return FP64 scalars on psi's device and work with ``torch.autograd.grad``.
Integrals kept with value zero still get their derivative (the model is built
without the reference's 1e-20 integral cutoff for this purpose).
"""
from __future__ import annotations

from typing import List, Sequence, Tuple

import torch

from .engine import DeviceMPSTensor, SiteProblem


class IntegralEnergy(torch.autograd.Function):
    """``IntegralEnergy.apply(values, keys, L, nelec, twoS, mps, engine)``: values is a 1-D
    FP64 tensor of integral values in the order of ``keys``."""

    @staticmethod
    def forward(ctx, values: torch.Tensor, keys: Sequence[Tuple[int, int, int, int]], L: int, nelec: int,
                twoS: int, mps: List[DeviceMPSTensor], engine=None):
        from .gradient import energy_gradient
        from .model import QCModel
        vals = values.detach().to("cpu", torch.float64).tolist()
        ints = {tuple(int(x) for x in k): float(v) for k, v in zip(keys, vals)}
        model = QCModel(L, ints, nelec, integral_cutoff=-1.0)
        g = energy_gradient(model, mps, nelec, twoS, engine=engine, device=mps[0].data.device)
        grad = torch.tensor([g.d_integrals.get(tuple(k), 0.0) for k in keys], dtype=torch.float64,
                            device=values.device)
        ctx.save_for_backward(grad)
        return torch.tensor(g.energy, dtype=torch.float64, device=values.device)

    @staticmethod
    def backward(ctx, g_e):
        (grad,) = ctx.saved_tensors
        return g_e * grad, None, None, None, None, None, None


class LocalEnergy(torch.autograd.Function):
    """``LocalEnergy.apply(psi, problem, like)``: psi a flat FP64 CUDA tensor in the layout
    of ``like`` (a DeviceMPSTensor), problem a ``SiteProblem``."""

    @staticmethod
    def forward(ctx, psi: torch.Tensor, problem: SiteProblem, like: DeviceMPSTensor):
        x = psi.detach().contiguous()
        hx = problem.apply(like.like(x)).data
        nrm = torch.dot(x, x)
        e = torch.dot(x, hx) / nrm
        ctx.save_for_backward(x, hx, nrm, e)
        return e

    @staticmethod
    def backward(ctx, g_e):
        x, hx, nrm, e = ctx.saved_tensors
        return g_e * 2.0 * (hx - e * x) / nrm, None, None


__all__ = ["IntegralEnergy", "LocalEnergy"]
