"""The adjoint behind ``torch.autograd.Function`` (``qcmaquis_gb300.autograd``):

* ``IntegralEnergy``: torch.autograd.grad of the energy with respect to every
  unique integral equals central differences (step 1e-5) of the oracle's energy
  of the same MPS under the perturbed Hamiltonian, on 20 random integrals, to
  1e-6 relative (the energy is linear in the integrals; the difference quotient
  carries about 1e-16 / 1e-5 of rounding); the forward energy equals the
  oracle's expectation value to 1e-10 Eh;
* ``LocalEnergy``: the gradient of the Rayleigh quotient of one site problem
  along random directions equals central differences to 1e-7 relative.
"""
import numpy as np
import pytest
import torch

from qcmaquis_gb300.autograd import IntegralEnergy, LocalEnergy
from qcmaquis_gb300.engine import DeviceBoundary, DeviceMPSTensor, Engine, SiteProblem
from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model import QCModel
from qcmaquis_gb300.mpo import make_mpo
from oracle import dmrg_ref as R
from oracle.sweep import SweepParams, expval, initial_state, overlap

from test_oracle import _random_site_problem

pytestmark = pytest.mark.gpu


def _oracle_energy(L, ints, N, mps_host):
    model = QCModel(L, ints, N, integral_cutoff=-1.0)
    mpo = make_mpo(model)
    return expval(mps_host, mpo) / overlap(mps_host) + mpo.core_energy


def test_integral_energy_autograd_matches_central_differences():
    L, N = 6, 6
    ints = synthetic_integral_map(L, seed=3)
    model = QCModel(L, ints, N)
    mpo = make_mpo(model)
    mps_host = initial_state(model, mpo, SweepParams(init_bond_dimension=16, seed=11), N, 0)
    mps = [DeviceMPSTensor.from_host(t.copy().make_left_paired()) for t in mps_host]
    keys = sorted(ints)
    values = torch.tensor([ints[k] for k in keys], dtype=torch.float64, requires_grad=True)
    E = IntegralEnergy.apply(values, keys, L, N, 0, mps, Engine("cuda:0"))
    (g,) = torch.autograd.grad(E, values)
    e_ref = _oracle_energy(L, ints, N, mps_host)
    assert abs(E.item() - e_ref) < 1e-10
    rng = np.random.default_rng(7)
    h = 1e-5
    for i in rng.choice(len(keys), 20, replace=False):
        k = keys[int(i)]
        up, dn = dict(ints), dict(ints)
        up[k] += h
        dn[k] -= h
        fd = (_oracle_energy(L, up, N, mps_host) - _oracle_energy(L, dn, N, mps_host)) / (2 * h)
        assert abs(fd - g[int(i)].item()) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[int(i)].item())


def test_local_energy_autograd_matches_central_differences():
    psi, left, right, ts, ots = _random_site_problem(site=2, m=16)
    eng = Engine("cuda:0")
    x = DeviceMPSTensor.from_host(psi.copy().make_left_paired())
    sp = SiteProblem(eng, DeviceBoundary.from_host(left), DeviceBoundary.from_host(right), ts)
    p = x.data.clone().requires_grad_(True)
    E = LocalEnergy.apply(p, sp, x)
    (g,) = torch.autograd.grad(E, p)
    ref = R.site_hamil2(psi.copy(), left, right, ots).make_left_paired()
    pl = psi.copy().make_left_paired()
    assert abs(E.item() - pl.dot(ref) / pl.dot(pl)) <= 1e-12 * abs(E.item())
    gen = torch.Generator(device="cuda").manual_seed(5)
    h = 1e-5
    for _ in range(3):
        d = torch.randn(p.shape, dtype=torch.float64, device="cuda", generator=gen)
        with torch.no_grad():
            ep = LocalEnergy.apply(p.detach() + h * d, sp, x)
            em = LocalEnergy.apply(p.detach() - h * d, sp, x)
        fd = ((ep - em) / (2 * h)).item()
        an = torch.dot(g, d).item()
        assert abs(fd - an) <= 1e-7 * max(1.0, abs(an)), (fd, an)
