"""The native term generator of the SU2U1 chemistry model (``qcm_chem_terms``)
against the Python restatement of ``models/chem/su2u1/model.hpp`` and its term
makers: the same terms in the same order, operator for operator, coefficients
equal to the last bit (signs of zeros included), the same fermion flags and the
same per-integral provenance in the same order; and the MPO built from either
is the same.  CPU only."""
import math

import numpy as np
import pytest

from conftest import integral_map
from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model import QCModel
from qcmaquis_gb300.mpo import TaggedMPOMaker
from test_mpo_maker_native import assert_same_mpo


def _bits(x: float):
    return (x, math.copysign(1.0, x))


def assert_same_terms(a, b):
    assert len(a) == len(b)
    for n, (x, y) in enumerate(zip(a, b)):
        assert x.ops == y.ops, n
        assert _bits(x.coeff) == _bits(y.coeff), (n, x.coeff, y.coeff)
        assert bool(x.is_fermionic) == bool(y.is_fermionic), n
        assert list(x.src.items()) == list(y.src.items()), n


def _with_zeros(ints, seed):
    """Some integrals set to exactly zero (kept: the unit-coefficient path) and
    some below the cutoff (dropped)."""
    rng = np.random.default_rng(seed)
    out = dict(ints)
    keys = list(out)
    for k in rng.choice(len(keys), size=max(1, len(keys) // 10), replace=False):
        out[keys[k]] = 0.0
    for k in rng.choice(len(keys), size=max(1, len(keys) // 20), replace=False):
        out[keys[k]] = 1e-30
    return out


@pytest.mark.parametrize("L,nelec,seed", [(2, 2, 1), (4, 2, 2), (6, 6, 3), (8, 8, 42), (9, 5, 7)])
def test_native_terms_equal_python(L, nelec, seed):
    ints = synthetic_integral_map(L, seed=seed)
    a = QCModel(L, ints, nelec, native=False)
    b = QCModel(L, ints, nelec, native=True)
    assert_same_terms(a.terms, b.terms)


def test_native_terms_with_zero_and_cut_integrals():
    ints = _with_zeros(synthetic_integral_map(6, seed=5), seed=6)
    assert_same_terms(QCModel(6, ints, 4, native=False).terms, QCModel(6, ints, 4, native=True).terms)
    assert_same_terms(QCModel(6, ints, 4, integral_cutoff=0.0, native=False).terms,
                      QCModel(6, ints, 4, integral_cutoff=0.0, native=True).terms)


@pytest.mark.parametrize("name", ["lih", "h2"])
def test_native_terms_of_the_golden_systems(golden, name):
    g = golden[name]
    ints = integral_map(g["integrals"])
    assert_same_terms(QCModel(g["L"], ints, g["nelec"], native=False).terms,
                      QCModel(g["L"], ints, g["nelec"], native=True).terms)


@pytest.mark.parametrize("merge", [True, False])
def test_mpo_from_native_terms_equals_python(merge):
    """The native maker reading the term arrays directly builds the MPO the Python
    maker builds from the Python generator's terms."""
    ints = synthetic_integral_map(7, seed=9)
    a = TaggedMPOMaker(QCModel(7, ints, 6, native=False), merge_site_terms=merge, native=False).create_mpo()
    b = TaggedMPOMaker(QCModel(7, ints, 6, native=True), merge_site_terms=merge, native=True).create_mpo()
    assert_same_mpo(a, b)


def test_native_terms_reject_bad_input():
    with pytest.raises(RuntimeError, match="out of range"):
        QCModel(3, {(5, 1, 0, 0): 0.3}, 2)
    with pytest.raises(RuntimeError, match="one-electron"):
        QCModel(3, {(2, 1, 0, 0): 0.3}, 1)
