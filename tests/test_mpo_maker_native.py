"""The native single-site MPO maker (``qcm_mpo_maker_*``) against the Python
restatement of TaggedMPOMaker (``models/generate_mpo/tagged_mpo_maker_optim.hpp``):
element for element, term order, labels, bond spins, Hermitian partners and
phases identical, for SU2U1, TwoU1 and U1 models, merged and labelled site
terms, and the RDM measurement MPO.  CPU only."""
import types

import numpy as np
import pytest

from conftest import integral_map
from qcmaquis_gb300.integrals import synthetic_integral_map
from qcmaquis_gb300.model import QCModel, SpinSum
from qcmaquis_gb300.model_2u1 import TwoU1Model
from qcmaquis_gb300.model_u1 import U1SpinOrbitalModel
from qcmaquis_gb300.mpo import TaggedMPOMaker
from qcmaquis_gb300.rdm import iterate_nrdm2


def _spins(ss):
    return [(s.get(), s.action()) for s in ss]


def assert_same_mpo(a, b):
    assert len(a) == len(b)
    assert a.core_energy == b.core_energy
    assert list(a.core_labels) == list(b.core_labels)
    for p, (x, y) in enumerate(zip(a, b)):
        assert (x.row_dim, x.col_dim) == (y.row_dim, y.col_dim), p
        assert x.symmetry == y.symmetry
        assert list(x.elements.keys()) == list(y.elements.keys()), p
        for k in x.elements:
            assert x.elements[k] == y.elements[k], (p, k)
            assert x.labels[k] == y.labels[k], (p, k)
        assert x.cols == y.cols and x.row_index == y.row_index, p
        assert x.row_nnz == y.row_nnz and x.col_nnz == y.col_nnz, p
        assert (x.num_one_rows, x.num_one_cols) == (y.num_one_rows, y.num_one_cols), p
        assert _spins(x.left_spins) == _spins(y.left_spins), p
        assert _spins(x.right_spins) == _spins(y.right_spins), p
        assert x.herm.LeftHerm == y.herm.LeftHerm and x.herm.RightHerm == y.herm.RightHerm, p
        assert x.herm.LeftPhase == y.herm.LeftPhase and x.herm.RightPhase == y.herm.RightPhase, p
        assert len(x.op_table) == len(y.op_table)


def _pair(make, merge=True):
    """The same model built twice (site operators are registered into the model's
    tag table while the MPO is made), one MPO from each maker."""
    a = TaggedMPOMaker(make(), merge_site_terms=merge, native=False).create_mpo()
    b = TaggedMPOMaker(make(), merge_site_terms=merge, native=True).create_mpo()
    return a, b


@pytest.mark.parametrize("merge", [True, False])
@pytest.mark.parametrize("L,nelec,seed", [(2, 2, 1), (5, 4, 2), (8, 8, 42)])
def test_su2u1_mpo_equals_python(L, nelec, seed, merge):
    a, b = _pair(lambda: QCModel(L, synthetic_integral_map(L, seed=seed), nelec), merge)
    assert_same_mpo(a, b)
    if L == 8:
        assert any(v != 1 for w in a for v in w.herm.RightPhase)   # the SU(2) phases are exercised


def test_lih_golden_mpo_equals_python(golden):
    lih = golden["lih"]
    a, b = _pair(lambda: QCModel(lih["L"], integral_map(lih["integrals"]), lih["nelec"]))
    assert_same_mpo(a, b)


@pytest.mark.parametrize("merge", [True, False])
def test_twou1_and_u1_mpo_equal_python(merge):
    ints = synthetic_integral_map(5, seed=4)
    assert_same_mpo(*_pair(lambda: TwoU1Model(5, ints, 3, 2), merge))
    ints = synthetic_integral_map(3, seed=5)
    assert_same_mpo(*_pair(lambda: U1SpinOrbitalModel(3, ints, 3), merge))


def test_rdm_measurement_mpo_equals_python():
    """The 2-RDM measurement MPO: one labelled scale per term of every element."""
    L = 5
    def make():
        model = QCModel(L, synthetic_integral_map(L, seed=6), 4)
        ss = SpinSum(model.col)
        terms = [t for pos in iterate_nrdm2(L) for t in ss.V_term(1.0, *pos)]
        return types.SimpleNamespace(L=L, tag_handler=model.tag_handler, ops=model.ops, terms=terms)
    assert_same_mpo(*_pair(make, merge=False))


def test_native_maker_rejects_malformed_input():
    from qcmaquis_gb300 import native as N
    model = QCModel(4, synthetic_integral_map(4, seed=1), 4)
    tags = N.FTagTable(model.tag_handler, model.ops.ident, model.ops.ident_full, model.ops.fill, "su2u1")
    ok = ([0, 2], [0, 3], [model.ops.ident, model.ops.ident], [1.0], [0])
    N.mpo_maker_sites(4, tags, ok, {}, 3, 0)
    with pytest.raises(RuntimeError, match="position out of range"):
        N.mpo_maker_sites(4, tags, ([0, 2], [0, 4], ok[2], [1.0], [0]), {}, 3, 0)
    with pytest.raises(RuntimeError, match="tag out of range"):
        N.mpo_maker_sites(4, tags, ([0, 2], [0, 3], [0, 10 ** 6], [1.0], [0]), {}, 3, 0)
    with pytest.raises(RuntimeError, match="fewer than two"):
        N.mpo_maker_sites(4, tags, ([0, 1], [0], [0], [1.0], [0]), {}, 3, 0)
    with pytest.raises(RuntimeError, match="another site term"):
        _site_terms_twice(N, tags)


def _site_terms_twice(N, tags):
    """Two (TL, TR) element lists for one site are refused."""
    import ctypes as C
    L = N.lib()
    h = C.c_void_p()
    N.check(L.qcm_mpo_maker_create(3, C.byref(tags.c), C.byref(h)))
    try:
        t = np.array([0], dtype=np.int32)
        s = np.array([1.0])
        lab = np.array([-1], dtype=np.int32)
        N.check(L.qcm_mpo_maker_site_terms(h, 1, 1, N._p(t, N.i32p), N._p(s, N.f64p), N._p(lab, N.i32p)))
        N.check(L.qcm_mpo_maker_site_terms(h, 1, 1, N._p(t, N.i32p), N._p(s, N.f64p), N._p(lab, N.i32p)))
    finally:
        L.qcm_mpo_maker_destroy(h)


def test_native_maker_is_finished_once():
    """A failed finish leaves the maker refusing further calls instead of
    building on its partial state."""
    import ctypes as C
    from qcmaquis_gb300 import native as N
    model = QCModel(4, synthetic_integral_map(4, seed=1), 4)
    th = model.tag_handler
    tags = N.FTagTable(th, model.ops.ident, model.ops.ident_full, model.ops.fill, "su2u1")
    L = N.lib()
    h = C.c_void_p()
    N.check(L.qcm_mpo_maker_create(4, C.byref(tags.c), C.byref(h)))
    try:
        t = np.array([0], dtype=np.int32)
        s = np.array([1.0])
        lab = np.array([-1], dtype=np.int32)
        N.check(L.qcm_mpo_maker_site_terms(h, 1, 1, N._p(t, N.i32p), N._p(s, N.f64p), N._p(lab, N.i32p)))
        # a leftmost_right before the chain start puts the trivial right key's identity
        # on site 0, where no bond leads to it: refused
        rc = L.qcm_mpo_maker_finish(h, C.byref(tags.c), -1, 0)
        assert rc != 0
        assert L.qcm_mpo_maker_finish(h, C.byref(tags.c), 3, 0) != 0
        assert "destroy" in L.qcm_last_error().decode()
        assert L.qcm_mpo_maker_site_terms(h, 2, 1, N._p(t, N.i32p), N._p(s, N.f64p), N._p(lab, N.i32p)) != 0
    finally:
        L.qcm_mpo_maker_destroy(h)
