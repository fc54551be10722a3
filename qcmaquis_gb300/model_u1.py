"""Quantum-chemistry Hamiltonian in U1 symmetry: spin orbitals as sites, only the
electron number conserved.

The reference's U1-charged chemistry model is the spinor model of
``dmrg/framework/dmrg/models/chem/rel/model.hpp:11-70`` (``rel_qc_model`` on the
``spinors`` lattice): every site is one spin orbital with the two states
|empty> (charge 0) and |occupied> (charge 1) and the local operators
create / destroy / count / fill (``model.hpp:33-44``).  This model keeps that
site basis and operator set for real integrals: the ``2L`` sites are the spin
orbitals of ``L`` spatial orbitals, site ``2p`` = (p, up) and ``2p + 1`` =
(p, down), and the Hamiltonian is the same operator as the SU2U1 and TwoU1
models' (one- and two-electron integrals from the same 8-fold-symmetric map),
now without any spin label on the charges.  Its spectrum in the N-electron
sector is the union of the spectra of every spin sector.

Charges are stored as the pair (N, 0): the reference's single ``int`` charge
(``block_matrix/symmetry/u1.h``) in the first component, so block order equals
the reference's U1 order, and the contractions are the abelian ones.  Fermion
signs come from the Jordan-Wigner string over the site order; the terms are
built as in ``model_2u1`` (one local operator per site per spin-orbital product,
equal strings merged, exact adjoint tags)."""
from __future__ import annotations

from typing import Dict, Tuple

import numpy as np

from .model_2u1 import AbelianChemModel
from .symmetry import Index

# local basis of one spin orbital (index = position in the dense 2x2 matrices)
STATES = [(0, 0), (1, 0)]
EMPTY, OCC = range(2)


def phys_index() -> Index:
    """Physical basis of one spin orbital, descending: (1,0), (0,0)."""
    return Index([((1, 0), 1), ((0, 0), 1)])


def _ladder() -> Dict[str, np.ndarray]:
    """Dense <out|O|in> of the spinor model's operators (``rel/model.hpp:33-44``)."""
    c = np.zeros((2, 2))
    c[OCC, EMPTY] = 1.0          # create: |empty> -> |occupied>
    return {"c": c, "d": c.T.copy(), "n": np.diag([0.0, 1.0]), "F": np.diag([1.0, -1.0]),
            "I": np.eye(2)}


class U1SpinOrbitalModel(AbelianChemModel):
    """``L`` spatial orbitals as ``2L`` spin-orbital sites, ``nelec`` electrons (the
    target charge ``(nelec, 0)``)."""

    symmetry = "u1"
    states = STATES

    def __init__(self, L: int, integrals: Dict[Tuple[int, int, int, int], float], nelec: int,
                 integral_cutoff: float = 1e-20):
        self.n_orb = L
        self.L = 2 * L
        self.nelec = nelec
        self.right_end = (nelec, 0)
        self.phys = phys_index()
        self.integrals = integrals
        self.integral_cutoff = integral_cutoff
        self._init_operators()
        self._create_terms(L)

    def _ladder(self) -> Dict[str, np.ndarray]:
        return _ladder()

    def _so(self, p: int, spin: int, create: bool) -> Tuple[int, str]:
        return 2 * p + spin, "c" if create else "d"


__all__ = ["U1SpinOrbitalModel", "phys_index", "STATES"]
