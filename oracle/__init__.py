"""CPU oracle for the two-site SU2U1 DMRG hot path -- TEST INFRASTRUCTURE ONLY.

This package restates, in numpy, the reference algorithm of QCMaquis's
two-site optimisation step (sigma vector, boundary updates, Jacobi-Davidson,
SVD truncation, sweep schedule); every function cites the reference file and
lines it follows.  It exists to check the GPU library.  Only ``tests/``,
``__graft_entry__.smoke()`` and the ``cpu_baseline`` / ``--impl reference``
legs of ``bench.py`` may import it; the product (``qcmaquis_gb300``) never
does, and never falls back to it.

Parity pin: the reference cannot be compiled here (it needs Boost, GSL and
HDF5), so the oracle is pinned by the reference's own golden values -- the
LiH and H2 ground-state energies of ``dmrg/tests/test2.cpp:57`` and
``dmrg/tests/test1.cpp:93`` and the Wigner 9j table of
``dmrg/tests/test_wigner.cpp:21-45`` -- and by exact diagonalisation
(``oracle/fci.py``) of the same Hamiltonians.
"""
