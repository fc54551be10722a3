"""Regenerate ``oracle_L8_m64.json``: the oracle's two-site sweep on the plain
L=8, N=8, S=0 SU2U1 case (seeded synthetic integrals, diagonal in [-2,-0.5]),
m=64, 6 sweeps, default_mps_init seed 42.  Run from the repository root."""
import json
import os
import sys
import time

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from qcmaquis_gb300.integrals import synthetic_integral_map  # noqa: E402
from qcmaquis_gb300.model import QCModel  # noqa: E402
from qcmaquis_gb300.mpo import make_mpo  # noqa: E402
from oracle.sweep import SweepParams, run_dmrg  # noqa: E402


def main():
    L, N = 8, 8
    model = QCModel(L, synthetic_integral_map(L, seed=0, diag_range=(-2.0, -0.5)), N)
    mpo = make_mpo(model)
    t = time.time()
    rec, _ = run_dmrg(model, mpo, SweepParams(nsweeps=6, max_bond_dimension=64), nelec=N)
    out = {"case": "L=8 N=8 S=0 m=64 6 sweeps, integrals seed 0, init seed 42",
           "energies": rec.energies, "sweep_energy": rec.sweep_energy, "tw": rec.truncated_weight,
           "sweep_tw": rec.sweep_truncated_weight, "bond_dimension": rec.bond_dimension,
           "oracle_seconds": time.time() - t}
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_L8_m64.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    main()
