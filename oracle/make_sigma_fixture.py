"""Writes ``oracle/fixtures/sigma_L24_m1024.npz``: the layouts of the benchmark's
sigma problem (L=24, N=24, S=0 SU2U1, middle sites (11, 12), m=1024) -- the
two-site tensor's indices and blocks, the boundary block layouts L[11] and R[13],
and the flattened two-site MPO tensor of sites (11, 12) -- so that the CPU
baseline runs the C++ oracle on exactly the GPU benchmark's problem without
building the model, the MPS or any layout at run time (and without loading the
library).  Values are not stored: the baseline fills the ket and the
boundaries with seeded normal numbers (the work of a sigma does not depend on
them).

Run once, here:  python oracle/make_sigma_fixture.py
It builds the workload with the package's model, MPS and two-site MPO
builders and takes the boundary layouts from its boundary-step planner.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

from oracle import cpu_sigma as CS  # noqa: E402
from oracle.cpu_sample import boundary_layouts  # noqa: E402


def main(L=24, m=1024):
    from qcmaquis_gb300.workloads import build_sigma_host
    w = build_sigma_host(L=L, m=m)
    Ll, Rl = boundary_layouts(w)
    p = w.psi_host
    keys, shapes = p.data.keys, [b.shape for b in p.data.blocks]
    offs = np.cumsum([0] + [r * c for r, c in shapes])[:-1]
    a = {}
    a.update(CS.index_arrays(p.phys_i, "phys"))
    a.update(CS.index_arrays(p.left_i, "left"))
    a.update(CS.index_arrays(p.right_i, "right"))
    a.update(CS.block_arrays(keys, shapes, offs, "psi"))
    for name, lay in (("L", Ll), ("R", Rl)):
        a.update(CS.block_arrays(lay.keys, lay.shapes, lay.offsets, name))
        a[name + ".blk_ptr"] = np.array(lay.blk_ptr, dtype=np.int32)
    a.update(CS.flatten_mpo(w.ts_mpo))
    a["meta"] = np.array([L, w.nelec, m, w.site], dtype=np.int64)
    os.makedirs(os.path.join(HERE, "fixtures"), exist_ok=True)
    out = os.path.join(HERE, "fixtures", f"sigma_L{L}_m{m}.npz")
    np.savez_compressed(out, **a)
    print(out, os.path.getsize(out), "bytes")


if __name__ == "__main__":
    main()
