"""Extract the reference's own golden values into ``reference_fixtures.json``.

Reads, as text, the reference test sources:

* ``dmrg/tests/Fixtures/LiHFixture.h:29-94`` -- LiH CAS integrals (L=4, N=2)
  and ``:112`` reference energy;
* ``dmrg/tests/Fixtures/H2Fixture.h:26-35`` -- H2 integrals (L=2, N=2);
* ``dmrg/tests/test1.cpp:93`` -- H2 ground-state energy; ``:95-118`` -- the sum of
  its 1-RDM elements (0,0) and (1,1) and its 2-RDM element (0,0,0,0);
* ``dmrg/tests/test_wigner.cpp:21-45`` -- 24 Wigner 9j values;
* ``dmrg/tests/test2.cpp:60-120`` -- the LiH (SU2U1) ground-state 2-RDM
  (measurement ``twoptdm``): index quadruples and values;
* ``dmrg/tests/test2.cpp:138`` -- the LiH (SU2U1) first excited singlet energy,
  optimised orthogonal to the ground state (``n_ortho_states = 1``).

Run from the repository root with the reference mounted at REFERENCE (default
``/root/reference``); the JSON it writes is committed so tests never need the
reference tree at run time.
"""
import json
import os
import re
import sys

REF = os.environ.get("REFERENCE", "/root/reference")
HERE = os.path.dirname(os.path.abspath(__file__))

NUM = r"[-+]?\d*\.?\d+(?:[eE][-+]?\d+)?"


def parse_integral_map(text):
    out = []
    for m in re.finditer(r"\{\s*\{\s*(\d+)\s*,\s*(\d+)\s*,\s*(\d+)\s*,\s*(\d+)\s*\}\s*,\s*(" + NUM + r")\s*\}", text):
        out.append([int(m.group(1)), int(m.group(2)), int(m.group(3)), int(m.group(4)), float(m.group(5))])
    return out


def main():
    lih = open(os.path.join(REF, "dmrg/tests/Fixtures/LiHFixture.h")).read()
    h2 = open(os.path.join(REF, "dmrg/tests/Fixtures/H2Fixture.h")).read()
    t1 = open(os.path.join(REF, "dmrg/tests/test1.cpp")).read()
    tw = open(os.path.join(REF, "dmrg/tests/test_wigner.cpp")).read()
    t2 = open(os.path.join(REF, "dmrg/tests/test2.cpp")).read()

    lih_ints = parse_integral_map(lih)
    lih_e = float(re.search(r"referenceEnergy\s*=\s*(" + NUM + ")", lih).group(1))
    h2_ints = parse_integral_map(h2)
    h2_e = float(re.search(r"BOOST_CHECK_CLOSE\(interface\.energy\(\),\s*(" + NUM + ")", t1).group(1))
    wig = []
    for m in re.finditer(r"\{\s*\{([-\d,\s]+)\}\s*,\s*(" + NUM + r")\s*\}", tw):
        args = [int(x) for x in m.group(1).replace(" ", "").split(",") if x]
        if len(args) == 9:
            wig.append([args, float(m.group(2))])

    # test2.cpp: const rdm_measurement ref_2rdm = { { {i,j,k,l}, ... }, std::vector<double> { ... } };
    blk = t2[t2.index("ref_2rdm"):]
    blk = blk[:blk.index("check_measurement_mat")]
    idx_part, val_part = blk.split("std::vector<double>")
    rdm_idx = [[int(x) for x in m.groups()] for m in
               re.finditer(r"\{\s*(\d+)\s*,\s*(\d+)\s*,\s*(\d+)\s*,\s*(\d+)\s*\}", idx_part)]
    rdm_val = [float(x) for x in re.findall(NUM, val_part[val_part.index("{"):])]
    if len(rdm_idx) != len(rdm_val):
        raise SystemExit(f"2-RDM parse mismatch: {len(rdm_idx)} indices, {len(rdm_val)} values")

    # test1.cpp: the H2 1-RDM's diagonal sum and the 2-RDM element {0,0,0,0}
    h2_1rdm_trace = float(re.search(r"BOOST_CHECK_CLOSE\(value,\s*(" + NUM + r")\s*,", t1).group(1))
    h2_2rdm_0000 = float(re.findall(r"BOOST_CHECK_CLOSE\(value,\s*(" + NUM + r")\s*,", t1)[1])

    s1 = re.search(r"ref_energy_excited_state\s*=\s*su2\s*\?\s*(" + NUM + ")", t2)
    lih_s1 = float(s1.group(1))

    data = {
        "source": "values read from the reference test sources by tests/golden/make_golden.py",
        "lih": {"L": 4, "nelec": 2, "spin": 0, "integrals": lih_ints, "energy": lih_e,
                "cite": "dmrg/tests/Fixtures/LiHFixture.h:29-94,112; dmrg/tests/test2.cpp:57"},
        "h2": {"L": 2, "nelec": 2, "spin": 0, "integrals": h2_ints, "energy": h2_e,
               "cite": "dmrg/tests/Fixtures/H2Fixture.h:26-35; dmrg/tests/test1.cpp:93"},
        "wigner9j": {"cases": wig, "rel_tol_percent": 1e-6, "cite": "dmrg/tests/test_wigner.cpp:21-45"},
        "lih_2rdm": {"index": rdm_idx, "value": rdm_val, "cite": "dmrg/tests/test2.cpp:60-120 (twoptdm)"},
        "h2_rdm": {"onerdm_00_plus_11": h2_1rdm_trace, "twordm_0000": h2_2rdm_0000, "rel_tol_percent": 1e-7,
                   "cite": "dmrg/tests/test1.cpp:95-118"},
        "lih_s1": {"energy": lih_s1, "rel_tol_percent": 1e-7,
                   "cite": "dmrg/tests/test2.cpp:122-139 (SU2U1 excited singlet, one orthogonal state)"},
    }
    with open(os.path.join(HERE, "reference_fixtures.json"), "w") as f:
        json.dump(data, f, indent=1)
    print(f"LiH {len(lih_ints)} integrals E={lih_e}; H2 {len(h2_ints)} integrals E={h2_e}; {len(wig)} 9j cases; "
          f"LiH 2-RDM {len(rdm_val)} elements; LiH S1 E={lih_s1}")


if __name__ == "__main__":
    sys.exit(main())
