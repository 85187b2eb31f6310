"""Writes input_random_init_golden.json and input_single_element_golden.json: the initial
configurations the reference's INIT RANDOM and cell-status draws produce for
input_two_element_2d.json and input_single_element_2d.json, computed by
reference_init.py on the reference's own Random:: functions (compiled from the reference
tree by oracle/ref_build.sh). tests/test_input.py compares the library's
cil_input_initial_state with it.

Usage: python tests/golden/make_input_golden.py   (needs the reference tree; not run by tests)
"""
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)

import reference_init as R  # noqa: E402


def main():
    subprocess.run(["bash", os.path.join(ROOT, "oracle", "ref_build.sh")], check=True)
    doc = json.load(open(os.path.join(HERE, "input_two_element_2d.json")))
    pos, tsw = R.reference_init(**R.from_fixture(doc))
    out = {"source": "reference Random.cpp + mt/dSFMT.c (oracle/ref_build.sh), draw order of Input.cpp:736-757 "
                     "and CIL.cuh:253-330, fixture input_two_element_2d.json",
           "pos": [float(x).hex() for x in pos.ravel()], "tswitch": [int(t) for t in tsw]}
    path = os.path.join(HERE, "input_random_init_golden.json")
    with open(path, "w") as f:
        json.dump(out, f)
    print(path, len(out["tswitch"]), "cells")
    # single-element species (the cell-cycle model)
    doc = json.load(open(os.path.join(HERE, "input_single_element_2d.json")))
    md, dv = doc["MD"], doc["SPECIES"]["C1"]["DIVISION"]
    pos, theta, angvel = R.reference_cycle_init(doc["RUNTIME"]["RNG"]["SEED"], doc["INIT"]["C1"]["RANDOM"]["NUMBER"],
                                                md["DIM"], md["BOX"],
                                                (dv["TAU_DIVISION"]["AVG"], dv["TAU_DIVISION"]["SIGMA"]),
                                                md["DT"]["MANUAL"])
    out = {"source": "reference Random.cpp + mt/dSFMT.c (oracle/ref_build.sh), draw order of Input.cpp:736-757 "
                     "(one element) and CIL.cuh:253-330, fixture input_single_element_2d.json",
           "pos": [float(x).hex() for x in pos.ravel()], "theta": [float(x).hex() for x in theta],
           "angvel": [float(x).hex() for x in angvel]}
    path = os.path.join(HERE, "input_single_element_golden.json")
    with open(path, "w") as f:
        json.dump(out, f)
    print(path, len(out["theta"]), "cells")


if __name__ == "__main__":
    main()
