"""Write tests/golden/dcc_traces.npz: the reference program's own outputs
(oracle/_ref/lakcluster_ref, GLOBAL_TEST_TYPE= dexcluster_driver) for the
dexcluster cases of tests/bcc_cases.py (out_trace / out_xdrop_a / out_xdrop_b
lines).

Run from the repository root on an x86-64 host with the reference build:
    python tests/golden/make_dcc_golden.py
"""
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, ".."))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

import bcc_cases as bc  # noqa: E402


def main():
    if not os.path.exists(bc.REF_PROGRAM):
        sys.exit("the reference program (oracle/_ref/lakcluster_ref) is not built")
    out = {}
    for name in bc.DCC_CASES:
        with tempfile.TemporaryDirectory() as td:
            p = bc.write_dcc_case(name, os.path.join(td, "in"), os.path.join(td, "out"))
            bc.run_reference(p)
            res = bc.read_outputs(os.path.join(td, "out"))
        for k in ("trace", "xdrop_a", "xdrop_b"):
            out[name + "/" + k] = np.array(res[k])
        print("%-34s %4d iterations  %5d drops" % (name, len(res["trace"]), len(res["xdrop_a"])))
    np.savez_compressed(bc.DCC_GOLDEN, **out)


if __name__ == "__main__":
    main()
