"""Write tests/golden/dcc_traces.npz: the reference program's own outputs
(oracle/_ref/lakcluster_ref, GLOBAL_TEST_TYPE= dexcluster_driver) for the
dexcluster cases of tests/bcc_cases.py (out_trace / out_xdrop_a / out_xdrop_b
lines), and of its scorebox (GLOBAL_TEST_TYPE= dexcluster_scorebox, the five
grid arrays) and scramble (the scrambled solve's lines and the sha1 of its
.b16 snapshots) over those solve orders.

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
    orders = {n: list(out[n + "/xdrop_a"]) for n in bc.DCC_CASES}
    for key, (name, grid) in bc.DCC_SCOREBOX.items():
        with tempfile.TemporaryDirectory() as td:
            p = bc.write_scorebox_case(key, orders[name], os.path.join(td, "in"), os.path.join(td, "out"))
            bc.run_reference(p)
            for a, v in bc.read_scorebox(os.path.join(td, "out"), grid).items():
                out["%s/%s" % (key, a)] = v
        print("%-22s %-34s grid %s" % (key, name, grid))
    for key, (name, specs) in bc.DCC_SCRAMBLE.items():
        with tempfile.TemporaryDirectory() as td:
            p = bc.write_scramble_case(key, orders[name], os.path.join(td, "in"), os.path.join(td, "out"))
            bc.run_reference(p)
            res = bc.read_outputs(os.path.join(td, "out"))
            out["%s/b16_sha1" % key] = np.array(bc.b16_digests(os.path.join(td, "out")))
        for k in ("trace", "xdrop_a", "xdrop_b"):
            out["%s/%s" % (key, k)] = np.array(res[k])
        print("%-22s %-34s %d iterations" % (key, name, len(res["trace"])))
    np.savez_compressed(bc.DCC_GOLDEN, **out)


if __name__ == "__main__":
    main()
