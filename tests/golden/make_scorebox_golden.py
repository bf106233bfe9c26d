"""Write tests/golden/bcc_scorebox.npz: outputs of the reference program itself
(oracle/_ref/lakcluster_ref, compiled from the reference's sources by
oracle/Makefile) for the scorebox and scramble cases of tests/bcc_cases.py.

Each case starts from the solve order of its plain solve -- the golden
out_xdrop_a lines of tests/golden/bcc_traces.npz, which are the reference
program's own for every case with controls:

  * scorebox (GLOBAL_TEST_TYPE lakcluster_scorebox): the five row_num x
    col_num arrays it writes (A_rpop_j_total, A_cpop_j, Irem, QR_avg, QC_avg);
  * scramble (GLOBAL_scramble_num > 0): the scrambled solve's out_trace /
    out_xdrop_a / out_xdrop_b lines and the sha1 of each
    *_scramble_{pre,pos}.b16 file it writes.

Run from the repository root on an x86-64 host with the reference build:
    python tests/golden/make_scorebox_golden.py
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
    golden = bc.load_golden()
    out = {}
    for key, (name, grid) in bc.SCOREBOX.items():
        with tempfile.TemporaryDirectory() as td:
            p = bc.write_scorebox_case(key, golden[name]["xdrop_a"], os.path.join(td, "in"), os.path.join(td, "out"))
            bc.run_reference(p)
            arrays = bc.read_scorebox(os.path.join(td, "out"), grid)
        for a, v in arrays.items():
            out["%s/%s" % (key, a)] = v
        print("%-22s %-34s grid %s" % (key, name, grid))
    for key, (name, specs) in bc.SCRAMBLE.items():
        with tempfile.TemporaryDirectory() as td:
            p = bc.write_scramble_case(key, golden[name]["xdrop_a"], os.path.join(td, "in"), os.path.join(td, "out"))
            bc.run_reference(p)
            res = bc.read_outputs(os.path.join(td, "out"))
            digests = bc.b16_digests(os.path.join(td, "out"))
        for k in ("trace", "xdrop_a", "xdrop_b"):
            out["%s/%s" % (key, k)] = np.array(res[k])
        out["%s/b16_sha1" % key] = np.array(digests)
        print("%-22s %-34s %d iterations, %d snapshot files" % (key, name, len(res["trace"]), len(digests)))
    np.savez_compressed(bc.SCOREBOX_GOLDEN, **out)


if __name__ == "__main__":
    main()
