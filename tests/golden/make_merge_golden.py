"""Write tests/golden/b16_merge.npz: the reference program's own outputs
(oracle/_ref/lakcluster_ref, GLOBAL_TEST_TYPE= b16_merge) for the synthetic
studies of tests/bed_cases.py (MERGE_CASES) -- the merged .b16, .bim and .fam
files it writes.

Run from the repository root on an x86-64 host with the reference build:
    python tests/golden/make_merge_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, ".."))
sys.path.insert(0, os.path.join(HERE, "..", ".."))

import bcc_cases as bc  # noqa: E402
import bed_cases as bd  # noqa: E402


def main():
    if not os.path.exists(bc.REF_PROGRAM):
        sys.exit("the reference program (oracle/_ref/lakcluster_ref) is not built")
    out = {}
    for name in bd.MERGE_CASES:
        with tempfile.TemporaryDirectory() as td:
            bd.write_merge_case(name, os.path.join(td, "in"))
            os.makedirs(os.path.join(td, "out"))
            p = os.path.join(td, "run.in")
            with open(p, "w") as f:
                f.write(bd.merge_in_text(name, os.path.join(td, "in"), os.path.join(td, "out")))
            with open(p) as f:
                r = subprocess.run([bc.REF_PROGRAM], stdin=f, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
            if r.returncode != 0:
                raise RuntimeError(name + ": reference program failed")
            files = bd.read_outputs(name, os.path.join(td, "out"))
        for k, v in files.items():
            out["%s/%s" % (name, k)] = np.frombuffer(v, np.uint8)
        print("%-16s b16 %7d  bim %7d  fam %6d bytes" % (name, len(files["b16"]), len(files["bim"]), len(files["fam"])))
    np.savez_compressed(bd.MERGE_GOLDEN, **out)


if __name__ == "__main__":
    main()
