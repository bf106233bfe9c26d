"""Generate tests/golden/bcc_traces.npz: whole-solve outputs of the reference.

For every case in tests/bcc_cases.py the inputs are written as .b16 / .in
files and solved by the reference built from its own sources
(oracle/_ref/lakcluster_ref, `make -C oracle ref`).  The stored golden values
are the text lines of out_trace.txt, out_xdrop_a.txt and out_xdrop_b.txt and,
for the small cases, a digest per (stage, iteration) of every intermediate
product (the LAKBCC_TRACE hash lines of the driver run on the reference's own
kernels), which localises a divergence to the stage that produced it.

Cases without controls: when a bin has no control rows, the reference sums
the columns of the empty control matrix with an SSE loop that always reads one
1920-bit block, i.e. past the end of zero-length buffers, and the neighbouring
allocator bookkeeping it reads adds a small layout-dependent constant to every
SNP's allele count (dir_c/bcc.c:1228 -> An_v.c:49 -> popcount.c:46-69).  The
golden trace for such a case is therefore taken from the reference's kernels
driven by this package's solve driver (oracle/_ref/lakbcc_refkernels), which
reads zeros there; the generator checks that, with the reference program's
constant injected into that one An_v call, the same driver reproduces the
reference program's files byte for byte.

The cases in LARGE_CASES (minutes of reference time) are solved by the
reference program with every host thread; the small cases with one.

usage: python tests/golden/make_bcc_golden.py [case ...]
       python tests/golden/make_bcc_golden.py --large [case ...]   (LARGE_CASES)
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import bcc_cases as bc  # noqa: E402
from lakcluster_c_gb300 import infiles  # noqa: E402


def empty_control_constant(out_dir, A_bins, col_mask):
    """The per-SNP constant the reference added for an empty control matrix."""
    v = infiles_read_mda(os.path.join(out_dir, "AZ_rsum.mda"))
    cs = sum(a.sum(0) for a in A_bins).astype(np.float64)
    d = v - cs
    if col_mask is not None:
        d = d[np.asarray(col_mask, bool)]
    if not np.all(d == d[0]):
        raise RuntimeError("empty-control constant is not uniform: %s" % np.unique(d))
    return float(d[0])


def infiles_read_mda(path):
    raw = open(path, "rb").read()
    hdr = np.frombuffer(raw[:12], np.int32)
    return np.frombuffer(raw[12:], np.float64)[: hdr[1] * hdr[2]]


def make(names):
    # The driver on reference kernels must be built from the current sources.
    subprocess.run(["make", "-s", "-C", os.path.join(os.path.dirname(bc.GOLDEN), "..", "..", "oracle"), "ref"],
                   check=True)
    out = {}
    if os.path.exists(bc.GOLDEN):
        z = np.load(bc.GOLDEN, allow_pickle=False)
        out = {k: z[k] for k in z.files}
    for name in names:
        with tempfile.TemporaryDirectory() as td:
            ind, ref_out, rk_out = os.path.join(td, "in"), os.path.join(td, "ref"), os.path.join(td, "rk")
            p_ref = bc.write_case(name, ind, ref_out, "ref.in")
            p_rk = bc.write_case(name, ind, rk_out, "rk.in")
            large = name in bc.LARGE_CASES
            bc.run_reference(p_ref, threads=(os.cpu_count() or 1) if large else 1)
            ref = bc.read_outputs(ref_out)
            if large or bc.CASES[name][1]:
                golden, source = ref, "reference program"
            else:
                d = bc.build(name)
                k = empty_control_constant(ref_out, d["A"], d.get("col_mask"))
                env = dict(os.environ, LAKREF_EMPTY_Z_ROWSUM=repr(k))
                bc.run_refkernels(p_rk, env=env)
                if bc.read_outputs(rk_out) != ref:
                    raise RuntimeError(name + ": driver on reference kernels does not reproduce the reference")
                bc.run_refkernels(p_rk)
                golden, source = bc.read_outputs(rk_out), "reference kernels (empty-control constant %g removed)" % k
            for key in ("trace", "xdrop_a", "xdrop_b"):
                out[name + "/" + key] = np.array(golden[key])
            if name in bc.SMALL:
                # Stage digests of every intermediate, from the reference kernels.
                tpath = os.path.join(td, "stages.trace")
                bc.run_refkernels(p_rk, env=dict(os.environ, LAKBCC_TRACE=tpath))
                if bc.read_outputs(rk_out) != golden:
                    raise RuntimeError(name + ": driver on reference kernels differs from the golden outputs")
                out[name + "/stages"] = np.array(bc.trace_digest(tpath))
            out[name + "/source"] = np.array([source])
            print("%-34s %4d iterations  %5d drops  (%s)" % (name, len(golden["trace"]), len(golden["xdrop_a"]), source))
    np.savez_compressed(bc.GOLDEN, **out)


if __name__ == "__main__":
    args = sys.argv[1:]
    if args[:1] == ["--large"]:
        make(args[1:] or list(bc.LARGE_CASES))
    else:
        make(args or list(bc.CASES))
