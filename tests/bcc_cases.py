"""Whole-solve parity cases: seeded inputs, how to write them, how to run them.

Each case is a bcc problem small enough for the reference to solve in seconds
on one core.  Inputs come from lakcluster_c_gb300.synth (numpy PCG64 streams,
identical on x86-64 and aarch64), so the committed golden traces
(tests/golden/bcc_traces.npz, made by tests/golden/make_bcc_golden.py) can be
checked on a machine without the reference.
"""
from __future__ import annotations

import os
import subprocess

import numpy as np

from lakcluster_c_gb300 import infiles, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_DIR = os.path.join(ROOT, "oracle", "_ref")
REF_PROGRAM = os.path.join(REF_DIR, "lakcluster_ref")
REF_KERNELS_DRIVER = os.path.join(REF_DIR, "lakbcc_refkernels")
GOLDEN = os.path.join(ROOT, "tests", "golden", "bcc_traces.npz")


def _masked_case_control():
    inst = synth.case_control(260, 230, 2000, 25, 50, 0.05, nbins=2, seed=5)
    rng = np.random.default_rng(7)
    Am = [(rng.random(a.shape[0]) < 0.85).astype(np.uint8) for a in inst.A_bins]
    Zm = [(rng.random(z.shape[0]) < 0.8).astype(np.uint8) for z in inst.Z_bins]
    cm = (rng.random(inst.ncols) < 0.9).astype(np.uint8)
    return dict(A=inst.A_bins, Z=inst.Z_bins, A_masks=Am, Z_masks=Zm, col_mask=cm, gamma=0.05)


def _case_only(n, m, k, seed):
    inst = synth.case_only(n, m, k=k, flip=0.1, seed=seed)
    return dict(A=inst.A_bins, Z=None, gamma=0.05)


def _covariates(d, T_ncols, seed, kappa_squared):
    """Covariate columns for every bin: column 0 all ones (the reference's
    default covariate), the others Bernoulli(0.5) per row."""
    rng = np.random.default_rng(seed)

    def cols(n):
        c = (rng.random((n, T_ncols)) < 0.5).astype(np.uint8)
        c[:, 0] = 1
        return c
    d["T"] = [cols(a.shape[0]) for a in d["A"]]
    d["S"] = [cols(z.shape[0]) for z in d["Z"]]
    d["kappa_squared"] = kappa_squared
    return d


def _case_control(nA, nZ, m, kr, kc, nbins, seed, gamma=0.05, gamma_type=None, Ireq=None):
    inst = synth.case_control(nA, nZ, m, kr, kc, 0.05, nbins=nbins, seed=seed)
    d = dict(A=inst.A_bins, Z=inst.Z_bins, gamma=gamma)
    if gamma_type is not None:
        d["gamma_type"] = gamma_type
    if Ireq is not None:
        d["Ireq"] = Ireq
    return d


# name -> (builder, has controls in every bin)
CASES = {
    "case_only_200x300": (lambda: _case_only(200, 300, 20, 1), False),
    "case_only_1024x1024": (lambda: _case_only(1024, 1024, 45, 1), False),
    "case_control_2bin_300x250x2100": (lambda: _case_control(300, 250, 2100, 30, 60, 2, 3), True),
    "case_control_2bin_masked": (_masked_case_control, True),
    "case_control_1bin_gamma_lin": (lambda: _case_control(180, 160, 1500, 20, 40, 1, 11, 0.1, 2), True),
    "case_control_3bin_ragged": (lambda: _case_control(333, 271, 1931, 21, 33, 3, 13), True),
    # GLOBAL_Ireq > 0: rows and columns scored by their Ireq-th highest bin
    "case_control_3bin_Ireq1": (lambda: _case_control(300, 280, 2100, 24, 40, 3, 17, Ireq=1), True),
    "case_control_3bin_Ireq2": (lambda: _case_control(330, 290, 1950, 24, 40, 3, 19, Ireq=2), True),
    "case_control_2bin_Ireq2": (lambda: _case_control(260, 240, 2300, 22, 44, 2, 23, Ireq=2), True),
    # covariate columns (T_n_cols > 1): products per covariate, and the MDS
    # correction of bcc_sumscores_ifT when GLOBAL_kappa_squared > 0
    "case_control_2bin_T3": (lambda: _covariates(_case_control(270, 250, 2000, 22, 40, 2, 29), 3, 31, None), True),
    "case_control_2bin_T3_kappa": (lambda: _covariates(_case_control(270, 250, 2000, 22, 40, 2, 29), 3, 31, 0.3),
                                   True),
    "case_control_3bin_T2_kappa_Ireq1": (
        lambda: dict(_covariates(_case_control(320, 300, 1940, 24, 40, 3, 37), 2, 41, 0.5), Ireq=1), True),
    # the ZtSWn column strategy: SNP x SNP products instead of the bit-plane product
    "case_control_2bin_qc_ZtSWn": (lambda: dict(_case_control(280, 240, 1900, 22, 40, 2, 43), qc="ZtSWn"), True),
    "case_control_2bin_T2_qc_ZtSWn": (
        lambda: dict(_covariates(_case_control(250, 230, 1700, 20, 36, 2, 47), 2, 53, 0.4), qc="ZtSWn"), True),
    # the condense row strategy (dense FP64 removed columns and their products)
    # and the store-one column strategy (one covariate at a time)
    "case_control_2bin_qr_condense": (lambda: dict(_case_control(280, 250, 2050, 22, 40, 2, 59), qr="YnWt condense"),
                                      True),
    "case_control_2bin_masked_qr_condense": (lambda: dict(_masked_case_control(), qr="YnWt condense"), True),
    "case_control_2bin_T2_qc_store_one": (
        lambda: dict(_covariates(_case_control(260, 240, 1900, 22, 40, 2, 61), 2, 67, 0.3), qc="YnWt store one"),
        True),
    "case_control_3bin_qr_condense_qc_store_one": (
        lambda: dict(_case_control(300, 270, 1800, 22, 36, 3, 71), qr="YnWt condense", qc="YnWt store one"), True),
}
# Cases whose reference solve takes minutes even on every host thread (the
# 4096 + 4096 x 16384 two-bin workload: 518 s on 8 cores): their golden
# outputs also come from the reference program, run once by the generator with
# all host threads (the reference's outputs do not depend on the thread
# count); the CPU test suite does not re-run them.
LARGE_CASES = {
    "case_control_4096x4096x16384": (lambda: _case_control(4096, 4096, 16384, 256, 512, 2, 2), True),
}
SMALL = ["case_only_200x300", "case_control_2bin_300x250x2100", "case_control_2bin_masked",
         "case_control_1bin_gamma_lin", "case_control_3bin_ragged", "case_control_3bin_Ireq1",
         "case_control_3bin_Ireq2", "case_control_2bin_Ireq2", "case_control_2bin_T3", "case_control_2bin_T3_kappa",
         "case_control_3bin_T2_kappa_Ireq1", "case_control_2bin_qc_ZtSWn", "case_control_2bin_T2_qc_ZtSWn",
         "case_control_2bin_qr_condense", "case_control_2bin_masked_qr_condense", "case_control_2bin_T2_qc_store_one",
         "case_control_3bin_qr_condense_qc_store_one"]


def build(name):
    return (CASES.get(name) or LARGE_CASES[name])[0]()


def write_case(name, in_dir, out_dir, fname="bcc.in", extra_statements=()):
    d = build(name)
    return infiles.write_bcc_inputs(in_dir, out_dir, d["A"], d.get("Z"), gamma=d["gamma"], B_MLT=32,
                                    A_row_masks=d.get("A_masks"), Z_row_masks=d.get("Z_masks"),
                                    col_mask=d.get("col_mask"), gamma_type=d.get("gamma_type"), Ireq=d.get("Ireq"),
                                    T_bins=d.get("T"), S_bins=d.get("S"), kappa_squared=d.get("kappa_squared"),
                                    qc_strategy=d.get("qc", "YnWt"), qr_strategy=d.get("qr", "YnWt"), name=fname,
                                    extra_statements=extra_statements)


# --- scorebox and scramble cases -------------------------------------------------
#
# Scorebox (GLOBAL_TEST_TYPE lakcluster_scorebox): (case, (row_max, row_num,
# col_max, col_num)) over the case's own solve order (its golden out_xdrop_a
# lines).  The per-step row count stays within the lrup row buffers the
# reference sizes from its gamma schedule (2 * ceil(0.05 * rows) here); larger
# steps write past them in the reference (see lakcluster_c_gb300/csrc/
# bcc_driver.cpp, load).  row_max > col_max steps rows in the inner loop
# (lakcluster_scorebox_rc), otherwise columns (_cr).
SCOREBOX = {
    "sb_2bin_cr": ("case_control_2bin_300x250x2100", (20, 3, 200, 3)),
    "sb_2bin_rc": ("case_control_2bin_300x250x2100", (45, 4, 40, 3)),
    "sb_3bin_ragged_cr": ("case_control_3bin_ragged", (20, 3, 200, 4)),
    "sb_3bin_Ireq1_rc": ("case_control_3bin_Ireq1", (24, 3, 10, 3)),
    "sb_2bin_T3_kappa_cr": ("case_control_2bin_T3_kappa", (20, 3, 200, 3)),
    "sb_2bin_qc_ZtSWn_rc": ("case_control_2bin_qc_ZtSWn", (24, 3, 10, 3)),
}
SCOREBOX_ARRAYS = ("A_rpop_j_total", "A_cpop_j", "Irem", "QR_avg", "QC_avg")

# Scramble (GLOBAL_scramble_num): (case, [(rows, cols, seed), ...]); each
# scramble redraws the case entries of the last `rows` rows and `cols`
# columns of the case's solve order (the planted block), with that seed.
SCRAMBLE = {
    "scr_2bin": ("case_control_2bin_300x250x2100", [(40, 200, 7)]),
    "scr_3bin_ragged": ("case_control_3bin_ragged", [(30, 150, 3)]),
    "scr_2bin_masked_two": ("case_control_2bin_masked", [(25, 300, 11), (10, 60, 2)]),
    "scr_2bin_T3": ("case_control_2bin_T3", [(40, 200, 5)]),
}


def scramble_xdrop_lines(xdrop_a, rows, cols):
    """The out_xdrop lines a scramble reads: the last `rows` row lines and the
    last `cols` column lines of a solve's out_xdrop_a."""
    r = [ln for ln in xdrop_a if not ln.startswith("-1")]
    c = [ln for ln in xdrop_a if ln.startswith("-1")]
    return r[len(r) - rows:] + c[len(c) - cols:]


def write_scorebox_case(key, xdrop_a, in_dir, out_dir, fname="bcc.in"):
    """The .in of scorebox `key` (of SCOREBOX or DCC_SCOREBOX) over the solve
    order xdrop_a (text lines); the order is written to
    in_dir/scorebox_xdrop.txt."""
    dcc = key in DCC_SCOREBOX
    name, (rmax, rnum, cmax, cnum) = (DCC_SCOREBOX if dcc else SCOREBOX)[key]
    os.makedirs(in_dir, exist_ok=True)
    xp = os.path.abspath(os.path.join(in_dir, "scorebox_xdrop.txt"))
    with open(xp, "w") as f:
        f.write("\n".join(xdrop_a) + "\n")
    return write_case(name, in_dir, out_dir, fname, extra_statements=(
        ("GLOBAL_TEST_TYPE", "dexcluster_scorebox" if dcc else "lakcluster_scorebox"), ("GLOBAL_scorebox_out_xdrop", xp),
        ("GLOBAL_scorebox_row_max", rmax), ("GLOBAL_scorebox_row_num", rnum),
        ("GLOBAL_scorebox_col_max", cmax), ("GLOBAL_scorebox_col_num", cnum)))


def write_scramble_case(key, xdrop_a, in_dir, out_dir, fname="bcc.in"):
    """The .in of scramble `key` (of SCRAMBLE or DCC_SCRAMBLE), its out_xdrop
    files cut from xdrop_a."""
    dcc = key in DCC_SCRAMBLE
    name, specs = (DCC_SCRAMBLE if dcc else SCRAMBLE)[key]
    os.makedirs(in_dir, exist_ok=True)
    files, seeds = [], []
    for i, (rows, cols, seed) in enumerate(specs):
        xp = os.path.abspath(os.path.join(in_dir, "scramble_xdrop_%d.txt" % i))
        with open(xp, "w") as f:
            f.write("\n".join(scramble_xdrop_lines(xdrop_a, rows, cols)) + "\n")
        files.append(xp)
        seeds.append(str(seed))
    return write_case(name, in_dir, out_dir, fname, extra_statements=(
        ("GLOBAL_TEST_TYPE", "dexcluster_driver" if dcc else "lakcluster_driver"), ("GLOBAL_scramble_num", len(specs)), ("GLOBAL_scramble_out_xdrop_", ",".join(files)),
        ("GLOBAL_scramble_rseed_", ",".join(seeds))))


def read_scorebox(out_dir, grid):
    """The five scorebox arrays (row_num x col_num) a scorebox run wrote."""
    rmax, rnum, cmax, cnum = grid
    out = {}
    for a in SCOREBOX_ARRAYS:
        path = os.path.join(out_dir, "scorebox_r%dn%d_c%dn%d_%s.mda" % (rmax, rnum, cmax, cnum, a))
        raw = open(path, "rb").read()
        hdr = np.frombuffer(raw[:12], np.int32)
        dt = np.float64 if a.endswith("avg") else np.int32
        assert list(hdr) == [2, rnum, cnum], (path, hdr)
        out[a] = np.frombuffer(raw[12:], dt).reshape(cnum, rnum).T.copy()
    return out


SCOREBOX_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bcc_scorebox.npz")


def load_scorebox_golden():
    z = np.load(SCOREBOX_GOLDEN, allow_pickle=False)
    sb = {k: {a: z["%s/%s" % (k, a)] for a in SCOREBOX_ARRAYS} for k in SCOREBOX}
    scr = {k: {key: [str(s) for s in z["%s/%s" % (k, key)]] for key in ("trace", "xdrop_a", "xdrop_b", "b16_sha1")}
           for k in SCRAMBLE}
    return sb, scr


def b16_digests(out_dir):
    """sha1 of each *_scramble_*.b16 file a scrambled solve wrote, by name."""
    import hashlib
    return sorted("%s %s" % (f, hashlib.sha1(open(os.path.join(out_dir, f), "rb").read()).hexdigest())
                  for f in os.listdir(out_dir) if f.endswith(".b16") and "_scramble_" in f)


def read_outputs(out_dir):
    """The three output files as lists of text lines."""
    res = {}
    for key, fn in (("trace", "out_trace.txt"), ("xdrop_a", "out_xdrop_a.txt"), ("xdrop_b", "out_xdrop_b.txt")):
        with open(os.path.join(out_dir, fn)) as f:
            res[key] = [ln.rstrip("\n") for ln in f if ln.strip()]
    return res


def run_reference(in_path, env=None, threads=1):
    """The reference program on a .in file; threads > 1 rewrites the .in's
    thread count (and turns on its OpenMP loops) first."""
    if threads > 1:
        txt = open(in_path).read().replace("GLOBAL_thread_count= 1;", "GLOBAL_thread_count= %d;" % threads)
        with open(in_path, "w") as f:
            f.write(txt.replace("GLOBAL_omp_type= 0;", "GLOBAL_omp_type= 1;"))
    with open(in_path) as f:
        r = subprocess.run([REF_PROGRAM], stdin=f, stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                           env=env, text=True)
    if r.returncode != 0:
        raise RuntimeError("reference program failed:\n" + r.stdout[-2000:])


def run_refkernels(in_path, env=None):
    r = subprocess.run([REF_KERNELS_DRIVER, in_path], stdout=subprocess.PIPE, stderr=subprocess.STDOUT,
                       env=env, text=True)
    if r.returncode != 0:
        raise RuntimeError("driver on reference kernels failed:\n" + r.stdout[-2000:])


def trace_digest(path):
    """Per (stage, iteration) digest of a LAKBCC_TRACE file: one line each."""
    import hashlib
    out, cur, h = [], None, None
    with open(path) as f:
        for ln in f:
            parts = ln.split(" ", 2)
            key = parts[0] + " " + parts[1]
            if key != cur:
                if cur is not None:
                    out.append(cur + " " + h.hexdigest()[:16])
                cur, h = key, hashlib.sha1()
            h.update(ln.encode())
    if cur is not None:
        out.append(cur + " " + h.hexdigest()[:16])
    return out


def load_golden():
    z = np.load(GOLDEN, allow_pickle=False)
    out = {}
    for name in list(CASES) + list(LARGE_CASES):
        if name + "/trace" in z:
            out[name] = {k: [str(s) for s in z[name + "/" + k]] for k in ("trace", "xdrop_a", "xdrop_b")}
            if name + "/stages" in z:
                out[name]["stages"] = [str(s) for s in z[name + "/stages"]]
    return out


# --- the GPU library's whole-solve entry points --------------------------------

def bind_solve(lib):
    from lakcluster_c_gb300 import solve as sv
    return sv.bind(lib)


def solve_in_memory(lib, name):
    """Run a case through lakgb_bcc_solve; returns the outputs as text lines."""
    return solve_arrays(lib, build(name))


def solve_arrays(lib, d):
    """lakgb_bcc_solve on a problem given as 0/1 arrays (see the CASES builders)."""
    from lakcluster_c_gb300 import solve as sv
    p = sv.Problem(d["A"], d.get("Z"), gamma=d["gamma"], gamma_type=d.get("gamma_type") or 0,
                   A_masks=d.get("A_masks"), Z_masks=d.get("Z_masks"), col_mask=d.get("col_mask"),
                   Ireq=d.get("Ireq") or 0, T_bins=d.get("T"), S_bins=d.get("S"),
                   kappa_squared=d.get("kappa_squared") or 0.0, qc_strategy=d.get("qc", "YnWt"),
                   qr_strategy=d.get("qr", "YnWt"), lib=lib)
    return p.solve()


# --- dexcluster (GLOBAL_TEST_TYPE dexcluster_driver) -------------------------------
# The dcc method on case/control inputs of the bcc cases (the case-only input
# is left out: without controls the reference reads past an empty buffer).
DCC_CASES = ["case_control_2bin_300x250x2100", "case_control_1bin_gamma_lin", "case_control_2bin_masked",
             "case_control_3bin_ragged", "case_control_3bin_Ireq1", "case_control_2bin_Ireq2",
             "case_control_2bin_T3_kappa", "case_control_3bin_T2_kappa_Ireq1"]
DCC_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "dcc_traces.npz")


def write_dcc_case(name, in_dir, out_dir, fname="bcc.in"):
    return write_case(name, in_dir, out_dir, fname, extra_statements=(("GLOBAL_TEST_TYPE", "dexcluster_driver"),))


def load_dcc_golden():
    z = np.load(DCC_GOLDEN, allow_pickle=False)
    return {n: {k: [str(s) for s in z[n + "/" + k]] for k in ("trace", "xdrop_a", "xdrop_b")} for n in DCC_CASES}

# dexcluster scorebox (dexcluster_scorebox, dir_c/dexcluster_scorebox.c) and
# scramble (wrap_dcc_scramble), over the dexcluster solve orders
DCC_SCOREBOX = {
    "dsb_2bin_cr": ("case_control_2bin_300x250x2100", (20, 3, 200, 3)),
    "dsb_3bin_Ireq1_rc": ("case_control_3bin_Ireq1", (45, 4, 40, 3)),
    "dsb_2bin_T3_kappa_cr": ("case_control_2bin_T3_kappa", (30, 4, 300, 3)),
}
DCC_SCRAMBLE = {
    "dscr_2bin": ("case_control_2bin_300x250x2100", [(40, 200, 5)]),
    "dscr_3bin_ragged": ("case_control_3bin_ragged", [(30, 150, 3), (12, 40, 8)]),
}


def load_dcc_extra_golden():
    z = np.load(DCC_GOLDEN, allow_pickle=False)
    sb = {k: {a: z["%s/%s" % (k, a)] for a in SCOREBOX_ARRAYS} for k in DCC_SCOREBOX}
    scr = {k: {key: [str(s) for s in z["%s/%s" % (k, key)]] for key in ("trace", "xdrop_a", "xdrop_b", "b16_sha1")}
           for k in DCC_SCRAMBLE}
    return sb, scr
