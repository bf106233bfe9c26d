"""Whole bcc solves on the GPU library (lakgb_bcc_solve / lakgb_bcc_run_in_file).

`solve(A_bins, Z_bins, ...)` takes per-bin 0/1 matrices (rows x SNPs, 1 = the
minor allele), packs them MSB-first the way the reference's .b16 files are,
and returns the solve's outputs: the per-iteration trace and the elimination
order, both as the text lines the reference writes to out_trace.txt and
out_xdrop_{a,b}.txt (dir_c/bcc_sumscores.c:143-153).  `run_in_file(path)`
runs a reference .in file and writes those files itself.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import load


class BccBin(C.Structure):
    _fields_ = [("A_nrows", C.c_int), ("A_rows", C.c_void_p), ("A_mr_b", C.c_void_p),
                ("Z_nrows", C.c_int), ("Z_rows", C.c_void_p), ("Z_mr_b", C.c_void_p),
                ("T_rows", C.c_void_p), ("S_rows", C.c_void_p)]


class BccProblem(C.Structure):
    _fields_ = [("ncols", C.c_int), ("row_bytes", C.c_longlong), ("mc_b", C.c_void_p),
                ("nbins", C.c_int), ("bins", C.POINTER(BccBin)),
                ("B_MLT", C.c_int), ("gamma", C.c_double), ("gamma_type", C.c_int), ("test_sparse", C.c_int),
                ("Ireq", C.c_int), ("T_ncols", C.c_int), ("kappa_squared", C.c_double),
                ("QC_strategy", C.c_char_p), ("QR_strategy", C.c_char_p)]


class BccResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("trace", C.POINTER(C.c_double)),
                ("n_xdrop", C.c_int), ("xdrop_a", C.POINTER(C.c_int)), ("xdrop_b", C.POINTER(C.c_int))]


def bind(lib):
    lib.lakgb_bcc_problem_init.argtypes = [C.POINTER(BccProblem)]
    lib.lakgb_bcc_solve.argtypes = [C.POINTER(BccProblem), C.POINTER(BccResult)]
    lib.lakgb_bcc_solve.restype = C.c_int
    lib.lakgb_bcc_result_free.argtypes = [C.POINTER(BccResult)]
    lib.lakgb_bcc_run_in_file.argtypes = [C.c_char_p]
    lib.lakgb_bcc_run_in_file.restype = C.c_int
    lib.lakgb_bcc_last_error.argtypes = [C.c_char_p, C.c_int]
    return lib


def pack_rows(bits) -> np.ndarray:
    """0/1 array (..., n) -> packed rows of rup(n,16)/8 bytes, MSB first."""
    bits = np.asarray(bits, np.uint8)
    n = bits.shape[-1]
    pad = (16 - n % 16) % 16
    if pad:
        bits = np.concatenate([bits, np.zeros(bits.shape[:-1] + (pad,), np.uint8)], axis=-1)
    return np.ascontiguousarray(np.packbits(bits, axis=-1, bitorder="big"))


class Problem:
    """A packed bcc problem kept alive for repeated solves.  A_bins / Z_bins
    are per-bin 0/1 arrays (rows x SNPs), or, with ``packed_ncols`` given,
    rows already packed as pack_rows packs them (``packed_ncols`` SNPs)."""

    def __init__(self, A_bins, Z_bins=None, *, gamma=0.125, B_MLT=32, gamma_type=0, A_masks=None,
                 Z_masks=None, col_mask=None, test_sparse=1, Ireq=0, T_bins=None, S_bins=None,
                 kappa_squared=0.0, qc_strategy="YnWt", qr_strategy="YnWt", lib=None, packed_ncols=None):
        self.lib = bind(lib or load())
        self._keep = []
        nb = len(A_bins)
        Z_bins = Z_bins if Z_bins is not None else [None] * nb
        ncols = packed_ncols if packed_ncols is not None else np.asarray(A_bins[0]).shape[1]
        pk = (lambda x: np.ascontiguousarray(x, np.uint8)) if packed_ncols is not None else pack_rows
        self.bins = (BccBin * nb)()
        for b in range(nb):
            a = np.asarray(A_bins[b], np.uint8)
            pa = self._hold(pk(a))
            self.bins[b].A_nrows = a.shape[0]
            self.bins[b].A_rows = pa.ctypes.data
            if A_masks is not None:
                self.bins[b].A_mr_b = self._hold(pack_rows(A_masks[b])).ctypes.data
            z = Z_bins[b]
            if z is not None and np.asarray(z).shape[0] > 0:
                z = np.asarray(z, np.uint8)
                self.bins[b].Z_nrows = z.shape[0]
                self.bins[b].Z_rows = self._hold(pk(z)).ctypes.data
                if Z_masks is not None:
                    self.bins[b].Z_mr_b = self._hold(pack_rows(Z_masks[b])).ctypes.data
        # covariates: per-bin 0/1 arrays (case rows x T_ncols, control rows x T_ncols)
        T_ncols = 1
        if T_bins is not None:
            T_ncols = np.asarray(T_bins[0]).shape[1]
            for b in range(nb):
                self.bins[b].T_rows = self._hold(pack_rows(T_bins[b])).ctypes.data
                self.bins[b].S_rows = self._hold(pack_rows(S_bins[b])).ctypes.data
        self.prob = BccProblem()
        self.lib.lakgb_bcc_problem_init(C.byref(self.prob))
        self.prob.T_ncols = T_ncols
        self.prob.kappa_squared = kappa_squared
        self._qc = qc_strategy.encode()
        self.prob.QC_strategy = self._qc
        self._qr = qr_strategy.encode()
        self.prob.QR_strategy = self._qr
        self.prob.ncols = ncols
        self.prob.row_bytes = (ncols + (16 - ncols % 16) % 16) // 8
        if col_mask is not None:
            self.prob.mc_b = self._hold(pack_rows(col_mask)).ctypes.data
        self.prob.nbins = nb
        self.prob.bins = self.bins
        self.prob.gamma = gamma
        self.prob.B_MLT = B_MLT
        self.prob.gamma_type = gamma_type
        self.prob.test_sparse = test_sparse
        self.prob.Ireq = Ireq
        self.ncols = ncols

    def _hold(self, x):
        self._keep.append(x)
        return x

    def solve(self):
        res = BccResult()
        rc = self.lib.lakgb_bcc_solve(C.byref(self.prob), C.byref(res))
        if rc != 0:
            buf = C.create_string_buffer(512)
            self.lib.lakgb_bcc_last_error(buf, 512)
            raise RuntimeError("lakgb_bcc_solve failed (%d): %s" % (rc, buf.value.decode()))
        try:
            tr = np.ctypeslib.as_array(res.trace, (6 * res.iterations,)).copy() if res.iterations else np.zeros(0)
            xa = np.ctypeslib.as_array(res.xdrop_a, (2 * res.n_xdrop,)).copy() if res.n_xdrop else np.zeros(0, int)
            xb = np.ctypeslib.as_array(res.xdrop_b, (2 * res.n_xdrop,)).copy() if res.n_xdrop else np.zeros(0, int)
        finally:
            self.lib.lakgb_bcc_result_free(C.byref(res))
        return format_outputs(tr, xa, xb)


def format_outputs(tr, xa, xb):
    """The reference's output-file lines from a trace / xdrop array triple."""
    trace = ["%d %d %d %0.16f %0.16f %d" % (int(tr[6 * i]), int(tr[6 * i + 1]), int(tr[6 * i + 2]),
                                             tr[6 * i + 3], tr[6 * i + 4], int(tr[6 * i + 5]))
             for i in range(len(tr) // 6)]
    return {"trace": trace,
            "xdrop_a": ["%d %d" % (xa[2 * i], xa[2 * i + 1]) for i in range(len(xa) // 2)],
            "xdrop_b": ["%d %d" % (xb[2 * i], xb[2 * i + 1]) for i in range(len(xb) // 2)]}


def solve(A_bins, Z_bins=None, **kw):
    return Problem(A_bins, Z_bins, **kw).solve()


def run_in_file(path: str) -> None:
    lib = bind(load())
    rc = lib.lakgb_bcc_run_in_file(path.encode())
    if rc != 0:
        buf = C.create_string_buffer(512)
        lib.lakgb_bcc_last_error(buf, 512)
        raise RuntimeError("lakgb_bcc_run_in_file failed (%d): %s" % (rc, buf.value.decode()))


WORKLOADS = {
    # name: description (see workload())
    "case_only_1024x1024": "cases 1024 x 1024 SNPs, 45 x 45 planted, gamma 0.05 (config 1)",
    "case_control_4096x4096x16384": "cases 4096 + controls 4096 x 16384 SNPs, 2 bins, gamma 0.05 (config 2)",
    "case_control_1024x1024x4096": "cases 1024 + controls 1024 x 4096 SNPs, 2 bins, gamma 0.05 (small config 2)",
    "case_control_32768x32768x131072": "cases 32768 + controls 32768 x 131072 SNPs, 3 bins, gamma 0.02, "
                                        "MAF U[0.01,0.5], 2048 x 4096 planted (config 3; drawn on the GPU)",
}


def large_problem(seed=3, lib=None, chunk_rows=2048, n_case=32768, n_ctrl=32768, ncols=131072, planted=(2048, 4096)):
    """The large single-solve configuration as a Problem of packed rows: the
    rows are drawn on the device in chunks (torch as plumbing: a seeded
    generator, comparisons, an MSB-first pack) and copied to host memory,
    since 4.3 G entries per matrix would not fit a host 0/1 array well."""
    import torch
    nbins, (pr, pc), flip = 3, planted, 0.05
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    p = 0.01 + 0.49 * torch.rand(ncols, generator=g, device="cuda")
    pattern = torch.rand(pc, generator=g, device="cuda") < 0.5
    w = torch.tensor([128, 64, 32, 16, 8, 4, 2, 1], dtype=torch.uint8, device="cuda")
    out = {"A": [[] for _ in range(nbins)], "Z": [[] for _ in range(nbins)]}
    for side, n in (("A", n_case), ("Z", n_ctrl)):
        bins = torch.randint(0, nbins, (n,), generator=g, device="cuda")
        for r0 in range(0, n, chunk_rows):
            r1 = min(n, r0 + chunk_rows)
            bits = torch.rand(r1 - r0, ncols, generator=g, device="cuda") < p
            if side == "A" and r0 < pr:
                k = min(r1, pr) - r0
                bits[:k, :pc] = pattern ^ (torch.rand(k, pc, generator=g, device="cuda") < flip)
            packed = (bits.view(r1 - r0, ncols // 8, 8).to(torch.uint8) * w).sum(dim=2, dtype=torch.uint8)
            b = bins[r0:r1]
            for nb in range(nbins):
                out[side][nb].append(packed[b == nb].cpu().numpy())
            del bits, packed
    A = [np.concatenate(x) for x in out["A"]]
    Z = [np.concatenate(x) for x in out["Z"]]
    return Problem(A, Z, gamma=0.02, lib=lib, packed_ncols=ncols)


def workload(name):
    """Synthetic problems of the benchmark configurations, as solve arguments."""
    from . import synth
    if name == "case_only_1024x1024":
        inst = synth.case_only(1024, 1024, k=45, flip=0.1, seed=1)
        return inst.A_bins, None, 0.05
    if name == "case_control_4096x4096x16384":
        inst = synth.case_control(4096, 4096, 16384, 256, 512, 0.05, nbins=2, seed=2)
        return inst.A_bins, inst.Z_bins, 0.05
    if name == "case_control_1024x1024x4096":
        inst = synth.case_control(1024, 1024, 4096, 64, 128, 0.05, nbins=2, seed=2)
        return inst.A_bins, inst.Z_bins, 0.05
    raise KeyError(name)


def main(argv=None):
    import argparse
    import time
    ap = argparse.ArgumentParser(description="Solve a synthetic bcc workload on the GPU and print its timing.")
    ap.add_argument("--workload", default="case_control_1024x1024x4096", choices=sorted(WORKLOADS))
    ap.add_argument("--reps", type=int, default=1)
    ap.add_argument("--gram-impl", default="auto", choices=["auto", "tensor", "popcount", "split"],
                    help="Gram kernel for every launch (default: autotuned per shape class)")
    args = ap.parse_args(argv)
    import json
    import os
    if args.workload == "case_control_32768x32768x131072":
        p = large_problem()
    else:
        A, Z, gamma = workload(args.workload)
        p = Problem(A, Z, gamma=gamma)
    p.lib.lakgb_set_gram_impl({"popcount": 0, "tensor": 1, "auto": 2, "split": 3}[args.gram_impl])
    profile = os.environ.get("LAKGB_PROFILE_CALLS", "0") not in ("", "0")
    for r in range(args.reps):
        if profile:
            p.lib.lakgb_call_profile_reset()
        t0 = time.perf_counter()
        out = p.solve()
        print("%s rep %d: %.3f s, %d iterations, %d eliminations" %
              (args.workload, r, time.perf_counter() - t0, len(out["trace"]), len(out["xdrop_a"])), flush=True)
        if profile:
            buf = C.create_string_buffer(1 << 16)
            p.lib.lakgb_call_profile(buf, len(buf))
            for name, v in sorted(json.loads(buf.value.decode()).items(), key=lambda kv: -kv[1]["seconds"]):
                print("  %-32s %6d calls %8.3f s (self %.3f s)" % (name, v["calls"], v["seconds"], v["self_seconds"]),
                      flush=True)


if __name__ == "__main__":
    main()
