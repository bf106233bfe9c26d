"""Per-entry-point timings of the scan, quantisation and loop-sum kernels,
each at a size whose operands are larger than the GPU's L2, called through the
reference's C entry points with the bit matrices resident on the device.

    python -m lakcluster_c_gb300.kernel_bench [--reps 5] [--only NAME ...]

prints one JSON object: per entry point the median wall time of a call (small
uploads and the result download included) and the algorithmic work of one
call (bytes for the HBM-bound scans, bit-ops for the popcount products).
Kernel-only durations come from a launch list of the same command, e.g.
``ncu --metrics gpu__time_duration.sum --clock-control none --csv ...``.

Entry points and sizes (synthetic bits, uniform bytes; FP64 normal):
  An_v        wrap_An_v__run on 131072 rows x 32768 columns (512 MB), dir_c/An_v.c:59
  An_ajdk_v   wrap_An_ajdk_v on 32768 x 131072 (512 MB), dir_c/An_ajdk_v.c:365
  xcalc       wrap_xcalc on an 8192 x 8192 FP64 matrix (512 MB), B_MLT 32, dir_c/xcalc.c:248
  AtTYn_vv    wrap_AtTYn_vv__run, 4096 x 4096 SNP pairs over 16384 rows, dir_c/AtTYn_vv.c:204
  An_ZtSn_ww  wrap_An_ZtSn_ww__run, 32768 rows x 16384 SNPs, 33 planes, dir_c/An_ZtSn_ww.c:110
  AnZt_S_WnYt wrap_AnZt_S_WnYt_vv__run on two 4096 x 4096 FP64 Grams, dir_c/AnZt_S_WnYt_vv.c:103
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import statistics
import time

import numpy as np

from . import abi
from ._lib import load

_DP = C.POINTER(C.c_double)


def _bits(rng, nrows, ncols):
    """An M_handle over uniform random bytes (all rows and columns retained)."""
    mcl = abi.bsize(ncols)
    return abi.MHandle(None, nrows=nrows, ncols=ncols, wX=rng.integers(0, 256, (nrows, mcl), dtype=np.uint8))


def _thread():
    return C.byref(C.c_int(0)), (C.c_void_p * 128)(), None


def _time(fn, reps):
    fn()  # first call: uploads the resident operands
    t = []
    for _ in range(reps):
        t0 = time.perf_counter()
        fn()
        t.append(time.perf_counter() - t0)
    return statistics.median(t)


def _out():
    return C.POINTER(abi.L_handle)()


def bench_an_v(lib, rng, reps):
    M = _bits(rng, 131072, 32768)
    out = _out()  # allocated by the first call, reused (zero-filled) by the others

    def call():
        lib.wrap_An_v__run(*_thread(), abi.TYPE_pm, abi.SPACING_a, M.ptr, C.byref(out))
    s = _time(call, reps)
    nbytes = M.s.rpop_b * M.s.mc_length + 8 * M.nrows
    return {"seconds": s, "bytes": nbytes, "kernel": "an_v_kernel", "bound": "hbm"}


def bench_an_ajdk(lib, rng, reps):
    M = _bits(rng, 32768, 131072)
    aj = abi.calc_A_ajdk(0.05 + 0.9 * rng.random(abi.psize(M.ncols)))
    out = _out()  # allocated by the first call, reused (zero-filled) by the others

    def call():
        lib.wrap_An_ajdk_v(*_thread(), abi.TYPE_pm, abi.SPACING_a, M.ptr, aj.ctypes.data_as(_DP), C.byref(out))
    s = _time(call, reps)
    nbytes = M.s.rpop_b * M.s.mc_length + 8 * 15 * M.nrows
    return {"seconds": s, "bytes": nbytes, "kernel": "an_ajdk_kernel", "bound": "hbm"}


def bench_xcalc(lib, rng, reps):
    n, B = 8192, 32
    lf = np.ascontiguousarray(rng.standard_normal(n * n))
    L = abi.L_handle()
    L.length = lf.size
    L.lf = lf.ctypes.data
    L.spacing_row = L.spacing_col = abi.SPACING_a
    L.row_stride = L.col_stride = n
    ones = abi.pack_bits(np.ones(n, np.uint8), abi.bsize(n))
    MX = abi.MHandle(None, nrows=(B + 1) * n, ncols=n, wX=np.zeros(((B + 1) * n, abi.bsize(n)), np.uint8))
    px = C.pointer(MX.s)
    lib.wrap_xcalc.restype = None

    def call():
        lib.wrap_xcalc(*_thread(), ones.ctypes.data_as(C.c_void_p), ones.ctypes.data_as(C.c_void_p),
                       ones.ctypes.data_as(C.c_void_p), ones.ctypes.data_as(C.c_void_p), C.byref(L),
                       lf.ctypes.data_as(C.c_void_p), C.byref(C.c_int(n)), C.byref(C.c_int(n)), C.byref(px),
                       C.byref(C.c_int(B)), 0)
    s = _time(call, reps)
    return {"seconds": s, "bytes_minmax": 8 * n * n, "bytes_planes": 8 * n * n + (B + 1) * n * abi.bsize(n) // 8,
            "kernel": "xcalc_minmax_kernel, xcalc_planes_kernel", "bound": "hbm",
            "note": "the call uploads the FP64 matrix (512 MB) from host memory each time"}


def bench_attyn(lib, rng, reps):
    nsnp, nrow = 4096, 16384
    At = _bits(rng, nsnp, nrow)
    Tt = abi.MHandle(np.ones((1, nrow), np.uint8))
    aj = abi.calc_A_ajdk(0.05 + 0.9 * rng.random(abi.psize(nsnp)))
    lt = abi.LHandle.from_matrix(np.zeros((nsnp, 1)))
    out = _out()  # allocated by the first call, reused (zero-filled) by the others

    def call():
        lib.wrap_AtTYn_vv__run(*_thread(), abi.SPACING_a, abi.SPACING_a, abi.SPACING_a, At.ptr, Tt.ptr, At.ptr,
                               aj.ctypes.data_as(_DP), aj.ctypes.data_as(_DP), lt.ptr, lt.ptr, C.byref(out))
    s = _time(call, reps)
    return {"seconds": s, "bitops": float(nsnp) * nsnp * At.s.mc_length * 8, "kernel": "attyn_kernel",
            "bound": "integer pipe", "note": "the call downloads the 4096 x 4096 FP64 output (134 MB)"}


def bench_an_ztsn(lib, rng, reps):
    n, m, B = 32768, 16384, 32
    An = _bits(rng, n, m)
    St = abi.MHandle(np.ones((1, 16), np.uint8))
    Z = _bits(rng, B + 1, m)
    Z.s.ncols_per_z, Z.s.min_d, Z.s.mlt_d = B + 1, -3.0, float(2 ** 32) / 9.0
    out = _out()  # allocated by the first call, reused (zero-filled) by the others

    def call():
        lib.wrap_An_ZtSn_ww__run(*_thread(), abi.SPACING_a, abi.SPACING_a, An.ptr, None, Z.ptr, St.ptr,
                                 C.byref(out))
    s = _time(call, reps)
    return {"seconds": s, "bitops": float(n) * (B + 1) * An.s.mc_length * 8, "bytes": An.s.rpop_b * An.s.mc_length,
            "kernel": "the masked-AND Gram of the An rows against the 33 planes (gram kernels), an_ztsn_finish_kernel",
            "bound": "integer or tensor pipe (the Gram)"}


def bench_anzt_s_wnyt(lib, rng, reps):
    nA, nZ = 4096, 4096
    An = abi.MHandle(None, nrows=nA, ncols=16, wX=np.zeros((nA, abi.bsize(16)), np.uint8))
    Zn = abi.MHandle(None, nrows=nZ, ncols=16, wX=np.zeros((nZ, abi.bsize(16)), np.uint8))
    St = abi.MHandle((rng.random((1, nZ)) < 0.5).astype(np.uint8))
    g1 = abi.LHandle.from_matrix(rng.standard_normal((nA, nZ)))
    g2 = abi.LHandle.from_matrix(rng.standard_normal((nA, nZ)))
    out = _out()  # allocated by the first call, reused (zero-filled) by the others

    def call():
        lib.wrap_AnZt_S_WnYt_vv__run(*_thread(), abi.SPACING_a, abi.SPACING_a, An.ptr, St.ptr, Zn.ptr, g1.ptr,
                                     g2.ptr, C.byref(out))
    s = _time(call, reps)
    return {"seconds": s, "bytes": 2 * 8 * nA * nZ, "kernel": "anzt_s_wnyt_kernel",
            "bound": "FP64 add chain (4096 dependent adds per output)",
            "note": "the call uploads the two FP64 Grams (268 MB) each time"}


BENCHES = {"An_v": bench_an_v, "An_ajdk_v": bench_an_ajdk, "xcalc": bench_xcalc, "AtTYn_vv": bench_attyn,
           "An_ZtSn_ww": bench_an_ztsn, "AnZt_S_WnYt": bench_anzt_s_wnyt}


def run(names=None, reps=5, seed=5):
    lib = load()
    rng = np.random.default_rng(seed)
    out = {}
    for name in names or list(BENCHES):
        # residency per entry point: turning it off frees the device copies, so
        # no later host buffer at a reused address meets an old copy
        lib.lakgb_set_residency(1)
        try:
            out[name] = BENCHES[name](lib, rng, reps)
        finally:
            lib.lakgb_set_residency(0)
    out["device_status"] = int(lib.lakgb_device_status())
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--reps", type=int, default=5)
    ap.add_argument("--only", nargs="*", choices=list(BENCHES))
    a = ap.parse_args()
    print(json.dumps(run(a.only, a.reps)))


if __name__ == "__main__":
    main()
