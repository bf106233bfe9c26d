"""The chain behind the bit-plane loop product An_ZtSWn_Yt_ww, as the
reference's own check builds it (dir_c/An_ZtSWn_Yt_ww.c:128-399): each
covariate slice of an FP64 ZtSWn array is quantised by wrap_xcalc into bit
planes (one M_handle per St row), and wrap_An_ZtSWn_Yt_ww__run evaluates the
loop product through them; An_ZtSWn_Yt_vv evaluates the same product from the
FP64 array directly.  ``chain(backend, x, h)`` runs the xcalc + ww steps on
one backend ("oracle" or "gpu")."""
from __future__ import annotations

import ctypes as C

import numpy as np

import kernel_cases as kc
import product_cases as pc
from lakcluster_c_gb300 import abi

B_MLT = 32
D_MLT = 1 << 32


def spec(seed=91):
    return dict(name="chain", nsnp=300, npat=500, nctl=400, nt=2, masked=True, seed=seed)


def planes(backend, x, h):
    """One xcalc'd M_handle per St row, from the slices of h["lf_ZtSWn"]."""
    lib = kc.load_backend(backend)
    Zt, Wt, L = h["Zt"], h["Wt"], h["lf_ZtSWn"]
    nY, nW = Zt.nrows, Wt.nrows
    base = L.buf.ctypes.data
    layer = int(L.s.row_stride) * int(L.s.col_stride)
    out = []
    for s in range(int(h["St"].s.rpop_j)):
        s_a = int(h["St"].m_a_[s])
        MX = abi.MHandle(None, nrows=(B_MLT + 1) * nW, ncols=nY,
                         wX=np.zeros(((B_MLT + 1) * nW, abi.bsize(nY)), np.uint8))
        ptr = base + 8 * s_a * layer  # the SPACING_a layer of St row s
        if backend == "oracle":
            lib.lako_set_d_mlt(C.c_longlong(D_MLT))
            lib.lako_xcalc(Zt.mr_j.ctypes.data_as(C.c_void_p), Zt.mr_b.ctypes.data_as(C.c_void_p),
                           Wt.mr_j.ctypes.data_as(C.c_void_p), Wt.mr_b.ctypes.data_as(C.c_void_p),
                           C.byref(L.s), C.c_void_p(ptr), nY, nW, C.byref(MX.s), B_MLT, 0)
        else:
            px = C.pointer(MX.s)
            vpra = (C.c_void_p * 128)()
            lib.wrap_xcalc(C.byref(C.c_int(0)), C.cast(vpra, C.c_void_p), None, Zt.mr_j.ctypes.data,
                           Zt.mr_b.ctypes.data, Wt.mr_j.ctypes.data, Wt.mr_b.ctypes.data, C.byref(L.s),
                           C.c_void_p(ptr), C.byref(C.c_int(nY)), C.byref(C.c_int(nW)), C.byref(px),
                           C.byref(C.c_int(B_MLT)), 0)
        out.append(MX)
    return out


def chain(backend, x, h, sa=abi.SPACING_a, sb=abi.SPACING_a):
    """xcalc every slice, then the ww product, on one backend."""
    ps = planes(backend, x, h)
    hh = dict(h)
    hh["ww_planes"] = ps
    hh["ww_arr"] = (C.POINTER(abi.M_handle) * len(ps))(*[C.pointer(m.s) for m in ps])
    return pc.run(backend, "An_ZtSWn_Yt_ww", hh, sa, sb), ps


def rel_err(a, b):
    """Largest difference relative to the largest magnitude of the reference."""
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))
