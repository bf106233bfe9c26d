"""The allocation-free quantisation entry point, lakgb_xcalc_noalloc.

It must produce exactly what wrap_xcalc produces (the planes and min / max /
mlt it stores in M_X) on the same matrix, on two calls in a row (its static
scratch array is reused), and reject a problem larger than its scratch.
The file name makes pytest collect it last; it also runs alone.
"""
import ctypes as C

import numpy as np
import pytest

from lakcluster_c_gb300 import abi

pytestmark = pytest.mark.gpu

MAXC = 32768


class NoAllocArgs(C.Structure):
    _fields_ = [("lf", C.c_void_p), ("row_off_a", C.c_void_p), ("nrows_a", C.c_int),
                ("rows_j", C.c_void_p), ("n_rows_j", C.c_int), ("cols_j", C.c_void_p), ("n_cols_j", C.c_int),
                ("row0", C.c_void_p), ("b_mlt", C.c_int), ("d_mlt", C.c_longlong), ("brows", C.c_longlong),
                ("planes", C.c_void_p), ("min_max_mlt", C.POINTER(C.c_double)), ("stream", C.c_void_p)]


def _bind(lib):
    lib.lakgb_xcalc_noalloc.argtypes = [C.POINTER(NoAllocArgs)]
    lib.lakgb_xcalc_noalloc.restype = C.c_int
    lib.wrap_xcalc.argtypes = [C.POINTER(C.c_int), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                               C.c_void_p, C.POINTER(abi.L_handle), C.c_void_p, C.POINTER(C.c_int),
                               C.POINTER(C.c_int), C.POINTER(C.POINTER(abi.M_handle)), C.POINTER(C.c_int), C.c_int]
    lib.wrap_xcalc.restype = None
    lib.lakgb_last_error.argtypes = [C.c_char_p, C.c_int]
    return lib


def _case(rng, Yn, Wn, trm):
    mr_b = rng.random(Yn) < 0.9
    mr_j = mr_b & (rng.random(Yn) < 0.85)
    mc_b = rng.random(Wn) < 0.9
    mc_j = mc_b & (rng.random(Wn) < 0.8)
    rb, cb = int(mr_b.sum()), int(mc_b.sum())
    shape = (cb, rb) if trm else (rb, cb)          # L rows x cols, spacing b on both
    lf = np.ascontiguousarray(rng.standard_normal(shape[0] * shape[1]) * 50.0)
    L = abi.L_handle()
    L.length = lf.size
    L.lf = lf.ctypes.data
    L.spacing_row = L.spacing_col = abi.SPACING_b
    L.row_stride, L.col_stride = shape
    rs = shape[0]
    row_off_a = np.full(Yn, -1, np.int64)
    rows_j, cols_j = [], []
    j = b = 0
    for a in range(Yn):
        if not mr_b[a]:
            continue
        if mr_j[a]:
            off = b * rs if trm else b
            row_off_a[a] = off
            rows_j.append(off)
            j += 1
        b += 1
    j = b = 0
    for a in range(Wn):
        if not mc_b[a]:
            continue
        if mc_j[a]:
            cols_j.append(b if trm else b * rs)
            j += 1
        b += 1
    return dict(mr_b=mr_b, mr_j=mr_j, mc_b=mc_b, mc_j=mc_j, lf=lf, L=L, row_off_a=row_off_a,
                rows_j=np.array(rows_j, np.int64), cols_j=np.array(cols_j, np.int64))


@pytest.mark.parametrize("Yn,Wn,trm", [(300, 77, 0), (1000, 513, 1), (2050, 33, 0)])
def test_noalloc_matches_wrap_xcalc(gpu_lib, Yn, Wn, trm):
    import torch
    lib = _bind(gpu_lib)
    rng = np.random.default_rng(Yn + Wn + trm)
    B = 32
    d = _case(rng, Yn, Wn, trm)
    ylen, wlen = abi.bsize(Yn), abi.bsize(Wn)
    mr_j, mr_b = abi.pack_bits(d["mr_j"], ylen), abi.pack_bits(d["mr_b"], ylen)
    mc_j, mc_b = abi.pack_bits(d["mc_j"], wlen), abi.pack_bits(d["mc_b"], wlen)
    # wrap_xcalc into a pre-allocated M_X
    MX = abi.MHandle(None, nrows=(B + 1) * Wn, ncols=Yn,
                     wX=np.zeros(((B + 1) * Wn, ylen), np.uint8))
    px = C.pointer(MX.s)
    tid, yn, wn, bm = C.c_int(0), C.c_int(Yn), C.c_int(Wn), C.c_int(B)
    vpra = (C.c_void_p * 128)()
    lib.wrap_xcalc(C.byref(tid), C.cast(vpra, C.c_void_p), None, mr_j.ctypes.data, mr_b.ctypes.data,
                   mc_j.ctypes.data, mc_b.ctypes.data, C.byref(d["L"]), d["lf"].ctypes.data, C.byref(yn),
                   C.byref(wn), C.byref(px), C.byref(bm), trm)
    nplanes = MX.s.nrows
    brows = MX.s.mc_length
    want = MX.wX.reshape(-1)[: nplanes * brows].copy()
    want_scalars = (MX.s.min_d, MX.s.max_d, MX.s.mlt_d)
    assert nplanes == (B + 1) * len(d["cols_j"])

    dev = torch.device("cuda")
    t_lf = torch.from_numpy(d["lf"]).to(dev)
    t_roa = torch.from_numpy(d["row_off_a"]).to(dev)
    t_rows = torch.from_numpy(d["rows_j"]).to(dev)
    t_cols = torch.from_numpy(d["cols_j"]).to(dev)
    t_row0 = torch.from_numpy(MX.wX.reshape(-1)[:brows].copy()).to(dev)
    t_planes = torch.full((max(1, nplanes * brows),), 0xAB, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    out = (C.c_double * 3)()
    a = NoAllocArgs(t_lf.data_ptr(), t_roa.data_ptr(), Yn, t_rows.data_ptr(), len(d["rows_j"]),
                    t_cols.data_ptr(), len(d["cols_j"]), t_row0.data_ptr(), B, 1 << B, brows,
                    t_planes.data_ptr(), C.cast(out, C.POINTER(C.c_double)),
                    C.c_void_p(torch.cuda.current_stream().cuda_stream))
    for call in range(2):
        t_planes.fill_(0xAB if call == 0 else 0x5C)
        torch.cuda.synchronize()
        rc = lib.lakgb_xcalc_noalloc(C.byref(a))
        assert rc == 0
        got = t_planes.cpu().numpy()[: nplanes * brows]
        assert np.array_equal(got, want), "planes differ on call %d" % call
        assert tuple(out) == want_scalars, "min / max / mlt differ on call %d" % call


@pytest.mark.parametrize("which", ["no_rows", "no_cols"])
def test_noalloc_matches_wrap_xcalc_with_nothing_retained(gpu_lib, which):
    """No retained rows (or columns): min / max / mlt come from the empty-set
    fallback, and the planes hold plane 0 only (or nothing)."""
    import torch
    lib = _bind(gpu_lib)
    rng = np.random.default_rng(11)
    Yn, Wn, B = 200, 40, 32
    d = _case(rng, Yn, Wn, 0)
    if which == "no_rows":
        d["mr_j"][:] = False
        d["row_off_a"][:] = -1
        d["rows_j"] = np.zeros(0, np.int64)
    else:
        d["mc_j"][:] = False
        d["cols_j"] = np.zeros(0, np.int64)
    ylen, wlen = abi.bsize(Yn), abi.bsize(Wn)
    mr_j, mr_b = abi.pack_bits(d["mr_j"], ylen), abi.pack_bits(d["mr_b"], ylen)
    mc_j, mc_b = abi.pack_bits(d["mc_j"], wlen), abi.pack_bits(d["mc_b"], wlen)
    MX = abi.MHandle(None, nrows=(B + 1) * Wn, ncols=Yn, wX=np.zeros(((B + 1) * Wn, ylen), np.uint8))
    px = C.pointer(MX.s)
    tid, yn, wn, bm = C.c_int(0), C.c_int(Yn), C.c_int(Wn), C.c_int(B)
    vpra = (C.c_void_p * 128)()
    lib.wrap_xcalc(C.byref(tid), C.cast(vpra, C.c_void_p), None, mr_j.ctypes.data, mr_b.ctypes.data,
                   mc_j.ctypes.data, mc_b.ctypes.data, C.byref(d["L"]), d["lf"].ctypes.data, C.byref(yn),
                   C.byref(wn), C.byref(px), C.byref(bm), 0)
    nplanes, brows = MX.s.nrows, MX.s.mc_length
    want = MX.wX.reshape(-1)[: nplanes * brows].copy()
    want_scalars = (MX.s.min_d, MX.s.max_d, MX.s.mlt_d)
    dev = torch.device("cuda")
    keep = [torch.from_numpy(x).to(dev) if x.size else torch.zeros(1, dtype=torch.int64, device=dev)
            for x in (d["lf"], d["row_off_a"], d["rows_j"], d["cols_j"])]
    t_row0 = torch.from_numpy(MX.wX.reshape(-1)[:brows].copy()).to(dev)
    t_planes = torch.full((max(16, nplanes * brows),), 0x77, dtype=torch.uint8, device=dev)
    torch.cuda.synchronize()
    out = (C.c_double * 3)()
    a = NoAllocArgs(keep[0].data_ptr(), keep[1].data_ptr(), Yn, keep[2].data_ptr(), len(d["rows_j"]),
                    keep[3].data_ptr(), len(d["cols_j"]), t_row0.data_ptr(), B, 1 << B, brows, t_planes.data_ptr(),
                    C.cast(out, C.POINTER(C.c_double)), C.c_void_p(torch.cuda.current_stream().cuda_stream))
    for call in range(2):
        assert lib.lakgb_xcalc_noalloc(C.byref(a)) == 0
        got = t_planes.cpu().numpy()[: nplanes * brows]
        assert np.array_equal(got, want), "planes differ on call %d" % call
        assert tuple(out) == want_scalars, "min / max / mlt differ on call %d: %s vs %s" % (
            call, tuple(out), want_scalars)


def test_noalloc_rejects_oversize(gpu_lib):
    import torch
    lib = _bind(gpu_lib)
    dummy = torch.zeros(16, dtype=torch.float64, device="cuda")
    out = (C.c_double * 3)()
    p = dummy.data_ptr()
    a = NoAllocArgs(p, p, 16, p, 1, p, MAXC + 1, p, 32, 1 << 32, 240, p, C.cast(out, C.POINTER(C.c_double)), None)
    lib.lakgb_last_error(None, 0)   # the library-wide status keeps the first error until read
    assert lib.lakgb_xcalc_noalloc(C.byref(a)) != 0
    buf = C.create_string_buffer(256)
    lib.lakgb_last_error(buf, 256)
    assert b"exceed the scratch limit" in buf.value
