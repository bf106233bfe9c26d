"""The deferral scope (lakgb_defer_begin / lakgb_defer_end): AnZt_S_WnYt
calls made inside it run as one grouped launch when the scope ends, and each
output equals the C oracle's for that call alone (bit for bit) -- calls of
different row, control and covariate counts and spacings, and a nested scope
that runs only when the outer one ends."""
import ctypes as C

import numpy as np
import pytest

import kernel_cases as kc
from lakcluster_c_gb300 import abi
from lakcluster_c_gb300.abi import LHandle, L_handle

pytestmark = pytest.mark.gpu


def _case(seed, nA, nZ, nS):
    rng = np.random.default_rng(seed)
    An = kc.mhandle(*kc.make_matrix_case(rng, nA, 32, 0.85, 0.9), np.ones(32, np.uint8), np.ones(32, np.uint8))
    zr, zb, zj = kc.make_matrix_case(rng, nZ, 32, 0.85, 0.9)
    Zn = kc.mhandle(zr, zb, zj, np.ones(32, np.uint8), np.ones(32, np.uint8))
    St = kc.mhandle(kc.random_bits(rng, (nS, nZ)), np.ones(nS, np.uint8), np.ones(nS, np.uint8),
                    np.ones(nZ, np.uint8), np.ones(nZ, np.uint8))
    L = LHandle.from_matrix(rng.standard_normal((nA, nZ)), abi.SPACING_a, abi.SPACING_a)
    Y = LHandle.from_matrix(rng.standard_normal((nA, nZ)), abi.SPACING_a, abi.SPACING_a)
    return An, Zn, St, L, Y


def _call(backend, sa, ss, c, out):
    An, Zn, St, L, Y = c
    lib = kc.load_backend(backend)
    if backend == "oracle":
        return lib.lako_AnZt_S_WnYt_vv(sa, ss, An.ptr, St.ptr, Zn.ptr, L.ptr, Y.ptr, C.byref(out))
    return lib.wrap_AnZt_S_WnYt_vv__run(*kc._thread_args(), sa, ss, An.ptr, St.ptr, Zn.ptr, L.ptr, Y.ptr,
                                        C.byref(out))


def test_deferred_group_equals_oracle(gpu_lib):
    cases = [(_case(1, 50, 40, 1), abi.SPACING_a, abi.SPACING_a), (_case(2, 333, 129, 2), abi.SPACING_j, abi.SPACING_b),
             (_case(3, 17, 500, 3), abi.SPACING_b, abi.SPACING_j), (_case(4, 1000, 64, 1), abi.SPACING_a, abi.SPACING_j)]
    lib = gpu_lib
    outs = [C.POINTER(L_handle)() for _ in cases]
    lib.lakgb_defer_begin()
    ns = [_call("gpu", sa, ss, c, o) for (c, sa, ss), o in zip(cases, outs)]
    lib.lakgb_defer_begin()  # nested: runs with the outer scope
    lib.lakgb_defer_end()
    lib.lakgb_defer_end()
    for (c, sa, ss), o, n in zip(cases, outs, ns):
        ref = C.POINTER(L_handle)()
        m = _call("oracle", sa, ss, c, ref)
        assert m == n
        assert kc._take(o, n).tobytes() == kc._take(ref, m).tobytes()


def _l3(rng, shape):
    """A 3-D L_handle (rows x columns x layers, a-spacing), lf[r + c*R + l*R*C]."""
    z = rng.standard_normal(shape)
    h = LHandle(z.size)
    h.buf[: z.size] = z.transpose(2, 1, 0).ravel()
    h.s.row_stride, h.s.col_stride, h.s.lyr_stride = shape
    h.s.spacing_row = h.s.spacing_col = h.s.spacing_lyr = abi.SPACING_a
    return h


def test_deferred_wtszn_group_equals_oracle(gpu_lib):
    """AtTYn____WtSZn calls (the QC update's b2 products) deferred together
    with an AnZt_S_WnYt call: every output equals the oracle's."""
    rng = np.random.default_rng(11)
    nsnp, npat, nctl, nt = 300, 64, 48, 2
    At = kc.mhandle(*kc.make_matrix_case(rng, nsnp, npat, 0.9, 0.9), np.ones(npat, np.uint8), np.ones(npat, np.uint8))
    Zt = kc.mhandle(*kc.make_matrix_case(rng, nsnp, nctl, 0.9, 0.9), np.ones(nctl, np.uint8), np.ones(nctl, np.uint8))
    Yt = kc.mhandle(*kc.make_matrix_case(rng, 40, npat, 0.9, 0.9), np.ones(npat, np.uint8), np.ones(npat, np.uint8))
    St = kc.mhandle(kc.random_bits(rng, (nt, nctl)), np.ones(nt, np.uint8), np.ones(nt, np.uint8),
                    np.ones(nctl, np.uint8), np.ones(nctl, np.uint8))
    Tt = kc.mhandle(kc.random_bits(rng, (nt, npat)), np.ones(nt, np.uint8), np.ones(nt, np.uint8),
                    np.ones(npat, np.uint8), np.ones(npat, np.uint8))
    Y_ajdk = abi.calc_A_ajdk(0.05 + 0.9 * rng.random(abi.psize(40)))
    LA, LZ = _l3(rng, (nsnp, 40, nt)), _l3(rng, (nsnp, 40, nt))

    def call(backend, out, M_Wt):
        args = (abi.SPACING_a, abi.SPACING_j, At.ptr, Tt.ptr, Yt.ptr, M_Wt.ptr, St.ptr, Zt.ptr,
                Y_ajdk.ctypes.data_as(C.POINTER(C.c_double)), LA.ptr, LZ.ptr, C.byref(out))
        blib = kc.load_backend(backend)
        if backend == "oracle":
            return blib.lako_AtTYn____WtSZn_vv(*args)
        return blib.wrap_AtTYn____WtSZn_vv__run(*kc._thread_args(), *args)

    Wt = kc.mhandle(*kc.make_matrix_case(rng, 40, nctl, 1.0, 0.8), np.ones(nctl, np.uint8), np.ones(nctl, np.uint8))
    c0 = _case(9, 120, 70, 2)
    outs = [C.POINTER(L_handle)() for _ in range(3)]
    lib = gpu_lib
    lib.lakgb_defer_begin()
    n0 = call("gpu", outs[0], Yt)
    nS = _call("gpu", abi.SPACING_a, abi.SPACING_a, c0, outs[1])
    n1 = call("gpu", outs[2], Wt)
    lib.lakgb_defer_end()
    refs = [C.POINTER(L_handle)() for _ in range(3)]
    m0 = call("oracle", refs[0], Yt)
    mS = _call("oracle", abi.SPACING_a, abi.SPACING_a, c0, refs[1])
    m1 = call("oracle", refs[2], Wt)
    assert (n0, nS, n1) == (m0, mS, m1)
    for o, r, n in zip(outs, refs, [n0, nS, n1]):
        assert kc._take(o, n).tobytes() == kc._take(r, n).tobytes()


def test_deferred_copies_of_other_entry_points(gpu_lib):
    """Inside a scope any entry point's host output is written when the scope
    ends (An_ajdk_v and the Gram here): the values equal the oracle's, and
    before the scope ends the host output still holds its zero fill."""
    rng = np.random.default_rng(21)
    spec = kc.gram_case_specs()[9]
    x = kc.build_gram_inputs(spec)
    MA = kc.mhandle(x["A"], x["ar_b"], x["ar_j"], x["mc_b"], x["mc_j"])
    MZ = kc.mhandle(x["Z"], x["zr_b"], x["zr_j"], x["mc_b"], x["mc_j"])
    A_ajdk = abi.calc_A_ajdk(0.02 + 0.96 * rng.random(abi.psize(spec["m"])))
    aj = A_ajdk.ctypes.data_as(C.POINTER(C.c_double))
    lib = gpu_lib
    o1, o2 = C.POINTER(L_handle)(), C.POINTER(L_handle)()
    lib.lakgb_defer_begin()
    n1 = lib.wrap_An_ajdk_v(*kc._thread_args(), abi.TYPE_pm, abi.SPACING_a, MA.ptr, aj, C.byref(o1))
    n2 = lib.wrap_AnZt_vv__run(*kc._thread_args(), abi.TYPE_pm, abi.SPACING_b, abi.SPACING_b, MA.ptr, MZ.ptr, aj,
                               None, None, C.byref(o2))
    assert not np.any(kc._take(o1, n1)) and not np.any(kc._take(o2, n2))
    lib.lakgb_defer_end()
    w1 = kc.call_an_ajdk("oracle", abi.TYPE_pm, abi.SPACING_a, MA, A_ajdk)
    w2 = kc.call_gram("oracle", False, abi.TYPE_pm, abi.SPACING_b, abi.SPACING_b, MA, MZ, A_ajdk, None, None)
    assert kc._take(o1, n1).tobytes() == w1.tobytes()
    assert kc._take(o2, n2).tobytes() == w2.tobytes()


def test_deferred_xcalc(gpu_lib):
    """wrap_xcalc inside a scope (device-only planes, residency on, as in a
    solve): M_X's min, max and mlt are set when the scope ends and equal the
    oracle's, and the planes it left on the device give the same An_ZtSn_ww
    product as a call made outside a scope."""
    from test_xcalc_gpu import _run
    from test_zz_no_alloc import _bind, _case
    _bind(gpu_lib)
    lib = gpu_lib
    rng = np.random.default_rng(31)
    Yn, Wn, B = 300, 4, 32
    d = _case(rng, Yn, Wn, 0)
    want = _run("oracle", d, Yn, Wn, 0)
    rows, mr_b, mr_j = kc.make_matrix_case(rng, 50, Yn, 0.9, 0.9)
    An = kc.mhandle(rows, mr_b, mr_j, np.ones(Yn, np.uint8), np.ones(Yn, np.uint8))
    ylen = abi.bsize(Yn)
    lib.lakgb_set_residency(1)
    lib.lakgb_device_only_planes(1)
    try:
        outs, scal = [], []
        for deferred in (False, True):
            MX = abi.MHandle(None, nrows=(B + 1) * Wn, ncols=Yn, wX=np.zeros(((B + 1) * Wn, ylen), np.uint8))
            px = C.pointer(MX.s)
            vpra = (C.c_void_p * 128)()
            mr_jp, mr_bp = abi.pack_bits(d["mr_j"], ylen), abi.pack_bits(d["mr_b"], ylen)
            wlen = abi.bsize(Wn)
            mc_jp, mc_bp = abi.pack_bits(d["mc_j"], wlen), abi.pack_bits(d["mc_b"], wlen)
            if deferred:
                lib.lakgb_defer_begin()
            lib.wrap_xcalc(C.byref(C.c_int(0)), C.cast(vpra, C.c_void_p), None, mr_jp.ctypes.data, mr_bp.ctypes.data,
                           mc_jp.ctypes.data, mc_bp.ctypes.data, C.byref(d["L"]), d["lf"].ctypes.data,
                           C.byref(C.c_int(Yn)), C.byref(C.c_int(Wn)), C.byref(px), C.byref(C.c_int(B)), 0)
            if deferred:
                lib.lakgb_defer_end()
            scal.append((MX.s.min_d, MX.s.max_d, MX.s.mlt_d, MX.s.nrows, MX.s.ncols))
            # one covariate row per retained W column (the planes' groups)
            St = abi.MHandle(np.ones((MX.s.nrows // (B + 1), 16), np.uint8))
            out = C.POINTER(L_handle)()
            n = lib.wrap_An_ZtSn_ww__run(*kc._thread_args(), abi.SPACING_a, abi.SPACING_a, An.ptr, None, px, St.ptr,
                                         C.byref(out))
            outs.append(kc._take(out, n))
        assert scal[0] == scal[1] == want[1]
        assert outs[0].size > 0 and np.any(outs[0]) and outs[0].tobytes() == outs[1].tobytes()
        buf = C.create_string_buffer(256)
        assert lib.lakgb_last_error(buf, 256) == 0, buf.value
    finally:
        lib.lakgb_device_only_planes(0)
        lib.lakgb_set_residency(0)
