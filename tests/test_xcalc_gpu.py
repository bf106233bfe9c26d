"""GPU parity of wrap_xcalc (dir_c/xcalc.c:248) against the C oracle's
restatement (lako_xcalc), including a tall matrix whose per-row offset arrays
are 1 MB or more (uploaded into their own device buffers rather than the
staging arena, which must outlive the kernels that read them)."""
import ctypes as C

import numpy as np
import pytest

import kernel_cases as kc
from lakcluster_c_gb300 import abi
from test_zz_no_alloc import _case

pytestmark = pytest.mark.gpu


def _run(backend, d, Yn, Wn, trm, B=32):
    ylen, wlen = abi.bsize(Yn), abi.bsize(Wn)
    mr_j, mr_b = abi.pack_bits(d["mr_j"], ylen), abi.pack_bits(d["mr_b"], ylen)
    mc_j, mc_b = abi.pack_bits(d["mc_j"], wlen), abi.pack_bits(d["mc_b"], wlen)
    MX = abi.MHandle(None, nrows=(B + 1) * Wn, ncols=Yn, wX=np.zeros(((B + 1) * Wn, ylen), np.uint8))
    lib = kc.load_backend(backend)
    if backend == "oracle":
        lib.lako_set_d_mlt(C.c_longlong(1 << 32))
        lib.lako_xcalc(mr_j.ctypes.data_as(C.c_void_p), mr_b.ctypes.data_as(C.c_void_p),
                       mc_j.ctypes.data_as(C.c_void_p), mc_b.ctypes.data_as(C.c_void_p), C.byref(d["L"]),
                       d["lf"].ctypes.data_as(C.c_void_p), Yn, Wn, C.byref(MX.s), B, trm)
    else:
        px = C.pointer(MX.s)
        vpra = (C.c_void_p * 128)()
        lib.wrap_xcalc(C.byref(C.c_int(0)), C.cast(vpra, C.c_void_p), None, mr_j.ctypes.data, mr_b.ctypes.data,
                       mc_j.ctypes.data, mc_b.ctypes.data, C.byref(d["L"]), d["lf"].ctypes.data,
                       C.byref(C.c_int(Yn)), C.byref(C.c_int(Wn)), C.byref(px), C.byref(C.c_int(B)), trm)
    n = MX.s.nrows * MX.s.mc_length
    return MX.wX.reshape(-1)[:n].copy(), (MX.s.min_d, MX.s.max_d, MX.s.mlt_d, MX.s.nrows, MX.s.ncols)


@pytest.mark.parametrize("Yn,Wn,trm", [(700, 90, 0), (333, 410, 1), (140000, 6, 0)])
def test_wrap_xcalc_matches_oracle(gpu_lib, Yn, Wn, trm):
    from test_zz_no_alloc import _bind
    _bind(gpu_lib)
    rng = np.random.default_rng(Yn * 3 + Wn + trm)
    d = _case(rng, Yn, Wn, trm)
    want = _run("oracle", d, Yn, Wn, trm)
    got = _run("gpu", d, Yn, Wn, trm)
    assert got[1] == want[1]
    assert np.array_equal(got[0], want[0])
    buf = C.create_string_buffer(256)
    assert gpu_lib.lakgb_last_error(buf, 256) == 0, buf.value
