"""Argument checks of lakgb_xcalc_noalloc, which run before any CUDA call.

The plane kernel stores whole 4-byte words, so a plane row length that is not
a multiple of 4, or a planes pointer that is not 4-byte aligned, must be
rejected; so must negative counts and d_mlt below 2.  None of these calls
reaches the GPU, so they run on a machine without one.
"""
import ctypes as C

from test_zz_no_alloc import NoAllocArgs


def _lib():
    from lakcluster_c_gb300 import build
    lib = C.CDLL(build.build_lib())
    lib.lakgb_xcalc_noalloc.argtypes = [C.POINTER(NoAllocArgs)]
    lib.lakgb_xcalc_noalloc.restype = C.c_int
    lib.lakgb_last_error.argtypes = [C.c_char_p, C.c_int]
    lib.lakgb_last_error.restype = C.c_int
    return lib


def _call(lib, **kw):
    out = (C.c_double * 3)()
    fake = 0x10000           # never dereferenced: every call below is rejected first
    a = dict(lf=fake, row_off_a=fake, nrows_a=100, rows_j=fake, n_rows_j=90, cols_j=fake, n_cols_j=10, row0=None,
             b_mlt=32, d_mlt=1 << 32, brows=240, planes=fake, min_max_mlt=C.cast(out, C.POINTER(C.c_double)),
             stream=None)
    a.update(kw)
    lib.lakgb_last_error(None, 0)
    rc = lib.lakgb_xcalc_noalloc(C.byref(NoAllocArgs(**a)))
    buf = C.create_string_buffer(256)
    code = lib.lakgb_last_error(buf, 256)
    return rc, code, buf.value.decode()


def test_rejects_plane_rows_not_multiple_of_4():
    rc, code, msg = _call(_lib(), brows=13 * 4 + 2)
    assert rc != 0 and code != 0 and "multiple of 4" in msg


def test_rejects_short_plane_rows():
    rc, code, msg = _call(_lib(), nrows_a=1000, brows=64)    # 1000 rows need 128 bytes
    assert rc != 0 and "too short" in msg


def test_rejects_misaligned_planes():
    rc, code, msg = _call(_lib(), planes=0x10002)
    assert rc != 0 and "aligned" in msg


def test_rejects_negative_counts_with_their_own_message():
    for kw in (dict(n_cols_j=-1), dict(n_rows_j=-5), dict(nrows_a=-3)):
        rc, code, msg = _call(_lib(), **kw)
        assert rc != 0 and "negative count" in msg, (kw, msg)


def test_rejects_small_d_mlt_and_bad_b_mlt():
    for kw in (dict(d_mlt=1), dict(d_mlt=0), dict(d_mlt=-7), dict(b_mlt=0), dict(b_mlt=63)):
        rc, code, msg = _call(_lib(), **kw)
        assert rc != 0 and "d_mlt" in msg, (kw, msg)


def test_rejects_oversize_before_launch():
    rc, code, msg = _call(_lib(), n_cols_j=32769)
    assert rc != 0 and "exceed the scratch limit" in msg
