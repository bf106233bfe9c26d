"""Loader for the product library liblakgb300.so (built in-tree by build.py).

There is no CPU fallback: if the library is missing or cannot be loaded the
import fails with an error naming the build step."""
from __future__ import annotations

import ctypes as C
import os

from .abi import L_handle, M_handle

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liblakgb300.so")

_lib: C.CDLL | None = None


def load() -> C.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is missing: build it first (python -c 'import __graft_entry__ as g; g.build()')")
    lib = C.CDLL(LIB_PATH)
    MP, LP, LPP = C.POINTER(M_handle), C.POINTER(L_handle), C.POINTER(C.POINTER(L_handle))
    thr = [C.POINTER(C.c_int), C.c_void_p, C.c_void_p]
    dp = C.POINTER(C.c_double)
    for name in ("wrap_AnZt_vv__run", "wrap_AnAt_vv__run"):
        f = getattr(lib, name)
        f.restype = C.c_int
        f.argtypes = thr + [C.c_int, C.c_int, C.c_int, MP, MP, dp, LP, LP, LPP]
    lib.wrap_An_v__run.restype = C.c_int
    lib.wrap_An_v__run.argtypes = thr + [C.c_int, C.c_int, MP, LPP]
    lib.wrap_An_ajdk_v.restype = C.c_int
    lib.wrap_An_ajdk_v.argtypes = thr + [C.c_int, C.c_int, MP, dp, LPP]
    lib.lakgb_last_error.restype = C.c_int
    lib.lakgb_last_error.argtypes = [C.c_char_p, C.c_int]
    lib.lakgb_set_residency.argtypes = [C.c_int]
    lib.lakgb_forget_host_buffer.argtypes = [C.c_void_p]
    lib.lakgb_kernel_launches.restype = C.c_ulonglong
    lib.lakgb_last_gram_ms.restype = C.c_double
    lib.lakgb_measure_fp64_add_rate.restype = C.c_double
    lib.lakgb_set_gram_impl.argtypes = [C.c_int]
    lib.lakgb_gram_impl.restype = C.c_int
    lib.lakgb_device_status.restype = C.c_int
    lib.lakgb_call_profile.argtypes = [C.c_char_p, C.c_int]
    lib.lakgb_call_profile.restype = C.c_int
    lib.lakgb_gram_autotune_table.argtypes = [C.c_char_p, C.c_int]
    lib.lakgb_gram_autotune_table.restype = C.c_int
    lib.lakgb_set_bitplane_impl.argtypes = [C.c_int]
    lib.lakgb_bitplane_impl.restype = C.c_int
    lib.lakgb_gram_group_create.argtypes = [C.c_void_p, C.c_int]
    lib.lakgb_gram_group_create.restype = C.c_void_p
    lib.lakgb_gram_group_run.argtypes = [C.c_void_p, C.c_void_p]
    lib.lakgb_gram_group_run.restype = C.c_int
    lib.lakgb_gram_group_destroy.argtypes = [C.c_void_p]
    lib.lakgb_gram_group_destroy.restype = None
    lib.wrap_transpose.argtypes = [C.c_char_p, C.c_char_p, C.c_int]
    lib.wrap_transpose.restype = None
    lib.lakgb_bits_transpose_device.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]
    lib.lakgb_bits_transpose_device.restype = C.c_int
    _lib = lib
    return lib


def last_error() -> tuple[int, str]:
    buf = C.create_string_buffer(512)
    code = load().lakgb_last_error(buf, 512)
    return code, buf.value.decode(errors="replace")
