"""Kernel-level parity harness shared by the fixture generator and the tests.

A *case* is a dict of numpy arrays (the packed inputs and masks) plus scalar
arguments.  ``run_case`` turns it into reference M_handle / L_handle structs and
calls one backend:

  ``ref``    the reference's own wrap_* kernels, compiled from its sources into
             oracle/_ref/liblakref.so (x86-64 container only; used to make the
             committed fixtures)
  ``oracle`` the plain-C restatement oracle/liblakoracle.so (any host)
  ``gpu``    the product library lakcluster_c_gb300/liblakgb300.so

All three receive the same structs and must produce the same FP64 outputs.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from lakcluster_c_gb300 import abi
from lakcluster_c_gb300.abi import LHandle, L_handle, MHandle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REF_LIB = os.path.join(ROOT, "oracle", "_ref", "liblakref.so")
ORACLE_LIB = os.path.join(ROOT, "oracle", "liblakoracle.so")

_libs: dict[str, C.CDLL] = {}


def load_backend(name: str) -> C.CDLL:
    if name in _libs:
        return _libs[name]
    if name == "ref":
        lib = C.CDLL(REF_LIB)
        lib.lakref_init.restype = C.c_int
        assert lib.lakref_init(C.c_longlong(2048), 4, 1) == 0
    elif name == "oracle":
        lib = C.CDLL(ORACLE_LIB)
    elif name == "gpu":
        from lakcluster_c_gb300 import _lib
        lib = _lib.load()
    else:
        raise ValueError(name)
    _libs[name] = lib
    return lib


# ---------------------------------------------------------------------------
# case generation


def random_bits(rng, shape, p=0.5):
    return (rng.random(shape) < p).astype(np.uint8)


def make_matrix_case(rng, nrows, ncols, mr_b_frac=1.0, mr_j_frac=1.0, p=0.5):
    rows = random_bits(rng, (nrows, ncols), p)
    mr_b = (rng.random(nrows) < mr_b_frac).astype(np.uint8)
    mr_j = mr_b & (rng.random(nrows) < mr_j_frac).astype(np.uint8)
    return rows, mr_b, mr_j


def mhandle(rows, mr_b, mr_j, mc_b, mc_j) -> MHandle:
    return MHandle(rows, mr_b=mr_b, mr_j=mr_j, mc_b=mc_b, mc_j=mc_j)


# ---------------------------------------------------------------------------
# backend calls (reference argument lists)


def _thread_args():
    return (C.byref(C.c_int(0)), (C.c_void_p * 128)(), C.byref(C.c_ulong(0)))


def _lf_arg(h: LHandle | None):
    return None if h is None else h.ptr


def call_gram(backend: str, symmetric: bool, type_flag: int, spr: int, spc: int,
              MA: MHandle, MZ: MHandle, A_ajdk: np.ndarray | None,
              lfA: LHandle | None, lfZ: LHandle | None) -> np.ndarray:
    lib = load_backend(backend)
    out = C.POINTER(L_handle)()
    aj = None if A_ajdk is None else A_ajdk.ctypes.data_as(C.POINTER(C.c_double))
    if backend == "oracle":
        fn = lib.lako_AnAt_vv if symmetric else lib.lako_AnZt_vv
        n = fn(type_flag, spr, spc, MA.ptr, MZ.ptr, aj, _lf_arg(lfA), _lf_arg(lfZ), C.byref(out))
    else:
        fn = lib.wrap_AnAt_vv__run if symmetric else lib.wrap_AnZt_vv__run
        n = fn(*_thread_args(), type_flag, spr, spc, MA.ptr, MZ.ptr, aj, _lf_arg(lfA), _lf_arg(lfZ),
               C.byref(out))
    return _take(out, n)


def call_an_v(backend: str, type_flag: int, spr: int, MA: MHandle) -> np.ndarray:
    lib = load_backend(backend)
    out = C.POINTER(L_handle)()
    if backend == "oracle":
        n = lib.lako_An_v(type_flag, spr, MA.ptr, C.byref(out))
    else:
        n = lib.wrap_An_v__run(*_thread_args(), type_flag, spr, MA.ptr, C.byref(out))
    return _take(out, n)


def call_an_ajdk(backend: str, type_flag: int, spr: int, MA: MHandle, A_ajdk: np.ndarray) -> np.ndarray:
    lib = load_backend(backend)
    out = C.POINTER(L_handle)()
    aj = A_ajdk.ctypes.data_as(C.POINTER(C.c_double))
    if backend == "oracle":
        n = lib.lako_An_ajdk_v(type_flag, spr, MA.ptr, aj, C.byref(out))
    else:
        n = lib.wrap_An_ajdk_v(*_thread_args(), type_flag, spr, MA.ptr, aj, C.byref(out))
    return _take(out, n)


def _take(out, n: int) -> np.ndarray:
    if not out:
        return np.zeros(0)
    L = out.contents
    if n <= 0:
        return np.zeros(0)
    arr = np.ctypeslib.as_array(C.cast(L.lf, C.POINTER(C.c_double)), shape=(n,)).copy()
    return arr


def lhandle_from(vec: np.ndarray, row_stride: int, col_stride: int, spacing_row: int) -> LHandle:
    h = LHandle(vec.size)
    h.buf[: vec.size] = vec
    h.s.row_stride, h.s.col_stride = row_stride, col_stride
    h.s.spacing_row, h.s.spacing_col = spacing_row, abi.SPACING_a
    return h


# ---------------------------------------------------------------------------
# the standard kernel case list


def gram_case_specs():
    """(name, nA, nZ, ncols, mask fractions, p, with_ajdk, symmetric) triples
    covering ragged sizes, block boundaries and partial masks."""
    specs = []
    shapes = [(1, 1, 1), (15, 17, 1919), (16, 16, 1920), (17, 33, 1921), (40, 24, 4000),
              (70, 50, 5777)]
    for i, (nA, nZ, m) in enumerate(shapes):
        for masked in (False, True):
            for ajdk in (False, True):
                specs.append(dict(name=f"g{i}_{int(masked)}{int(ajdk)}", nA=nA, nZ=nZ, m=m,
                                  masked=masked, ajdk=ajdk, seed=1000 + 17 * i + 2 * int(masked) + int(ajdk)))
    return specs


def build_gram_inputs(spec):
    rng = np.random.default_rng(spec["seed"])
    nA, nZ, m = spec["nA"], spec["nZ"], spec["m"]
    frac = 0.8 if spec["masked"] else 1.0
    A, ar_b, ar_j = make_matrix_case(rng, nA, m, frac, frac)
    Z, zr_b, zr_j = make_matrix_case(rng, nZ, m, frac, frac)
    mc_b = (rng.random(m) < frac).astype(np.uint8)
    mc_j = mc_b & (rng.random(m) < frac).astype(np.uint8)
    P = abi.psize(m)
    A_p = 0.02 + 0.96 * rng.random(P) if spec["ajdk"] else None
    return dict(A=A, ar_b=ar_b, ar_j=ar_j, Z=Z, zr_b=zr_b, zr_j=zr_j, mc_b=mc_b, mc_j=mc_j, A_p=A_p)


# ---------------------------------------------------------------------------
# the condense row strategy's entry points (M_Ax_to_L2.c, AnZt_mm.c)


def call_m_to_l2(backend: str, at: bool, type_flag: int, spr: int, spc: int, M: MHandle,
                 A_ajdk: np.ndarray | None, out_length: int | None = None) -> tuple[np.ndarray, LHandle | None]:
    """wrap_M_At_to_L2_run (at) / wrap_M_An_to_L2_run; returns the output's
    first rows x columns values and, with ``out_length``, the caller-owned
    handle it was written into (longer than the product: the whole handle is
    zeroed)."""
    lib = load_backend(backend)
    aj = None if A_ajdk is None else A_ajdk.ctypes.data_as(C.POINTER(C.c_double))
    own = LHandle(out_length) if out_length else None
    if own is not None:
        own.buf[:] = 7.0
    out = C.pointer(own.s) if own is not None else C.POINTER(L_handle)()
    if backend == "oracle":
        n = lib.lako_M_to_L2(int(at), type_flag, spr, spc, M.ptr, aj, C.byref(out))
    else:
        fn = lib.wrap_M_At_to_L2_run if at else lib.wrap_M_An_to_L2_run
        n = fn(*_thread_args(), type_flag, spr, spc, M.ptr, aj, C.byref(out))
    if own is not None:
        return own.buf.copy(), own
    return _take(out, n), None


def call_anzt_mm(backend: str, lfA: LHandle, lfZ: LHandle) -> np.ndarray:
    lib = load_backend(backend)
    out = C.POINTER(L_handle)()
    if backend == "oracle":
        n = lib.lako_AnZt_mm(lfA.ptr, lfZ.ptr, C.byref(out))
    else:
        n = lib.wrap_AnZt_mm__run(*_thread_args(), lfA.ptr, lfZ.ptr, C.byref(out))
    return _take(out, n)


def to_l2_specs():
    """(name, nrows (SNPs for At), ncols, masked, type, spacings, ajdk) covering
    ragged sizes, partial masks, both value types and every spacing."""
    out = []
    shapes = [(1, 1), (17, 33), (40, 1921), (129, 300)]
    spac = [(abi.SPACING_j, abi.SPACING_b), (abi.SPACING_a, abi.SPACING_a), (abi.SPACING_b, abi.SPACING_j)]
    for i, (nr, nc) in enumerate(shapes):
        for t, tf in enumerate((abi.TYPE_pm, abi.TYPE_00)):
            for s, (sr, sc) in enumerate(spac):
                out.append(dict(name=f"l{i}{t}{s}", nr=nr, nc=nc, masked=bool((i + s) % 2), type=tf, sr=sr, sc=sc,
                                ajdk=(t + s) % 3 != 2, seed=3000 + 31 * i + 7 * t + s))
    return out


def build_to_l2(spec, at=True):
    """M with SNPs as rows (at) or columns, and the A_ajdk of those SNPs."""
    rng = np.random.default_rng(spec["seed"])
    frac = 0.7 if spec["masked"] else 1.0
    rows, mr_b, mr_j = make_matrix_case(rng, spec["nr"], spec["nc"], frac, frac)
    mc_b = (rng.random(spec["nc"]) < frac).astype(np.uint8)
    mc_j = mc_b & (rng.random(spec["nc"]) < frac).astype(np.uint8)
    M = mhandle(rows, mr_b, mr_j, mc_b, mc_j)
    snps = spec["nr"] if at else spec["nc"]
    A_ajdk = abi.calc_A_ajdk(0.02 + 0.96 * rng.random(abi.psize(snps))) if spec["ajdk"] else None
    return M, A_ajdk


def mm_specs():
    """(K, m, n, extra rows per Zt column) for AnZt_mm: single elements, tile
    edges (16 in k, 64 in i and j), and a Zt with more rows per column than K."""
    return [(1, 1, 1, 0), (16, 64, 64, 0), (17, 65, 63, 0), (5, 130, 200, 3), (300, 97, 129, 0), (0, 4, 5, 0)]


def build_mm(K, m, n, extra, seed):
    rng = np.random.default_rng(seed)
    A = rng.standard_normal((K, m)) * rng.choice([1e-3, 1.0, 1e3], size=(K, m))
    B = rng.standard_normal((K + extra, n))
    lfA = LHandle.from_matrix(A, abi.SPACING_j, abi.SPACING_b)
    lfZ = LHandle.from_matrix(B, abi.SPACING_j, abi.SPACING_a)
    return A, B, lfA, lfZ


def mm_numpy(A, B):
    """The GSL dgemm order: one running sum from +0 over k ascending."""
    K, m = A.shape
    S = np.zeros((m, B.shape[1]))
    for k in range(K):
        S = S + np.multiply.outer(A[k], B[k])
    return S
