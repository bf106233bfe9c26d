"""ctypes mirror of the reference's C data model for the bcc path.

``struct M_handle`` (dir_h/M_handle.h:1-27) and ``struct L_handle``
(dir_h/L_handle.h:1-11) are laid out field for field as in the reference so a
pointer built here can be handed either to the reference's own ``wrap_*``
kernels (the oracle library) or to this package's GPU library, which exports the
same symbols.  The helpers below build those structs from numpy arrays and keep
the arrays alive for as long as the struct is referenced.

Bit layout (dir_h/lakcluster_header.h:24-36): bits are MSB-first within a byte,
a set bit means +1 and a clear bit -1, and each packed row is padded to a
multiple of POPLENGTH = 1920 bits (240 bytes) -- ``bsize(n)`` bytes.
"""
from __future__ import annotations

import ctypes as C
import numpy as np

FNAMESIZE = 4096 + 256
BIT8 = 8
BITJ = 16
POPLENGTH = 1920
AJDK_TOT = 15
(AJDK_0_0, AJDK_1_0, AJDK_2_0, AJDK_3_0, AJDK_4_0,
 AJDK_0_1, AJDK_1_1, AJDK_2_1, AJDK_3_1, AJDK_4_1,
 AJDK_0_2, AJDK_1_2, AJDK_2_2, AJDK_3_2, AJDK_4_2) = range(15)
TYPE_p0, TYPE_pm, TYPE_00 = 0, 1, 2
SPACING_b, SPACING_j, SPACING_a = 0, 1, 2


def rup(a: int, b: int) -> int:
    return a + (b - a % b) % b


def bsize(n: int) -> int:
    """Bytes of one packed row of n bits (lakcluster_header.h:262)."""
    return rup(n + (BITJ - n % BITJ) % BITJ, POPLENGTH) // BIT8


def psize(n: int) -> int:
    """Number of 1920-bit blocks in a row of n bits (lakcluster_header.h:263)."""
    return rup(n + (BITJ - n % BITJ) % BITJ, POPLENGTH) // POPLENGTH


class M_handle(C.Structure):
    _fields_ = [
        ("mark", C.c_void_p),
        ("header_length", C.c_int),
        ("A_name", C.c_char * FNAMESIZE),
        ("A_fp", C.c_void_p),
        ("Ara", C.c_void_p),
        ("bitj", C.c_int),
        ("nrows", C.c_int), ("ncols", C.c_int),
        ("nrows_extend", C.c_int), ("ncols_extend", C.c_int),
        ("rpop_b", C.c_longlong), ("rpop_j", C.c_longlong),
        ("cpop_b", C.c_longlong), ("cpop_j", C.c_longlong),
        ("wX", C.c_void_p),
        ("mr_b", C.c_void_p), ("mr_j", C.c_void_p),
        ("mc_b", C.c_void_p), ("mc_j", C.c_void_p),
        ("rsum", C.c_void_p),
        ("m_a_", C.c_void_p), ("m_b_", C.c_void_p),
        ("n_a_", C.c_void_p), ("n_b_", C.c_void_p),
        ("mr_length", C.c_ulong), ("mc_length", C.c_ulong),
        ("cc_length", C.c_ulong),
        ("wt_length", C.c_ulong),
        ("wt", C.c_void_p),
        ("length_total", C.c_ulonglong),
        ("ncols_per_z", C.c_int),
        ("max_d", C.c_double), ("min_d", C.c_double), ("mlt_d", C.c_double),
    ]


class L_handle(C.Structure):
    _fields_ = [
        ("length", C.c_ulonglong),
        ("lf", C.c_void_p),
        ("spacing_row", C.c_int), ("row_stride", C.c_ulonglong),
        ("spacing_col", C.c_int), ("col_stride", C.c_ulonglong),
        ("spacing_lyr", C.c_int), ("lyr_stride", C.c_ulonglong),
    ]


def _ptr(a: np.ndarray | None) -> int | None:
    return None if a is None else a.ctypes.data


# ---------------------------------------------------------------------------
# bit packing helpers


def pack_bits(bits: np.ndarray, nbytes: int) -> np.ndarray:
    """Pack a 0/1 vector MSB-first into ``nbytes`` bytes (zero padded)."""
    bits = np.asarray(bits, dtype=np.uint8).ravel()
    out = np.zeros(nbytes, dtype=np.uint8)
    p = np.packbits(bits, bitorder="big")
    out[: p.size] = p
    return out


def pack_rows(mat: np.ndarray, nbytes: int) -> np.ndarray:
    """Pack each row of a 0/1 matrix MSB-first into ``nbytes`` bytes."""
    mat = np.asarray(mat, dtype=np.uint8)
    r = mat.shape[0]
    out = np.zeros((r, nbytes), dtype=np.uint8)
    if mat.shape[1] > 0 and r > 0:
        p = np.packbits(mat, axis=1, bitorder="big")
        out[:, : p.shape[1]] = p
    return out


def unpack_bits(b: np.ndarray, n: int) -> np.ndarray:
    return np.unpackbits(np.asarray(b, dtype=np.uint8), bitorder="big")[:n]


def mask_index_lists(n: int, m_b: np.ndarray, m_j: np.ndarray):
    """Index lists of M_mxget (M_init.c:244-295): for the k-th row set in both
    masks, its position among all rows (``a``) and among rows set in m_b (``b``)."""
    bb = unpack_bits(m_b, n).astype(bool)
    bj = unpack_bits(m_j, n).astype(bool) & bb
    pos_b = np.cumsum(bb) - 1
    a = np.nonzero(bj)[0].astype(np.uint32)
    b = pos_b[bj].astype(np.uint32)
    return a, b


class MHandle:
    """An ``M_handle`` whose buffers are numpy arrays owned by this object.

    ``rows`` is the full 0/1 matrix (nrows x ncols); only rows set in ``mr_b``
    are stored in ``wX`` (compacted, M_init.c:376-416 with Ara given)."""

    def __init__(self, rows01: np.ndarray, mr_b=None, mr_j=None, mc_b=None, mc_j=None,
                 wX: np.ndarray | None = None, nrows: int | None = None, ncols: int | None = None):
        if rows01 is not None:
            rows01 = np.asarray(rows01, dtype=np.uint8)
            nrows, ncols = rows01.shape
        self.nrows, self.ncols = int(nrows), int(ncols)
        self.mr_length = bsize(self.nrows)
        self.mc_length = bsize(self.ncols)
        ones_r = np.ones(self.nrows, np.uint8)
        ones_c = np.ones(self.ncols, np.uint8)
        self.mr_b = pack_bits(ones_r if mr_b is None else mr_b, self.mr_length)
        self.mr_j = pack_bits(ones_r if mr_j is None else mr_j, self.mr_length) & self.mr_b
        self.mc_b = pack_bits(ones_c if mc_b is None else mc_b, self.mc_length)
        self.mc_j = pack_bits(ones_c if mc_j is None else mc_j, self.mc_length) & self.mc_b
        rb = unpack_bits(self.mr_b, self.nrows).astype(bool)
        if wX is None:
            wX = pack_rows(rows01[rb], self.mc_length)
        self.wX = np.ascontiguousarray(wX, dtype=np.uint8).reshape(-1, self.mc_length)
        self.rsum = np.zeros(max(1, self.nrows), np.float64)
        self.m_a_ = np.zeros(max(1, self.nrows), np.uint32)
        self.m_b_ = np.zeros(max(1, self.nrows), np.uint32)
        self.n_a_ = np.zeros(max(1, self.ncols), np.uint32)
        self.n_b_ = np.zeros(max(1, self.ncols), np.uint32)
        self.wt = np.zeros(POPLENGTH, np.uint8)
        self.s = M_handle()
        s = self.s
        s.header_length = 12
        s.bitj = BITJ
        s.nrows, s.ncols = self.nrows, self.ncols
        s.nrows_extend = (BITJ - self.nrows % BITJ) % BITJ
        s.ncols_extend = (BITJ - self.ncols % BITJ) % BITJ
        s.mr_length, s.mc_length = self.mr_length, self.mc_length
        s.cc_length = (self.ncols + s.ncols_extend) // BIT8
        s.Ara = _ptr(self.wX)
        s.wX = _ptr(self.wX)
        s.mr_b, s.mr_j = _ptr(self.mr_b), _ptr(self.mr_j)
        s.mc_b, s.mc_j = _ptr(self.mc_b), _ptr(self.mc_j)
        s.rsum = _ptr(self.rsum)
        s.m_a_, s.m_b_ = _ptr(self.m_a_), _ptr(self.m_b_)
        s.n_a_, s.n_b_ = _ptr(self.n_a_), _ptr(self.n_b_)
        s.wt = _ptr(self.wt)
        s.mlt_d = 1.0
        self.mxget()

    def mxget(self):
        """Recompute pops and index lists from the masks (M_init.c:268-295)."""
        s = self.s
        a, b = mask_index_lists(self.nrows, self.mr_b, self.mr_j)
        self.m_a_[: a.size] = a
        self.m_b_[: b.size] = b
        s.rpop_b = int(unpack_bits(self.mr_b, self.nrows).sum())
        s.rpop_j = int(a.size)
        a, b = mask_index_lists(self.ncols, self.mc_b, self.mc_j)
        self.n_a_[: a.size] = a
        self.n_b_[: b.size] = b
        s.cpop_b = int(unpack_bits(self.mc_b, self.ncols).sum())
        s.cpop_j = int(a.size)

    def set_masks(self, mr_j=None, mc_j=None):
        """M_mxset (M_init.c:359-374): new current masks, intersected with the base masks."""
        if mr_j is not None:
            self.mr_j[:] = pack_bits(mr_j, self.mr_length) & self.mr_b
        if mc_j is not None:
            self.mc_j[:] = pack_bits(mc_j, self.mc_length) & self.mc_b
        self.mxget()

    @property
    def ptr(self):
        return C.pointer(self.s)

    @property
    def rpop_j(self):
        return int(self.s.rpop_j)

    @property
    def rpop_b(self):
        return int(self.s.rpop_b)


class LHandle:
    """An ``L_handle`` over a numpy float64 buffer owned by this object."""

    def __init__(self, length: int):
        self.buf = np.zeros(max(1, int(length)), np.float64)
        self.s = L_handle()
        self.s.length = int(length)
        self.s.lf = _ptr(self.buf)

    @property
    def ptr(self):
        return C.pointer(self.s)

    def matrix(self) -> np.ndarray:
        """Return lf as a (row_stride x col_stride) matrix, lf[r + c*row_stride]."""
        r, c = int(self.s.row_stride), int(self.s.col_stride)
        return self.buf[: r * c].reshape(c, r).T.copy()

    @classmethod
    def from_matrix(cls, mat: np.ndarray, spacing_row=SPACING_a, spacing_col=SPACING_a):
        mat = np.asarray(mat, dtype=np.float64)
        r, c = mat.shape
        h = cls(r * c)
        h.buf[: r * c] = mat.T.ravel()
        h.s.row_stride, h.s.col_stride = r, c
        h.s.spacing_row, h.s.spacing_col = spacing_row, spacing_col
        return h


def calc_A_ajdk(A_p: np.ndarray) -> np.ndarray:
    """alpha^j * D^k per 1920-column block (An_ajdk_v.c:5-30), with the
    reference's own libm pow() so the values match it bit for bit."""
    libm = C.CDLL("libm.so.6")
    libm.pow.restype = C.c_double
    libm.pow.argtypes = [C.c_double, C.c_double]
    A_p = np.asarray(A_p, dtype=np.float64)
    P = A_p.size
    out = np.zeros(AJDK_TOT * P, np.float64)
    for k in range(3):
        for j in range(5):
            idx = j + 5 * k
            for nc in range(P):
                p = float(A_p[nc])
                a = p - (1 - p)
                d = 1.0 / max(0.01, 4.0 * p * (1 - p))
                out[nc + idx * P] = libm.pow(a, float(j)) * libm.pow(d, float(k))
    return out
