"""Cases for the .b16 transpose (wrap_transpose, dir_c/binary_read.c:174-269):
random 0/1 matrices written as .b16 files (infiles.write_b16: bitj 16), and
the three implementations that turn a file's bytes around:

  ``ref``     the reference's own wrap_transpose (oracle/_ref/liblakref.so)
  ``oracle``  the plain-C restatement on memory (lako_bits_transpose)
  ``gpu``     the product library's wrap_transpose (file to file)
"""
from __future__ import annotations

import ctypes as C
import os
import struct

import numpy as np

import kernel_cases as kc
from lakcluster_c_gb300 import infiles

# (records, bits per record, density): ragged sizes around the 16-bit
# padding, the kernel's 256 x 256 tiles and the byte boundaries
SHAPES = [(1, 1, 0.5), (3, 15, 0.5), (17, 33, 0.7), (16, 16, 1.0), (0, 5, 0.5), (5, 0, 0.5),
          (300, 250, 0.5), (257, 513, 0.3), (1000, 16, 0.5), (16, 1000, 0.5), (600, 2049, 0.02)]


def matrix(i, shape):
    n, m, p = shape
    rng = np.random.default_rng(7100 + i)
    return (rng.random((n, m)) < p).astype(np.uint8)


def write_file(path, x):
    infiles.write_b16(path, x)
    return open(path, "rb").read()


def header(b):
    return struct.unpack("<3i", b[:12])


def oracle_transpose(raw: bytes) -> bytes:
    """The C restatement on the data of a .b16 file's bytes; returns the
    transposed file's bytes (header bitj, n_col, n_row)."""
    bitj, n_row, n_col = header(raw)
    in_rec = (n_row + (bitj - n_row % bitj) % bitj) // 8
    out_rec = (n_col + (bitj - n_col % bitj) % bitj) // 8
    src = np.frombuffer(raw, np.uint8, count=in_rec * n_col, offset=12).copy()
    dst = np.zeros(max(1, out_rec * n_row), np.uint8)
    lib = kc.load_backend("oracle")
    lib.lako_bits_transpose(src.ctypes.data_as(C.c_void_p), C.c_longlong(in_rec), n_col,
                            dst.ctypes.data_as(C.c_void_p), C.c_longlong(out_rec), n_row)
    return struct.pack("<3i", bitj, n_col, n_row) + dst[: out_rec * n_row].tobytes()


def file_transpose(backend, in_path, out_path, n_bytes_per_read=1024):
    lib = kc.load_backend(backend)
    lib.wrap_transpose(in_path.encode(), out_path.encode(), n_bytes_per_read)
    return open(out_path, "rb").read()


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "b16_transpose.npz")
