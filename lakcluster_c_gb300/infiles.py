"""Writers for the reference's bcc input files.

``.b16`` bit-matrix files (read by binary_read, dir_c/binary_read.c:5-37):
three native ints (bitj = 16, nbits, nchunks) followed by ``nchunks`` chunks of
``rup(nbits, 16) / 8`` bytes, each holding ``nbits`` bits MSB-first.  A case
matrix A (patients x SNPs) is stored twice: ``A_t`` with one chunk per patient
(header nbits = SNPs) and ``A_n`` with one chunk per SNP.  Row and column
masks are single-chunk files.

``.in`` parameter files (read_input / updateglobals, dir_c/updateglobals.c):
``NAME= value;`` statements, per-bin lists comma separated, ending in
``END= 0;`` -- the same statements the reference's MATLAB driver writes
(dir_m/lakcluster_test_AAAA_ver5.m:95-116).
"""
from __future__ import annotations

import os

import numpy as np

BITJ = 16


def write_b16(path: str, chunks: np.ndarray) -> None:
    """Write a (nchunks, nbits) 0/1 array as a .b16 file."""
    chunks = np.asarray(chunks, dtype=np.uint8)
    if chunks.ndim != 2:
        raise ValueError("chunks must be 2-D")
    nchunks, nbits = chunks.shape
    padded = (nbits + (BITJ - nbits % BITJ) % BITJ)
    buf = np.zeros((nchunks, padded), np.uint8)
    buf[:, :nbits] = chunks
    packed = np.packbits(buf, axis=1, bitorder="big")
    with open(path, "wb") as f:
        f.write(np.array([BITJ, nbits, nchunks], dtype=np.int32).tobytes())
        f.write(packed.tobytes())


def read_b16(path: str) -> np.ndarray:
    """Read a .b16 file back into a (nchunks, nbits) 0/1 array."""
    with open(path, "rb") as f:
        bitj, nbits, nchunks = np.frombuffer(f.read(12), dtype=np.int32)
        padded = nbits + (bitj - nbits % bitj) % bitj
        data = np.frombuffer(f.read(), dtype=np.uint8)[: nchunks * padded // 8]
    bits = np.unpackbits(data.reshape(nchunks, padded // 8), axis=1, bitorder="big")
    return bits[:, :nbits]


def write_bcc_inputs(in_dir: str, out_dir: str, A_bins, Z_bins=None, *, gamma=0.05, B_MLT=32,
                     A_row_masks=None, Z_row_masks=None, col_mask=None, gamma_type=None, Ireq=None,
                     T_bins=None, S_bins=None, kappa_squared=None, qc_strategy="YnWt", qr_strategy="YnWt",
                     name="bcc.in", extra_statements=()) -> str:
    """Write the .b16 files of one bcc problem and the .in file that names them.

    A_bins / Z_bins: per-bin 0/1 arrays (rows x SNPs).  Masks (0/1 vectors) are
    optional; absent masks mean every row / column is used.  T_bins / S_bins:
    per-bin 0/1 covariate arrays (case rows x T_ncols, control rows x
    T_ncols), written as T_t / T_n and S_t / S_n files like A; absent means
    the reference's single column of ones.  Returns the path of the .in file.
    Outputs of a solve go to ``out_dir``.  ``extra_statements`` (name, value)
    pairs are written before END, e.g. ("GLOBAL_TEST_TYPE", ...) to replace
    the solve by the scorebox, or the GLOBAL_scramble_* statements.
    """
    os.makedirs(in_dir, exist_ok=True)
    nbins = len(A_bins)
    Z_bins = Z_bins if Z_bins is not None else [None] * nbins
    ncols = A_bins[0].shape[1]
    has_Z = any(z is not None and z.shape[0] > 0 for z in Z_bins)
    for nb in range(nbins):
        A = np.asarray(A_bins[nb], np.uint8)
        write_b16(os.path.join(in_dir, "A_%02d_t.b16" % nb), A)
        write_b16(os.path.join(in_dir, "A_%02d_n.b16" % nb), A.T)
        m = np.ones(A.shape[0], np.uint8) if A_row_masks is None else np.asarray(A_row_masks[nb], np.uint8)
        write_b16(os.path.join(in_dir, "mr_A_%02d.b16" % nb), m[None, :])
        if has_Z:
            Z = np.asarray(Z_bins[nb], np.uint8)
            write_b16(os.path.join(in_dir, "Z_%02d_t.b16" % nb), Z)
            write_b16(os.path.join(in_dir, "Z_%02d_n.b16" % nb), Z.T)
            mz = np.ones(Z.shape[0], np.uint8) if Z_row_masks is None else np.asarray(Z_row_masks[nb], np.uint8)
            write_b16(os.path.join(in_dir, "mr_Z_%02d.b16" % nb), mz[None, :])
    T_ncols = 1
    if T_bins is not None:
        T_ncols = np.asarray(T_bins[0]).shape[1]
        for nb in range(nbins):
            T = np.asarray(T_bins[nb], np.uint8)
            S = np.asarray(S_bins[nb], np.uint8)
            write_b16(os.path.join(in_dir, "T_%02d_t.b16" % nb), T)
            write_b16(os.path.join(in_dir, "T_%02d_n.b16" % nb), T.T)
            write_b16(os.path.join(in_dir, "S_%02d_t.b16" % nb), S)
            write_b16(os.path.join(in_dir, "S_%02d_n.b16" % nb), S.T)
    mc = np.ones(ncols, np.uint8) if col_mask is None else np.asarray(col_mask, np.uint8)
    write_b16(os.path.join(in_dir, "mc_A.b16"), mc[None, :])

    def lst(fmt):
        return ",".join(fmt % nb for nb in range(nbins))

    lines = [
        "GLOBAL_verbose= 0;",
        "GLOBAL_thread_count= 1;",
        "GLOBAL_omp_type= 0;",
        "GLOBAL_TEST_TYPE= lakcluster_driver;",
        "GLOBAL_QR_strategy= %s;" % qr_strategy,
        "GLOBAL_QC_strategy= %s;" % qc_strategy,
        "GLOBAL_NBINS= %d;" % nbins,
        "GLOBAL_B_MLT= %d;" % B_MLT,
        "GLOBAL_gamma= %0.4f;" % gamma,
    ]
    if gamma_type is not None:
        lines.append("GLOBAL_gamma_type= %d;" % gamma_type)
    if Ireq is not None:
        lines.append("GLOBAL_Ireq= %d;" % Ireq)
    if kappa_squared is not None:
        lines.append("GLOBAL_kappa_squared= %0.6f;" % kappa_squared)
    lines += [
        "GLOBAL_DIR_XPRE= %s;" % os.path.abspath(in_dir),
        "GLOBAL_A_n_name_= %s;" % lst("A_%02d_n.b16"),
        "GLOBAL_A_t_name_= %s;" % lst("A_%02d_t.b16"),
        "GLOBAL_A_n_rows_= %s;" % ",".join(str(np.asarray(a).shape[0]) for a in A_bins),
        "GLOBAL_A_n_cols= %d;" % ncols,
        "GLOBAL_A_n_rind_= %s;" % lst("mr_A_%02d.b16"),
        "GLOBAL_A_n_cind= mc_A.b16;",
    ]
    if has_Z:
        lines += [
            "GLOBAL_Z_n_name_= %s;" % lst("Z_%02d_n.b16"),
            "GLOBAL_Z_t_name_= %s;" % lst("Z_%02d_t.b16"),
            "GLOBAL_Z_n_rows_= %s;" % ",".join(str(np.asarray(z).shape[0]) for z in Z_bins),
            "GLOBAL_Z_n_rind_= %s;" % lst("mr_Z_%02d.b16"),
        ]
    if T_bins is not None:
        lines += [
            "GLOBAL_T_t_name_= %s;" % lst("T_%02d_t.b16"),
            "GLOBAL_T_n_name_= %s;" % lst("T_%02d_n.b16"),
            "GLOBAL_S_t_name_= %s;" % lst("S_%02d_t.b16"),
            "GLOBAL_S_n_name_= %s;" % lst("S_%02d_n.b16"),
        ]
    lines += [
        "GLOBAL_Y_n_cols= 0;",
        "GLOBAL_T_n_cols= %d;" % T_ncols,
        "GLOBAL_DIR_NAME= %s;" % os.path.abspath(out_dir),
    ]
    lines += ["%s= %s;" % (k, v) for k, v in extra_statements]
    lines += ["END= 0;"]
    path = os.path.join(in_dir, name)
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")
    return path


def read_trace(out_dir: str):
    """(trace rows, xdrop_a pairs, xdrop_b pairs) from a solve's output files."""
    def rows(fn, conv):
        p = os.path.join(out_dir, fn)
        with open(p) as f:
            return [tuple(conv(t) for t in line.split()) for line in f if line.strip()]
    trace = rows("out_trace.txt", float)
    xa = rows("out_xdrop_a.txt", int)
    xb = rows("out_xdrop_b.txt", int)
    return trace, xa, xb
