"""Seeded synthetic bcc inputs with the shapes of the benchmark configurations.

No genotype data ships with the reference or this repository, so every input
is generated: a numpy PCG64 stream from the given seed, Bernoulli draws by
comparing uniforms to the per-column minor-allele frequency, and a planted
bicluster (rows share a random column pattern, each bit flipped with the
stated probability).  Bit 1 is the minor allele (+1), bit 0 is -1.

Configurations (rows x SNP columns):
  case_only_1024   1024 x 1024 cases, Bernoulli(0.5), 45 x 45 bicluster with
                   10% flips, one bin, no controls
  case_control_2bin cases 4096 x 16384 and controls 4096 x 16384, MAF U[0.05,0.5],
                   256 x 512 bicluster in the cases with 5% flips, rows assigned
                   uniformly to 2 covariate bins
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


@dataclass
class BccInstance:
    name: str
    ncols: int
    A_bins: list = field(default_factory=list)   # per bin: uint8 0/1 matrix (rows x ncols)
    Z_bins: list = field(default_factory=list)
    planted_rows: np.ndarray | None = None       # global case-row indices of the bicluster
    planted_cols: np.ndarray | None = None

    @property
    def nbins(self):
        return len(self.A_bins)


def _bernoulli_cols(rng, nrows, f):
    return (rng.random((nrows, f.size)) < f[None, :]).astype(np.uint8)


def case_only(n_rows=1024, n_cols=1024, k=45, flip=0.1, seed=1) -> BccInstance:
    rng = np.random.default_rng(seed)
    A = (rng.random((n_rows, n_cols)) < 0.5).astype(np.uint8)
    r = rng.permutation(n_rows)[:k]
    c = rng.permutation(n_cols)[:k]
    pat = (rng.random(k) < 0.5).astype(np.uint8)
    blk = np.tile(pat, (k, 1)) ^ (rng.random((k, k)) < flip).astype(np.uint8)
    A[np.ix_(r, c)] = blk
    return BccInstance("case_only_%d" % n_rows, n_cols, [A], [np.zeros((0, n_cols), np.uint8)], r, c)


def case_control(n_case=4096, n_ctrl=4096, n_cols=16384, k_rows=256, k_cols=512, flip=0.05,
                 nbins=2, maf=(0.05, 0.5), seed=2) -> BccInstance:
    rng = np.random.default_rng(seed)
    f = maf[0] + (maf[1] - maf[0]) * rng.random(n_cols)
    A = _bernoulli_cols(rng, n_case, f)
    Z = _bernoulli_cols(rng, n_ctrl, f)
    r = rng.permutation(n_case)[:k_rows]
    c = rng.permutation(n_cols)[:k_cols]
    pat = (rng.random(k_cols) < 0.5).astype(np.uint8)
    A[np.ix_(r, c)] = np.tile(pat, (k_rows, 1)) ^ (rng.random((k_rows, k_cols)) < flip).astype(np.uint8)
    bA = (rng.random(n_case) * nbins).astype(np.int64)
    bZ = (rng.random(n_ctrl) * nbins).astype(np.int64)
    inst = BccInstance("case_control_%dbin" % nbins, n_cols, planted_rows=r, planted_cols=c)
    for b in range(nbins):
        inst.A_bins.append(np.ascontiguousarray(A[bA == b]))
        inst.Z_bins.append(np.ascontiguousarray(Z[bZ == b]))
    return inst
