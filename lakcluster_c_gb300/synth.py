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

import math
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


def log_uniform_int(rng, lo, hi):
    return int(round(math.exp(rng.uniform(math.log(lo), math.log(hi)))))


def null_instance(seed, rows=(1024, 8192), cols=(4096, 32768), maf=(0.05, 0.5), k_rows=None, k_cols=None,
                  flip=0.05):
    """One label-shuffled null instance of the case/control setup: a pooled
    sample of r rows x c SNPs (MAF U[maf]), with a planted bicluster in the
    first half, then case/control labels assigned by a random permutation of
    the pooled rows (so the planted rows are spread over both groups).
    r ~ logU[rows], c ~ logU[cols]; one covariate bin."""
    rng = np.random.default_rng(seed)
    r = log_uniform_int(rng, *rows)
    c = log_uniform_int(rng, *cols)
    f = maf[0] + (maf[1] - maf[0]) * rng.random(c)
    X = _bernoulli_cols(rng, r, f)
    kr = k_rows or max(2, r // 16)
    kc = k_cols or max(2, c // 32)
    rr = rng.permutation(r // 2)[:kr]
    cc = rng.permutation(c)[:kc]
    pat = (rng.random(kc) < 0.5).astype(np.uint8)
    X[np.ix_(rr, cc)] = np.tile(pat, (kr, 1)) ^ (rng.random((kr, kc)) < flip).astype(np.uint8)
    perm = rng.permutation(r)
    A = np.ascontiguousarray(X[perm[: r // 2]])
    Z = np.ascontiguousarray(X[perm[r // 2:]])
    inst = BccInstance("null_%d" % seed, c)
    inst.A_bins.append(A)
    inst.Z_bins.append(Z)
    return inst


def served_request(seed, rows=(512, 16384), cols=(2048, 65536), maf=(0.05, 0.5), case_fraction=0.5,
                   max_categories=3, flip=0.05):
    """One request of the served stream: r ~ logU[rows] rows (case fraction
    0.5), c ~ logU[cols] SNPs, MAF U[maf], k ~ U{0..3} covariate categories
    (NBINS = max(1, k), rows assigned uniformly), a planted bicluster in the
    cases."""
    rng = np.random.default_rng(seed)
    r = log_uniform_int(rng, *rows)
    c = log_uniform_int(rng, *cols)
    k = int(rng.integers(0, max_categories + 1))
    nb = max(1, k)
    n_case = max(2, int(round(r * case_fraction)))
    n_ctrl = max(2, r - n_case)
    f = maf[0] + (maf[1] - maf[0]) * rng.random(c)
    A = _bernoulli_cols(rng, n_case, f)
    Z = _bernoulli_cols(rng, n_ctrl, f)
    kr, kc = max(2, n_case // 16), max(2, c // 32)
    rr = rng.permutation(n_case)[:kr]
    cc = rng.permutation(c)[:kc]
    pat = (rng.random(kc) < 0.5).astype(np.uint8)
    A[np.ix_(rr, cc)] = np.tile(pat, (kr, 1)) ^ (rng.random((kr, kc)) < flip).astype(np.uint8)
    bA = (rng.random(n_case) * nb).astype(np.int64)
    bZ = (rng.random(n_ctrl) * nb).astype(np.int64)
    inst = BccInstance("req_%d" % seed, c)
    for b in range(nb):
        a, z = A[bA == b], Z[bZ == b]
        if a.shape[0] == 0 or z.shape[0] == 0:   # keep every bin populated
            a, z = A[:2], Z[:2]
        inst.A_bins.append(np.ascontiguousarray(a))
        inst.Z_bins.append(np.ascontiguousarray(z))
    return inst


def _packed_bernoulli_rows(rng, nrows, f, planted=None, chunk=1024):
    """Rows of Bernoulli(f) bits packed as solve.pack_rows packs them (MSB
    first, rows padded to 16 bits), drawn `chunk` rows at a time from float32
    uniforms so that host memory stays at a few chunks whatever the size.
    `planted` = (row indices, column indices, 0/1 pattern, flip) overwrites
    those entries of the listed rows with the pattern, each bit flipped with
    probability flip."""
    c = f.size
    rb = (c + 15) // 16 * 2
    out = np.zeros((nrows, rb), np.uint8)
    f32 = f.astype(np.float32)[None, :]
    if planted is not None:
        prow, pcol, pat, flip = planted
        in_plant = np.zeros(nrows, bool)
        in_plant[prow] = True
    for r0 in range(0, nrows, chunk):
        r1 = min(nrows, r0 + chunk)
        bits = (rng.random((r1 - r0, c), dtype=np.float32) < f32).astype(np.uint8)
        if planted is not None:
            rows = np.nonzero(in_plant[r0:r1])[0]
            if rows.size:
                flips = (rng.random((rows.size, pcol.size)) < flip).astype(np.uint8)
                bits[np.ix_(rows, pcol)] = pat[None, :] ^ flips
        pad = rb * 8 - c
        if pad:
            bits = np.concatenate([bits, np.zeros((r1 - r0, pad), np.uint8)], axis=1)
        out[r0:r1] = np.packbits(bits, axis=1, bitorder="big")
    return out


def served_request_packed(seed, rows=(512, 16384), cols=(2048, 65536), maf=(0.05, 0.5), case_fraction=0.5,
                          max_categories=3, flip=0.05):
    """A served-stream request drawn like served_request (r ~ logU[rows] rows,
    case fraction 0.5, c ~ logU[cols] SNPs, MAF U[maf], k ~ U{0..3} covariate
    categories with NBINS = max(1, k) and rows assigned uniformly, a planted
    bicluster of r_case/16 rows x c/32 SNPs in the cases), with the rows
    generated and packed in chunks so that requests at the top of the size
    range (16384 x 65536) need no unpacked copy.  Returns a BccInstance whose
    A_bins / Z_bins hold packed rows (solve.Problem's packed_ncols form)."""
    rng = np.random.default_rng(seed)
    r = log_uniform_int(rng, *rows)
    c = log_uniform_int(rng, *cols)
    k = int(rng.integers(0, max_categories + 1))
    nb = max(1, k)
    n_case = max(2, int(round(r * case_fraction)))
    n_ctrl = max(2, r - n_case)
    f = maf[0] + (maf[1] - maf[0]) * rng.random(c)
    kr, kc = max(2, n_case // 16), max(2, c // 32)
    prow = rng.permutation(n_case)[:kr]
    pcol = np.sort(rng.permutation(c)[:kc])
    pat = (rng.random(kc) < 0.5).astype(np.uint8)
    A = _packed_bernoulli_rows(rng, n_case, f, (prow, pcol, pat, flip))
    Z = _packed_bernoulli_rows(rng, n_ctrl, f)
    bA = (rng.random(n_case) * nb).astype(np.int64)
    bZ = (rng.random(n_ctrl) * nb).astype(np.int64)
    inst = BccInstance("req_packed_%d" % seed, c, planted_rows=prow, planted_cols=pcol)
    for b in range(nb):
        a, z = A[bA == b], Z[bZ == b]
        if a.shape[0] == 0 or z.shape[0] == 0:   # keep every bin populated
            a, z = A[:2], Z[:2]
        inst.A_bins.append(np.ascontiguousarray(a))
        inst.Z_bins.append(np.ascontiguousarray(z))
    return inst


def _pack_bits_torch(bits):
    """(n, c) bool tensor -> (n, rup(c,16)/8) uint8 tensor, MSB first (the
    layout of solve.pack_rows)."""
    import torch
    n, c = bits.shape
    pad = (16 - c % 16) % 16
    if pad:
        bits = torch.cat([bits, torch.zeros((n, pad), dtype=torch.bool, device=bits.device)], dim=1)
    w = torch.tensor([128, 64, 32, 16, 8, 4, 2, 1], dtype=torch.int32, device=bits.device)
    return (bits.view(n, -1, 8).to(torch.int32) * w).sum(dim=2).to(torch.uint8)


def null_instance_packed(seed, rows=(1024, 8192), cols=(4096, 32768), maf=(0.05, 0.5), flip=0.05,
                         device="cuda"):
    """A label-shuffled null instance drawn like null_instance (r ~ logU[rows]
    pooled rows, c ~ logU[cols] SNPs, MAF U[maf], an r/16 x c/32 bicluster
    planted in the first half of the pooled rows with the given flip rate,
    then case/control labels from a random permutation of the pooled rows,
    one covariate bin), with the Bernoulli draws made on `device` by a torch
    Philox generator seeded with `seed` and the rows packed there, so that
    hundreds of instances are drawn in seconds.  Sizes, frequencies, the
    bicluster and the permutation come from the numpy stream of `seed`.
    Returns a BccInstance of packed rows (solve.Problem's packed_ncols form)."""
    import torch
    rng = np.random.default_rng(seed)
    r = log_uniform_int(rng, *rows)
    c = log_uniform_int(rng, *cols)
    f = maf[0] + (maf[1] - maf[0]) * rng.random(c)
    kr, kc = max(2, r // 16), max(2, c // 32)
    rr = rng.permutation(r // 2)[:kr]
    cc = rng.permutation(c)[:kc]
    pat = (rng.random(kc) < 0.5).astype(np.uint8)
    flips = rng.random((kr, kc)) < flip
    perm = rng.permutation(r)
    g = torch.Generator(device=device)
    g.manual_seed(int(seed))
    fd = torch.from_numpy(f.astype(np.float32)).to(device)
    X = torch.rand((r, c), generator=g, device=device) < fd[None, :]
    blk = torch.from_numpy((pat[None, :].astype(bool) ^ flips)).to(device)
    X[torch.from_numpy(rr).to(device)[:, None], torch.from_numpy(cc).to(device)[None, :]] = blk
    P = _pack_bits_torch(X[torch.from_numpy(perm).to(device)])
    del X
    host = P.cpu().numpy()
    inst = BccInstance("null_packed_%d" % seed, c, planted_rows=rr, planted_cols=cc)
    inst.A_bins.append(np.ascontiguousarray(host[: r // 2]))
    inst.Z_bins.append(np.ascontiguousarray(host[r // 2:]))
    return inst
