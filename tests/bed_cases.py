"""Synthetic PLINK inputs (.bed / .bim / .fam) for the bed_to_b16 tests.

No genotype files ship with the reference or this repository.  Each case is
drawn from a seeded numpy stream: per-SNP minor-allele frequencies, genotype
codes from Hardy-Weinberg proportions, a share of SNPs pushed outside the
conversion's filters (rare, often missing, or out of Hardy-Weinberg
proportions), and a share of patients with many missing calls, so that every
filter of bed_to_b16 (dir_c/bed_to_b16.c:956-975) removes something.
"""
import os

import numpy as np

# name: (SNPs, patients, seed, thresholds (snp_mss, snp_maf, snp_I_opt, pat_mss))
BED_CASES = {
    "bed_301x97": (301, 97, 11, (0.01, 0.25, 0.01, 0.04)),
    "bed_1000x512": (1000, 512, 12, (0.05, 0.10, 0.02, 0.10)),
    "bed_777x1030": (777, 1030, 13, (0.02, 0.05, 0.05, 0.05)),
    "bed_64x4": (64, 4, 14, (0.5, 0.0, 1.0, 0.5)),
}


def genotypes(n_snp, n_fam, seed):
    """n_snp x n_fam codes: 0 hom minor, 1 missing, 2 het, 3 hom major."""
    rng = np.random.default_rng(seed)
    q = rng.uniform(0.02, 0.5, n_snp)                       # minor-allele frequency
    q[rng.random(n_snp) < 0.1] = rng.uniform(0.0, 0.02, int(np.sum(rng.random(n_snp) < 0.1)) or 1)[0]
    p = 1 - q
    probs = np.stack([q * q, 2 * p * q, p * p], 1)          # nor, xor, and
    skew = rng.random(n_snp) < 0.1                          # out of Hardy-Weinberg proportions
    probs[skew] = np.stack([q[skew], np.zeros(skew.sum()) + 0.05, 1 - q[skew] - 0.05], 1).clip(0.0, 1.0)
    probs /= probs.sum(1, keepdims=True)
    u = rng.random((n_snp, n_fam))
    cum = np.cumsum(probs, 1)
    g = np.where(u < cum[:, :1], 0, np.where(u < cum[:, 1:2], 2, 3)).astype(np.uint8)
    miss_snp = np.where(rng.random(n_snp) < 0.15, 0.08, 0.003)
    miss_pat = np.where(rng.random(n_fam) < 0.1, 0.1, 0.0)
    m = rng.random((n_snp, n_fam)) < (miss_snp[:, None] + miss_pat[None, :])
    g[m] = 1
    return g


def pack_bed(g):
    """Codes (n_snp x n_fam) -> .bed records: 4 patients per byte, first patient in the low bits."""
    n_snp, n_fam = g.shape
    n_bam = (n_fam + 3) // 4
    pad = np.zeros((n_snp, 4 * n_bam), np.uint8)
    pad[:, :n_fam] = g
    q = pad.reshape(n_snp, n_bam, 4).astype(np.uint32)
    return (q[..., 0] | (q[..., 1] << 2) | (q[..., 2] << 4) | (q[..., 3] << 6)).astype(np.uint8)


def write_case(name, d):
    """Write <d>/<name>.{bed,bim,fam}; returns their paths."""
    n_snp, n_fam, seed, _ = BED_CASES[name]
    g = genotypes(n_snp, n_fam, seed)
    os.makedirs(d, exist_ok=True)
    base = os.path.join(d, name)
    with open(base + ".bed", "wb") as f:
        f.write(bytes([108, 27, 1]))
        f.write(pack_bed(g).tobytes())
    with open(base + ".bim", "w") as f:
        for s in range(n_snp):
            f.write("%d\trs%d\t0\t%d\t%s\t%s\n" % (1 + s % 22, 1000 + s, 10000 + 37 * s, "ACGT"[s % 4], "ACGT"[(s + 1) % 4]))
    with open(base + ".fam", "w") as f:
        for i in range(n_fam):
            f.write("FAM%d IND%d 0 0 %d %d\n" % (i // 3, i, 1 + i % 2, 1 + (i % 5 == 0)))
    return base + ".bed", base + ".bim", base + ".fam"


def in_text(name, d, out_dir):
    """The .in statements of the conversion of case `name` (files in d)."""
    _, _, _, (smss, smaf, sI, pmss) = BED_CASES[name]
    base = os.path.join(d, name)
    out = os.path.join(out_dir, name)
    return "\n".join([
        "GLOBAL_verbose= 0;", "GLOBAL_thread_count= 1;", "GLOBAL_omp_type= 0;",
        "GLOBAL_TEST_TYPE= bed_to_b16;",
        "GLOBAL_fname_bed_0in= %s.bed;" % base, "GLOBAL_fname_bim_0in= %s.bim;" % base,
        "GLOBAL_fname_fam_0in= %s.fam;" % base,
        "GLOBAL_fname_b16_out= %s_out.b16;" % out, "GLOBAL_fname_bim_out= %s_out.bim;" % out,
        "GLOBAL_fname_fam_out= %s_out.fam;" % out,
        "GLOBAL_snp_mss_threshold= %r;" % smss, "GLOBAL_snp_maf_threshold= %r;" % smaf,
        "GLOBAL_snp_I_opt_threshold= %r;" % sI, "GLOBAL_pat_mss_threshold= %r;" % pmss,
        "GLOBAL_DIR_NAME= %s;" % out_dir,
        "END= 0;", ""])


def read_outputs(name, out_dir):
    out = os.path.join(out_dir, name)
    return {k: open(out + "_out." + k, "rb").read() for k in ("b16", "bim", "fam")}


# --- oracle -----------------------------------------------------------------------
# TEST INFRASTRUCTURE ONLY: a numpy / Python restatement of bed_to_b16
# (dir_c/bed_to_b16.c:711-1355), the checker of the GPU conversion; pinned to
# the reference program's own outputs by tests/test_bed_cpu.py.

def _quicksort_index(d, idx, limit=1024 * 32):
    """dQuickSort_index (dir_c/Quicksort.c:216-248) on lists d, idx."""
    st = [(0, len(d) - 1, 0)] if d else []
    while st:
        l, r, depth = st.pop()
        if l >= r:
            continue
        pivot = d[l]
        i, j = l, r + 1
        while True:
            i += 1
            while i <= r and d[i] <= pivot:
                i += 1
            j -= 1
            while d[j] > pivot:
                j -= 1
            if i >= j:
                break
            d[i], d[j] = d[j], d[i]
            idx[i], idx[j] = idx[j], idx[i]
        d[l], d[j] = d[j], d[l]
        idx[l], idx[j] = idx[j], idx[l]
        if depth < limit:
            st.append((l, j - 1, depth + 1))
            st.append((j + 1, r, depth + 1))


def oracle(records, n_fam, thresholds):
    """records: n_snp x n_bam .bed bytes.  Returns (b16 bytes, list of
    (bim index, type, I, freq, mss, maf) per sorted allele, kept patients)."""
    import math
    smss, smaf, sI, pmss = thresholds
    n_snp, n_bam = records.shape
    codes = np.stack([(records >> (2 * k)) & 3 for k in range(4)], 2).reshape(n_snp, 4 * n_bam)
    cnt = np.stack([(codes == c).sum(1) for c in range(4)], 1)     # all 4 * n_bam slots, as the reference
    miss = (codes[:, :n_fam] == 1).sum(0)
    keep_s, stats, mode = [], {}, np.zeros(n_snp, np.uint8)
    for s in range(n_snp):
        c0, c1, c2, c3 = (int(x) for x in cnt[s])
        tot = c3 + c2 + c0
        tmp_min = 1.0 / tot if tot else math.inf
        fm = c1 / n_fam
        fa, fx, fn = (c3 / tot, c2 / tot, c0 / tot) if tot else (math.nan,) * 3
        p, q = fa + 0.5 * fx, fn + 0.5 * fx
        def term(f, e):
            return f * math.log(f / max(tmp_min, e)) if f > 0 else math.nan
        I = term(fa, math.pow(p, 2)) + term(fx, 2 * p * q) + term(fn, math.pow(q, 2))
        m = 2
        if c2 >= c3 and c2 >= c0: m = 2
        if c0 >= c3 and c0 >= c2: m = 0
        if c3 >= c2 and c3 >= c0: m = 3
        mode[s] = m
        stats[s] = (fa, fx, fn, fm, p, q, I)
        if tot > 0 and fa > 0 and fx > 0 and fn > 0 and min(p, q) >= smaf and fm <= smss and I <= sI:
            keep_s.append(s)
    keep_p = [f for f in range(n_fam) if n_snp - miss[f] > 0 and miss[f] / n_snp <= pmss]
    freq, info = [], []
    for s in keep_s:
        fa, fx, fn, fm, p, q, I = stats[s]
        for f in (fn, fx, fa):
            freq.append(f)
            info.append((s, I, f, fm, min(p, q)))
    d, order = list(freq), list(range(len(freq)))
    _quicksort_index(d, order)
    n_pat = len(keep_p)
    row_bytes = (n_pat + 15) // 16 * 2
    sub = codes[np.ix_(keep_s, keep_p)] if keep_s and keep_p else np.zeros((len(keep_s), n_pat), np.uint8)
    sub = np.where(sub == 1, mode[keep_s][:, None], sub)
    rows = np.zeros((3 * len(keep_s), row_bytes * 8), np.uint8)
    for a, code in enumerate((0, 2, 3)):
        rows[a::3, :n_pat] = (sub == code)
    A_n = np.packbits(rows, axis=1, bitorder="big")
    b16 = np.array([16, n_pat, 3 * len(keep_s)], np.int32).tobytes() + A_n[order].tobytes()
    bim = [(info[o][0], "and(orig)") + tuple(info[o][1:]) for o in order]
    return b16, bim, keep_p


def oracle_files(name, d):
    """The three output files of case `name` as the oracle writes them."""
    bed, bim, fam = (os.path.join(d, name + x) for x in (".bed", ".bim", ".fam"))
    n_snp, n_fam, _, thr = BED_CASES[name]
    raw = np.fromfile(bed, np.uint8)[3:].reshape(n_snp, (n_fam + 3) // 4)
    b16, alleles, keep_p = oracle(raw, n_fam, thr)
    bl = open(bim).read().split()
    fl = open(fam).read().split()
    bim_txt = "".join("%s\t%s\t%s\t%s\t%s\t%s\t%s\t%f\t%f\t%f\t%f\n" % (tuple(bl[6 * s:6 * s + 6]) + (t, I, f, m, maf))
                      for s, t, I, f, m, maf in alleles)
    fam_txt = "".join(" ".join(fl[6 * p:6 * p + 6]) + "\n" for p in keep_p)
    return {"b16": b16, "bim": bim_txt.encode(), "fam": fam_txt.encode()}


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "bed_to_b16.npz")


def load_golden():
    z = np.load(GOLDEN, allow_pickle=False)
    return {n: {k: z["%s/%s" % (n, k)].tobytes() for k in ("b16", "bim", "fam")} for n in BED_CASES}
