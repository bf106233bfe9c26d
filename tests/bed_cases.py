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


# --- b16_merge --------------------------------------------------------------------
# Several converted studies (.b16 / .bim / .fam triples as bed_to_b16 writes
# them) merged into one (dir_c/bed_to_b16.c:1659-1985): the patients common to
# every study (by FID + IID), the SNP alleles of all studies interleaved by
# allele frequency.  Each study draws its patients from a shared pool in its
# own order, and its allele frequencies from a coarse grid so that studies tie.
#
# name: (seed, [(patients, alleles), ...])
MERGE_CASES = {
    "merge_2x": (21, [(90, 40), (75, 33)]),
    "merge_3x_ragged": (22, [(301, 97), (257, 130), (280, 61)]),
    "merge_4x_small": (23, [(20, 9), (17, 12), (25, 7), (19, 15)]),
}


def merge_inputs(name):
    """Per study: (fam lines, bim lines, b16 bytes)."""
    seed, studies = MERGE_CASES[name]
    rng = np.random.default_rng(seed)
    pool = max(n for n, _ in studies) + 40
    out = []
    for n_pat, n_all in studies:
        pats = rng.permutation(pool)[:n_pat]
        fam = ["F%d I%d 0 0 %d %d" % (p // 4, p, 1 + p % 2, 1 + (p % 3 == 0)) for p in pats]
        freq = np.sort(rng.integers(1, 40, n_all) / 40.0)
        bim = ["%d\trs%d\t0\t%d\tA\tG\tand(orig)\t%f\t%f\t%f\t%f" % (1 + a % 22, int(rng.integers(1, 10 ** 6)),
                                                                    100 * a, rng.random() * 0.01, f,
                                                                    rng.random() * 0.02, min(f, 1 - f))
               for a, f in enumerate(freq)]
        row_bytes = (n_pat + 15) // 16 * 2
        bits = np.zeros((n_all, 8 * row_bytes), np.uint8)
        bits[:, :n_pat] = rng.random((n_all, n_pat)) < 0.4
        b16 = np.array([16, n_pat, n_all], np.int32).tobytes() + np.packbits(bits, 1, bitorder="big").tobytes()
        out.append((fam, bim, b16))
    return out


def write_merge_case(name, d):
    """Write the studies as <d>/<name>_<k>.{b16,bim,fam}; returns the file lists."""
    os.makedirs(d, exist_ok=True)
    files = []
    for k, (fam, bim, b16) in enumerate(merge_inputs(name)):
        base = os.path.join(d, "%s_%d" % (name, k))
        with open(base + ".fam", "w") as f:
            f.write("".join(x + "\n" for x in fam))
        with open(base + ".bim", "w") as f:
            f.write("".join(x + "\n" for x in bim))
        with open(base + ".b16", "wb") as f:
            f.write(b16)
        files.append((base + ".b16", base + ".bim", base + ".fam"))
    return files


def merge_in_text(name, d, out_dir):
    files = [tuple(os.path.join(d, "%s_%d.%s" % (name, k, x)) for x in ("b16", "bim", "fam"))
             for k in range(len(MERGE_CASES[name][1]))]
    out = os.path.join(out_dir, name)
    return "\n".join([
        "GLOBAL_verbose= 0;", "GLOBAL_thread_count= 1;", "GLOBAL_omp_type= 0;",
        "GLOBAL_TEST_TYPE= b16_merge;", "GLOBAL_n_file= %d;" % len(files),
        "GLOBAL_fname_b16_0in_= %s;" % ",".join(f[0] for f in files),
        "GLOBAL_fname_bim_0in_= %s;" % ",".join(f[1] for f in files),
        "GLOBAL_fname_fam_0in_= %s;" % ",".join(f[2] for f in files),
        "GLOBAL_fname_b16_out= %s_out.b16;" % out, "GLOBAL_fname_bim_out= %s_out.bim;" % out,
        "GLOBAL_fname_fam_out= %s_out.fam;" % out, "END= 0;", ""])


def _quicksort_str(keys, idx, limit=1024 * 32):
    """charpQuickSort_index (dir_c/Quicksort.c:364-414): the partition of
    dQuickSort_index with strcmp order (byte order of the strings)."""
    st = [(0, len(keys) - 1, 0)] if keys else []
    while st:
        l, r, depth = st.pop()
        if l >= r:
            continue
        pivot = keys[l]
        i, j = l, r + 1
        while True:
            i += 1
            while i <= r and keys[i] <= pivot:
                i += 1
            j -= 1
            while keys[j] > pivot:
                j -= 1
            if i >= j:
                break
            keys[i], keys[j] = keys[j], keys[i]
            idx[i], idx[j] = idx[j], idx[i]
        keys[l], keys[j] = keys[j], keys[l]
        idx[l], idx[j] = idx[j], idx[l]
        if depth < limit:
            st.append((l, j - 1, depth + 1))
            st.append((j + 1, r, depth + 1))


def merge_oracle(studies):
    """TEST INFRASTRUCTURE ONLY: b16_merge (dir_c/bed_to_b16.c:1659-1985) in
    Python.  studies: [(fam lines, bim lines, b16 bytes)].  Returns the three
    output files' bytes."""
    n_file = len(studies)
    keys, order = [], []
    for fam, _, _ in studies:
        k = [(ln.split()[0] + ln.split()[1]).encode() for ln in fam]
        idx = list(range(len(k)))
        kk = list(k)
        _quicksort_str(kk, idx)
        keys.append(kk)
        order.append(idx)
    # charpIntersectall_index_index_driver (dir_c/Quicksort.c:624-690)
    pos = [0] * n_file
    inter = []  # per intersected patient: original index in each study
    while all(pos[f] < len(keys[f]) for f in range(n_file)):
        fmin, found = 0, False
        for f in range(n_file):
            if keys[fmin][pos[fmin]] > keys[f][pos[f]]:
                fmin, found = f, True
            elif keys[fmin][pos[fmin]] < keys[f][pos[f]]:
                found = True
        if found:
            pos[fmin] += 1
        else:
            inter.append([order[f][pos[f]] for f in range(n_file)])
            for f in range(n_file):
                pos[f] += 1
    n_int = len(inter)
    fam0 = studies[0][0]
    fam_txt = "".join(" ".join(fam0[p[0]].split()[:6]) + "\n" for p in inter)
    # SNPs interleaved by allele frequency, ties to the lower study
    rows = []
    nb = [0] * n_file
    bim_txt = []
    heads = []
    for fam, bim, b16 in studies:
        n_pat = len(fam)
        rb = (n_pat + 15) // 16 * 2
        heads.append(np.frombuffer(b16[12:], np.uint8).reshape(-1, rb))
    while True:
        fmin = -1
        for f in range(n_file):
            if nb[f] < len(studies[f][1]):
                if fmin < 0 or float(studies[f][1][nb[f]].split()[8]) < float(studies[fmin][1][nb[fmin]].split()[8]):
                    fmin = f
        if fmin < 0:
            break
        bim_txt.append("\t".join(studies[fmin][1][nb[fmin]].split()[:11]) + "\n")
        src = np.unpackbits(heads[fmin][nb[fmin]], bitorder="big")
        rows.append(src[[p[fmin] for p in inter]])
        nb[fmin] += 1
    rb = (n_int + 15) // 16 * 2
    out = np.zeros((len(rows), 8 * rb), np.uint8)
    for r, v in enumerate(rows):
        out[r, :n_int] = v
    n_bim = sum(len(s[1]) for s in studies)
    b16 = np.array([16, n_int, n_bim], np.int32).tobytes() + np.packbits(out, 1, bitorder="big").tobytes()
    return {"b16": b16, "bim": "".join(bim_txt).encode(), "fam": fam_txt.encode()}


MERGE_GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "b16_merge.npz")


def load_merge_golden():
    z = np.load(MERGE_GOLDEN, allow_pickle=False)
    return {n: {k: z["%s/%s" % (n, k)].tobytes() for k in ("b16", "bim", "fam")} for n in MERGE_CASES}
