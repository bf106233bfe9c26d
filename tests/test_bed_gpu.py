"""bed_to_b16 on the GPU (lakcluster_c_gb300/csrc/bed.cu).

  * the four synthetic PLINK cases through the reference's own .in interface
    (lakgb_bcc_run_in_file, GLOBAL_TEST_TYPE= bed_to_b16): the .b16, .bim and
    .fam files byte for byte equal to the reference program's
    (tests/golden/bed_to_b16.npz);
  * a larger case through the in-memory entry point (lakgb_bed_to_b16_mem)
    against the numpy restatement: kept SNPs and patients, allele order and
    every bit of the allele matrix; and, on it, the matrix's structure: every
    kept patient has exactly one of the three allele bits of every kept SNP,
    and the padding bits past the last patient are zero.
"""
import ctypes as C

import numpy as np
import pytest

import bcc_cases as bc
import bed_cases as bd

pytestmark = pytest.mark.gpu


class BedParams(C.Structure):
    _fields_ = [("snp_mss_threshold", C.c_double), ("snp_maf_threshold", C.c_double),
                ("snp_I_opt_threshold", C.c_double), ("pat_mss_threshold", C.c_double)]


class BedResult(C.Structure):
    _fields_ = [("n_snp", C.c_int), ("n_fam", C.c_int), ("n_snp_retain", C.c_int), ("n_pat_retain", C.c_int),
                ("n_allele", C.c_int), ("row_bytes", C.c_longlong),
                ("snp_from_retain", C.POINTER(C.c_int)), ("pat_from_retain", C.POINTER(C.c_int)),
                ("allele_orig_from_sort", C.POINTER(C.c_int)),
                ("allele_frequency", C.POINTER(C.c_double)), ("allele_maf", C.POINTER(C.c_double)),
                ("allele_mss", C.POINTER(C.c_double)), ("allele_I_opt", C.POINTER(C.c_double)),
                ("A_n", C.POINTER(C.c_ubyte))]


@pytest.fixture(scope="module")
def golden():
    return bd.load_golden()


@pytest.mark.parametrize("name", list(bd.BED_CASES))
def test_gpu_bed_to_b16_equals_reference(gpu_lib, golden, tmp_path, name):
    lib = bc.bind_solve(gpu_lib)
    bd.write_case(name, str(tmp_path / "in"))
    (tmp_path / "out").mkdir()
    p = tmp_path / "run.in"
    p.write_text(bd.in_text(name, str(tmp_path / "in"), str(tmp_path / "out")))
    assert lib.lakgb_bcc_run_in_file(str(p).encode()) == 0
    got = bd.read_outputs(name, str(tmp_path / "out"))
    for k in ("b16", "bim", "fam"):
        assert got[k] == golden[name][k], (name, k)


def test_gpu_bed_mem_equals_oracle_on_a_larger_case(gpu_lib):
    lib = gpu_lib
    lib.lakgb_bed_to_b16_mem.argtypes = [C.c_void_p, C.c_int, C.c_int, C.POINTER(BedParams), C.POINTER(BedResult)]
    lib.lakgb_bed_result_free.argtypes = [C.POINTER(BedResult)]
    n_snp, n_fam = 3000, 10001
    thr = (0.05, 0.1, 0.02, 0.1)
    rec = np.ascontiguousarray(bd.pack_bed(bd.genotypes(n_snp, n_fam, 21)))
    prm = BedParams(*thr)
    res = BedResult()
    assert lib.lakgb_bed_to_b16_mem(rec.ctypes.data, n_snp, n_fam, C.byref(prm), C.byref(res)) == 0
    try:
        b16, alleles, keep_p = bd.oracle(rec, n_fam, thr)
        hdr = np.frombuffer(b16[:12], np.int32)
        assert (res.n_pat_retain, res.n_allele) == (hdr[1], hdr[2])
        assert res.n_snp_retain * 3 == res.n_allele and 0 < res.n_snp_retain < n_snp
        assert [res.pat_from_retain[i] for i in range(res.n_pat_retain)] == keep_p
        order = [res.allele_orig_from_sort[a] for a in range(res.n_allele)]
        got_snps = [res.snp_from_retain[o // 3] for o in order]
        assert got_snps == [a[0] for a in alleles]
        n = res.row_bytes * res.n_allele
        A = np.ctypeslib.as_array(res.A_n, shape=(n,)).copy()
        assert A.tobytes() == b16[12:]
        # structure: one allele bit per kept SNP and kept patient, zero padding
        rows = np.unpackbits(A.reshape(res.n_allele, res.row_bytes), axis=1, bitorder="big")
        per_snp = np.zeros((res.n_snp_retain, rows.shape[1]), np.int64)
        for r, o in enumerate(order):
            per_snp[o // 3] += rows[r]
        assert np.all(per_snp[:, :res.n_pat_retain] == 1)
        assert not np.any(rows[:, res.n_pat_retain:])
    finally:
        lib.lakgb_bed_result_free(C.byref(res))


@pytest.mark.parametrize("name", list(bd.MERGE_CASES))
def test_gpu_b16_merge_equals_reference(gpu_lib, tmp_path, name):
    """b16_merge through the reference's .in interface: the merged .b16, .bim
    and .fam byte for byte equal to the reference program's."""
    lib = bc.bind_solve(gpu_lib)
    g = bd.load_merge_golden()[name]
    bd.write_merge_case(name, str(tmp_path / "in"))
    (tmp_path / "out").mkdir()
    p = tmp_path / "merge.in"
    p.write_text(bd.merge_in_text(name, str(tmp_path / "in"), str(tmp_path / "out")))
    assert lib.lakgb_bcc_run_in_file(str(p).encode()) == 0
    got = bd.read_outputs(name, str(tmp_path / "out"))
    for k in ("b16", "bim", "fam"):
        assert got[k] == g[k], (name, k)


def test_gpu_b16_merge_larger_equals_oracle(gpu_lib, tmp_path):
    """Three studies of 3000-4100 patients and 700-1200 alleles against the
    Python restatement (pinned to the reference program above)."""
    rng = np.random.default_rng(77)
    studies = []
    for n_pat, n_all in [(4100, 1200), (3000, 700), (3650, 950)]:
        pats = rng.permutation(5000)[:n_pat]
        fam = ["F%d I%d 0 0 1 2" % (p // 7, p) for p in pats]
        freq = np.sort(rng.integers(1, 200, n_all) / 200.0)
        bim = ["1\trs%d\t0\t%d\tA\tG\tand(orig)\t0.001\t%f\t0.002\t%f" % (a, a, f, min(f, 1 - f))
               for a, f in enumerate(freq)]
        rb = (n_pat + 15) // 16 * 2
        bits = np.zeros((n_all, 8 * rb), np.uint8)
        bits[:, :n_pat] = rng.random((n_all, n_pat)) < 0.3
        studies.append((fam, bim, np.array([16, n_pat, n_all], np.int32).tobytes()
                        + np.packbits(bits, 1, bitorder="big").tobytes()))
    files = []
    for k, (fam, bim, b16) in enumerate(studies):
        base = tmp_path / ("s%d" % k)
        (tmp_path / ("s%d.fam" % k)).write_text("".join(x + "\n" for x in fam))
        (tmp_path / ("s%d.bim" % k)).write_text("".join(x + "\n" for x in bim))
        (tmp_path / ("s%d.b16" % k)).write_bytes(b16)
        files.append(str(base))
    lib = gpu_lib
    arr = lambda ext: (C.c_char_p * 3)(*[(f + ext).encode() for f in files])  # noqa: E731
    out = str(tmp_path / "m")
    lib.lakgb_b16_merge.argtypes = [C.c_int, C.c_void_p, C.c_void_p, C.c_void_p, C.c_char_p, C.c_char_p, C.c_char_p]
    assert lib.lakgb_b16_merge(3, arr(".b16"), arr(".bim"), arr(".fam"), (out + ".b16").encode(),
                               (out + ".bim").encode(), (out + ".fam").encode()) == 0
    want = bd.merge_oracle(studies)
    for k in ("b16", "bim", "fam"):
        assert open(out + "." + k, "rb").read() == want[k], k
