"""bed_to_b16 without a GPU: the numpy restatement in tests/bed_cases.py (the
checker of the GPU conversion) writes exactly the .b16, .bim and .fam files
the reference program wrote for the same synthetic PLINK inputs
(tests/golden/bed_to_b16.npz), and the input generator is reproducible."""
import numpy as np
import pytest

import bed_cases as bd


@pytest.fixture(scope="module")
def golden():
    return bd.load_golden()


@pytest.mark.parametrize("name", list(bd.BED_CASES))
def test_oracle_equals_reference_outputs(golden, tmp_path, name):
    bd.write_case(name, str(tmp_path))
    got = bd.oracle_files(name, str(tmp_path))
    for k in ("b16", "bim", "fam"):
        assert got[k] == golden[name][k], (name, k)


def test_filters_remove_snps_and_patients(golden):
    n_snp, n_fam, _, _ = bd.BED_CASES["bed_1000x512"]
    hdr = np.frombuffer(golden["bed_1000x512"]["b16"][:12], np.int32)
    assert hdr[0] == 16 and 0 < hdr[1] < n_fam and 0 < hdr[2] < 3 * n_snp and hdr[2] % 3 == 0


def test_generator_is_reproducible():
    a = bd.genotypes(50, 33, 7)
    b = bd.genotypes(50, 33, 7)
    assert np.array_equal(a, b) and set(np.unique(a)) <= {0, 1, 2, 3}
    rec = bd.pack_bed(a)
    assert rec.shape == (50, 9)
    for p in range(33):
        assert np.array_equal((rec[:, p // 4] >> (2 * (p % 4))) & 3, a[:, p])


@pytest.mark.parametrize("name", list(bd.MERGE_CASES))
def test_merge_oracle_equals_reference_outputs(name):
    """b16_merge: the Python restatement writes exactly the files the
    reference program wrote for the same studies (tests/golden/b16_merge.npz)."""
    g = bd.load_merge_golden()[name]
    got = bd.merge_oracle(bd.merge_inputs(name))
    for k in ("b16", "bim", "fam"):
        assert got[k] == g[k], (name, k)


def test_merge_keeps_only_common_patients():
    g = bd.load_merge_golden()["merge_3x_ragged"]
    hdr = np.frombuffer(g["b16"][:12], np.int32)
    studies = bd.merge_inputs("merge_3x_ragged")
    common = set.intersection(*[set(tuple(x.split()[:2]) for x in fam) for fam, _, _ in studies])
    assert hdr[1] == len(common) and hdr[2] == sum(len(b) for _, b, _ in studies)
