"""The .b16 transpose oracle (lako_bits_transpose, a restatement of
dir_c/binary_read.c:174-269) against the reference's own outputs: the
committed golden files made by the reference's wrap_transpose, and, where
the reference builds here, fresh random cases run through it."""
import os

import numpy as np
import pytest

import kernel_cases as kc
import transpose_cases as tc
from lakcluster_c_gb300 import infiles


def _golden():
    d = np.load(tc.GOLDEN)
    return [(d["case%02d/in" % i].tobytes(), d["case%02d/out" % i].tobytes()) for i in range(len(tc.SHAPES))]


def test_oracle_matches_reference_golden(tmp_path):
    for i, (raw, want) in enumerate(_golden()):
        assert tc.oracle_transpose(raw) == want, tc.SHAPES[i]
        # and the golden input is the case generator's file
        assert tc.write_file(str(tmp_path / ("c%d.b16" % i)), tc.matrix(i, tc.SHAPES[i])) == raw


def test_transpose_is_the_matrix_transpose(tmp_path):
    for i, (raw, want) in enumerate(_golden()):
        n, m, _ = tc.SHAPES[i]
        p_in, p_out = str(tmp_path / "a.b16"), str(tmp_path / "b.b16")
        open(p_in, "wb").write(raw)
        open(p_out, "wb").write(want)
        x, y = infiles.read_b16(p_in), infiles.read_b16(p_out)
        assert x.shape == (n, m) and y.shape == (m, n)
        assert np.array_equal(y, x.T), tc.SHAPES[i]
        bitj, n_col, n_row = tc.header(want)
        assert (bitj, n_col, n_row) == (16, n, m)


@pytest.mark.skipif(not os.path.exists(kc.REF_LIB), reason="reference not built here (x86-64 with its sources)")
def test_oracle_matches_reference_fresh_cases(tmp_path):
    rng = np.random.default_rng(31)
    for k in range(6):
        n, m = int(rng.integers(1, 700)), int(rng.integers(1, 700))
        x = (rng.random((n, m)) < rng.random()).astype(np.uint8)
        src = str(tmp_path / ("r%d.b16" % k))
        raw = tc.write_file(src, x)
        want = tc.file_transpose("ref", src, str(tmp_path / ("r%d_t.b16" % k)), int(rng.choice([8, 64, 4096])))
        assert tc.oracle_transpose(raw) == want, (n, m)
