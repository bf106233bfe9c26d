"""The synthetic workload generators behind the many-solve measurements.

The packed generators must write rows in the layout solve.pack_rows writes
(MSB first, rows padded to 16 bits), be reproducible from their seed, and
draw the sizes, bins and planted bicluster their docstrings state.
"""
import numpy as np
import pytest

from lakcluster_c_gb300 import synth
from lakcluster_c_gb300.solve import pack_rows


def _unpack(rows, ncols):
    return np.unpackbits(rows, axis=1, bitorder="big")[:, :ncols]


def test_packed_rows_match_pack_rows_of_the_same_draws():
    f = 0.05 + 0.45 * np.random.default_rng(1).random(37)
    got = synth._packed_bernoulli_rows(np.random.default_rng(3), 50, f, chunk=16)
    r = np.random.default_rng(3)
    bits = np.concatenate([(r.random((min(16, 50 - i), 37), dtype=np.float32) < f.astype(np.float32)[None])
                           for i in range(0, 50, 16)]).astype(np.uint8)
    assert np.array_equal(got, pack_rows(bits))


def test_served_request_packed_shapes_and_planted_block():
    a = synth.served_request_packed(5003, rows=(512, 2048), cols=(2048, 4096))
    b = synth.served_request_packed(5003, rows=(512, 2048), cols=(2048, 4096))
    assert a.ncols == b.ncols and a.nbins == b.nbins and 1 <= a.nbins <= 3
    for x, y in zip(a.A_bins + a.Z_bins, b.A_bins + b.Z_bins):
        assert np.array_equal(x, y)
        assert x.shape[1] == (a.ncols + 15) // 16 * 2
        assert not np.any(_unpack(x, x.shape[1] * 8)[:, a.ncols:])   # padding bits are zero
    assert len(a.planted_rows) >= 2 and len(a.planted_cols) == max(2, a.ncols // 32)


def test_null_instance_packed_is_reproducible_on_cpu():
    pytest.importorskip("torch")
    a = synth.null_instance_packed(1007, rows=(256, 512), cols=(1024, 2048), device="cpu")
    b = synth.null_instance_packed(1007, rows=(256, 512), cols=(1024, 2048), device="cpu")
    assert a.nbins == 1 and np.array_equal(a.A_bins[0], b.A_bins[0]) and np.array_equal(a.Z_bins[0], b.Z_bins[0])
    r = a.A_bins[0].shape[0] + a.Z_bins[0].shape[0]
    assert 256 <= r <= 512 and 1024 <= a.ncols <= 2048
    assert a.A_bins[0].shape[0] == r // 2
    X = np.concatenate([_unpack(a.A_bins[0], a.ncols), _unpack(a.Z_bins[0], a.ncols)])
    m = X.mean()
    assert 0.2 < m < 0.35   # MAF U[0.05, 0.5] has mean 0.275
