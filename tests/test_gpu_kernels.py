"""GPU parity: the product library, called through the reference's C entry
points, reproduces the reference's kernel outputs bit for bit (committed
fixtures) and agrees with the C oracle on larger seeded inputs."""
import numpy as np
import pytest

import golden_cases as gc
import kernel_cases as kc
from lakcluster_c_gb300 import abi

pytestmark = pytest.mark.gpu

FIXTURES = gc.load_gram_fixtures()


def _bits_equal(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.mark.parametrize("fx", FIXTURES, ids=[f.name for f in FIXTURES])
def test_gpu_matches_reference_fixtures(gpu_lib, fx):
    for key in gc.all_keys(fx):
        got = gc.run_key("gpu", fx, key)
        assert _bits_equal(got, fx.expected(key)), (fx.name, key)


@pytest.mark.parametrize("nA,nZ,m,sym", [(513, 389, 17280, False), (700, 700, 9000, True),
                                          (1024, 1024, 1024, True), (257, 1000, 40000, False)])
def test_gpu_matches_oracle_larger(gpu_lib, oracle_lib, nA, nZ, m, sym):
    rng = np.random.default_rng(nA * 7 + m)
    A, ar_b, ar_j = kc.make_matrix_case(rng, nA, m, 0.97, 0.9)
    Z, zr_b, zr_j = (A, ar_b, ar_j) if sym else kc.make_matrix_case(rng, nZ, m, 0.97, 0.9)
    mc_b = (rng.random(m) < 0.98).astype(np.uint8)
    mc_j = mc_b & (rng.random(m) < 0.9).astype(np.uint8)
    MA = kc.mhandle(A, ar_b, ar_j, mc_b, mc_j)
    MZ = MA if sym else kc.mhandle(Z, zr_b, zr_j, mc_b, mc_j)
    A_p = 0.05 + 0.9 * rng.random(abi.psize(m))
    A_ajdk = abi.calc_A_ajdk(A_p)
    vA = kc.call_an_ajdk("oracle", abi.TYPE_pm, abi.SPACING_a, MA, A_ajdk)
    assert _bits_equal(kc.call_an_ajdk("gpu", abi.TYPE_pm, abi.SPACING_a, MA, A_ajdk), vA)
    vZ = vA if sym else kc.call_an_ajdk("oracle", abi.TYPE_pm, abi.SPACING_a, MZ, A_ajdk)
    lfA = kc.lhandle_from(vA, MA.nrows, abi.AJDK_TOT, abi.SPACING_a)
    lfZ = lfA if sym else kc.lhandle_from(vZ, MZ.nrows, abi.AJDK_TOT, abi.SPACING_a)
    for t in (abi.TYPE_pm, abi.TYPE_00):
        want = kc.call_gram("oracle", sym, t, abi.SPACING_b, abi.SPACING_j, MA, MZ, A_ajdk, lfA, lfZ)
        got = kc.call_gram("gpu", sym, t, abi.SPACING_b, abi.SPACING_j, MA, MZ, A_ajdk, lfA, lfZ)
        assert _bits_equal(got, want)


@pytest.mark.parametrize("n,frac", [(21001, 1.0), (23000, 0.9)])
def test_an_ajdk_two_rows_per_warp(gpu_lib, oracle_lib, n, frac):
    """Launches of 16384 rows or more take two rows per warp; an odd row count
    (21001 rows, all retained) leaves the last warp with one row."""
    rng = np.random.default_rng(n)
    A, r_b, r_j = kc.make_matrix_case(rng, n, 2500, frac, frac)
    assert int(r_j.sum()) >= 16384
    mc_b = (rng.random(2500) < 0.95).astype(np.uint8)
    mc_j = mc_b & (rng.random(2500) < 0.9).astype(np.uint8)
    MA = kc.mhandle(A, r_b, r_j, mc_b, mc_j)
    A_ajdk = abi.calc_A_ajdk(0.05 + 0.9 * rng.random(abi.psize(2500)))
    for t in (abi.TYPE_pm, abi.TYPE_00):
        for sp in (abi.SPACING_a, abi.SPACING_j):
            want = kc.call_an_ajdk("oracle", t, sp, MA, A_ajdk)
            assert _bits_equal(kc.call_an_ajdk("gpu", t, sp, MA, A_ajdk), want), (t, sp)
