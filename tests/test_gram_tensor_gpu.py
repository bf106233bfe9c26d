"""GPU parity of the Gram kernels: the tcgen05 tensor-core kernel, the
popcount kernel and the popcount kernel split over blocks give bit-identical
outputs to each other and to the C oracle
(AnZt_vv / AnAt_vv, both types), including partial tiles, full blocks
(counts of 1920), fully masked blocks and unweighted (D = NULL) calls, and the
tensor-core kernels' device status word stays 0."""
import ctypes as C

import numpy as np
import pytest

import kernel_cases as kc
from lakcluster_c_gb300 import abi

pytestmark = pytest.mark.gpu

POPCOUNT, TENSOR, SPLIT = 0, 1, 3


def _bits_equal(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.fixture
def impl_switch(gpu_lib):
    gpu_lib.lakgb_set_gram_impl.argtypes = [C.c_int]
    gpu_lib.lakgb_gram_impl.restype = C.c_int
    gpu_lib.lakgb_device_status.restype = C.c_int
    before = gpu_lib.lakgb_gram_impl()
    yield gpu_lib
    gpu_lib.lakgb_set_gram_impl(before)


def _case(rng, nA, nZ, m, sym, density=0.5, mask_keep=0.9, dead_blocks=()):
    A, ar_b, ar_j = kc.make_matrix_case(rng, nA, m, 0.97, 0.9)
    if density != 0.5:
        A = (rng.random(A.shape) < density).astype(np.uint8)
    Z, zr_b, zr_j = (A, ar_b, ar_j) if sym else kc.make_matrix_case(rng, nZ, m, 0.97, 0.9)
    if density != 0.5 and not sym:
        Z = (rng.random(Z.shape) < density).astype(np.uint8)
    mc_b = (rng.random(m) < 0.98).astype(np.uint8)
    mc_j = mc_b & (rng.random(m) < mask_keep).astype(np.uint8)
    for blk in dead_blocks:
        mc_j[blk * 1920:(blk + 1) * 1920] = 0
    MA = kc.mhandle(A, ar_b, ar_j, mc_b, mc_j)
    MZ = MA if sym else kc.mhandle(Z, zr_b, zr_j, mc_b, mc_j)
    return MA, MZ


def _run_both(lib, sym, t, MA, MZ, A_ajdk, lfA, lfZ):
    outs = {}
    for impl in (POPCOUNT, TENSOR, SPLIT):
        lib.lakgb_set_gram_impl(impl)
        outs[impl] = kc.call_gram("gpu", sym, t, abi.SPACING_b, abi.SPACING_j, MA, MZ, A_ajdk, lfA, lfZ)
        assert lib.lakgb_device_status() == 0
    return outs


@pytest.mark.parametrize("nA,nZ,m,sym", [(1, 1, 2000, False), (129, 255, 3840, False), (300, 300, 5000, True),
                                          (128, 128, 1920, False), (640, 384, 9600, False),
                                          (200, 200, 21000, True)])
def test_tensor_matches_popcount_and_oracle(impl_switch, oracle_lib, nA, nZ, m, sym):
    rng = np.random.default_rng(nA * 13 + nZ + m)
    MA, MZ = _case(rng, nA, nZ, m, sym)
    A_p = 0.05 + 0.9 * rng.random(abi.psize(m))
    A_ajdk = abi.calc_A_ajdk(A_p)
    vA = kc.call_an_ajdk("oracle", abi.TYPE_pm, abi.SPACING_a, MA, A_ajdk)
    vZ = vA if sym else kc.call_an_ajdk("oracle", abi.TYPE_pm, abi.SPACING_a, MZ, A_ajdk)
    lfA = kc.lhandle_from(vA, MA.nrows, abi.AJDK_TOT, abi.SPACING_a)
    lfZ = lfA if sym else kc.lhandle_from(vZ, MZ.nrows, abi.AJDK_TOT, abi.SPACING_a)
    for t in (abi.TYPE_pm, abi.TYPE_00):
        for lf in ((lfA, lfZ), (None, None)):
            want = kc.call_gram("oracle", sym, t, abi.SPACING_b, abi.SPACING_j, MA, MZ, A_ajdk, *lf)
            outs = _run_both(impl_switch, sym, t, MA, MZ, A_ajdk, *lf)
            assert _bits_equal(outs[TENSOR], outs[POPCOUNT]), (t, lf[0] is None)
            assert _bits_equal(outs[SPLIT], outs[POPCOUNT]), (t, lf[0] is None)
            assert _bits_equal(outs[TENSOR], want), (t, lf[0] is None)


@pytest.mark.parametrize("density,mask_keep,dead", [(1.0, 1.0, ()), (0.0, 1.0, ()), (0.5, 0.9, (0, 2)),
                                                    (0.95, 0.3, (1,))])
def test_tensor_extreme_counts(impl_switch, oracle_lib, density, mask_keep, dead):
    """All-ones rows (a block count of 1920 in the accumulator), all-zero rows,
    fully masked blocks, sparse masks; unweighted (D = NULL) and weighted."""
    rng = np.random.default_rng(int(density * 100) + len(dead))
    m = 4 * 1920
    MA, MZ = _case(rng, 190, 140, m, False, density=density, mask_keep=mask_keep, dead_blocks=dead)
    A_ajdk = abi.calc_A_ajdk(0.05 + 0.9 * rng.random(abi.psize(m)))
    for aj in (A_ajdk, None):
        for t in (abi.TYPE_pm, abi.TYPE_00):
            want = kc.call_gram("oracle", False, t, abi.SPACING_b, abi.SPACING_j, MA, MZ, aj, None, None)
            outs = _run_both(impl_switch, False, t, MA, MZ, aj, None, None)
            assert _bits_equal(outs[TENSOR], want), (t, aj is None)
            assert _bits_equal(outs[POPCOUNT], want), (t, aj is None)
            assert _bits_equal(outs[SPLIT], want), (t, aj is None)


def test_host_buffer_rewritten_in_place(impl_switch, oracle_lib):
    """A wX buffer rewritten in place (same address, same size) between two
    reference-API calls is read afresh: no stale device copy by default."""
    rng = np.random.default_rng(77)
    m = 2 * 1920
    MA, MZ = _case(rng, 150, 130, m, False)
    A_ajdk = abi.calc_A_ajdk(0.05 + 0.9 * rng.random(abi.psize(m)))
    for impl in (TENSOR, POPCOUNT, SPLIT):
        impl_switch.lakgb_set_gram_impl(impl)
        first = kc.call_gram("gpu", False, abi.TYPE_pm, abi.SPACING_b, abi.SPACING_j, MA, MZ, A_ajdk, None, None)
        MA.wX[:] = rng.integers(0, 256, MA.wX.shape, dtype=np.uint8)
        want = kc.call_gram("oracle", False, abi.TYPE_pm, abi.SPACING_b, abi.SPACING_j, MA, MZ, A_ajdk, None, None)
        got = kc.call_gram("gpu", False, abi.TYPE_pm, abi.SPACING_b, abi.SPACING_j, MA, MZ, A_ajdk, None, None)
        assert not _bits_equal(first, want)
        assert _bits_equal(got, want), impl


def test_autotuned_dispatch_matches_oracle(impl_switch, oracle_lib):
    """LAKGB_GRAM_AUTO: the first launch of a shape class times every
    candidate; results equal the oracle's before and after the class is
    tuned, and the table records a choice with a time per candidate."""
    import json
    lib = impl_switch
    lib.lakgb_set_gram_impl(2)
    lib.lakgb_gram_autotune_reset()
    rng = np.random.default_rng(4242)
    MA, MZ = _case(rng, 333, 222, 4000, False)
    A_ajdk = abi.calc_A_ajdk(0.05 + 0.9 * rng.random(abi.psize(4000)))
    want = kc.call_gram("oracle", False, abi.TYPE_pm, abi.SPACING_b, abi.SPACING_j, MA, MZ, A_ajdk, None, None)
    for _ in range(2):
        got = kc.call_gram("gpu", False, abi.TYPE_pm, abi.SPACING_b, abi.SPACING_j, MA, MZ, A_ajdk, None, None)
        assert _bits_equal(got, want)
        assert lib.lakgb_device_status() == 0
    buf = C.create_string_buffer(1 << 14)
    lib.lakgb_gram_autotune_table(buf, len(buf))
    table = json.loads(buf.value.decode())
    assert len(table) == 1
    assert table[0]["choice"] in table[0]["ms"] and len(table[0]["ms"]) == 5


@pytest.mark.parametrize("sa,sb", [(abi.SPACING_b, abi.SPACING_b), (abi.SPACING_j, abi.SPACING_j),
                                   (abi.SPACING_a, abi.SPACING_b), (abi.SPACING_b, abi.SPACING_a)])
def test_large_host_output_two_part_download(impl_switch, oracle_lib, sa, sb):
    """Host outputs of 8 MB or more of a non-symmetric Gram come back in two
    parts (two launches over halves of the Z rows, the first half's columns
    downloaded while the second computes): same values as the oracle for
    every output spacing, with masked rows and columns."""
    rng = np.random.default_rng(9000 + sa * 3 + sb)
    MA, MZ = _case(rng, 1250, 1150, 3 * 1920 + 77, False)
    A_ajdk = abi.calc_A_ajdk(0.05 + 0.9 * rng.random(abi.psize(3 * 1920 + 77)))
    vA = kc.call_an_ajdk("oracle", abi.TYPE_pm, abi.SPACING_a, MA, A_ajdk)
    vZ = kc.call_an_ajdk("oracle", abi.TYPE_pm, abi.SPACING_a, MZ, A_ajdk)
    lfA = kc.lhandle_from(vA, MA.nrows, abi.AJDK_TOT, abi.SPACING_a)
    lfZ = kc.lhandle_from(vZ, MZ.nrows, abi.AJDK_TOT, abi.SPACING_a)
    want = kc.call_gram("oracle", False, abi.TYPE_pm, sa, sb, MA, MZ, A_ajdk, lfA, lfZ)
    assert want.size * 8 >= 8 << 20  # large enough for the two-part download
    for impl in (TENSOR, 2):
        impl_switch.lakgb_set_gram_impl(impl)
        got = kc.call_gram("gpu", False, abi.TYPE_pm, sa, sb, MA, MZ, A_ajdk, lfA, lfZ)
        assert _bits_equal(got, want), impl
        assert impl_switch.lakgb_device_status() == 0
