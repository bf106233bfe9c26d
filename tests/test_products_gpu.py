"""GPU parity of AtTAn_vv, At_T_YnWt_S_Zn_vv, An_ZtSWn_Yt_vv and the bit-plane
An_ZtSWn_Yt_ww: the product library, through the reference's C entry points,
reproduces the reference's outputs bit for bit on the committed fixtures and
the C oracle's on a larger seeded case; the xcalc -> An_ZtSWn_Yt_ww chain
equals the oracle's chain bit for bit and the element-wise product to the
quantisation error."""
import numpy as np
import pytest

import product_cases as pc
import ztswn_chain as zc

pytestmark = pytest.mark.gpu

CASES = pc.load_golden()


def _bits_equal(a, b):
    return a.shape == b.shape and np.array_equal(a.view(np.uint64), b.view(np.uint64))


@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_reference_products(gpu_lib, name):
    ins, outs = CASES[name]
    h = pc.handles(ins)
    for kind, sa, sb in pc.keys():
        got = pc.run("gpu", kind, h, sa, sb)
        assert _bits_equal(got, outs[pc.key_name(kind, sa, sb)]), (name, kind, sa, sb)


def test_gpu_matches_oracle_products_larger(gpu_lib, oracle_lib):
    x = pc.build(dict(name="large", nsnp=300, npat=900, nctl=700, nt=2, masked=True, seed=77))
    h = pc.handles(x)
    for kind, sa, sb in pc.keys():
        want = pc.run("oracle", kind, h, sa, sb)
        got = pc.run("gpu", kind, h, sa, sb)
        assert _bits_equal(got, want), (kind, sa, sb)


def test_gpu_ww_chain(gpu_lib, oracle_lib):
    from test_zz_no_alloc import _bind
    _bind(gpu_lib)
    x = pc.build(zc.spec(seed=93))
    h = pc.handles(x)
    for sa, sb in pc.SPACING_PAIRS:
        want, wp = zc.chain("oracle", x, h, sa, sb)
        got, gp = zc.chain("gpu", x, h, sa, sb)
        for a, b in zip(gp, wp):
            assert (a.s.nrows, a.s.min_d, a.s.mlt_d) == (b.s.nrows, b.s.min_d, b.s.mlt_d)
            assert np.array_equal(a.wX, b.wX)
        assert _bits_equal(got, want), (sa, sb)
        vv = pc.run("gpu", "An_ZtSWn_Yt_vv", h, sa, sb)
        assert zc.rel_err(got, vv) < 1e-6
    assert gpu_lib.lakgb_device_status() == 0
