"""The reference's own consistency check of the bit-plane loop product
(dir_c/An_ZtSWn_Yt_ww.c:380-391), on the C oracle: ZtSWn slices quantised by
xcalc into 32 bit planes and evaluated by An_ZtSWn_Yt_ww agree with the
element-wise FP64 An_ZtSWn_Yt_vv to the quantisation error (relative 1e-6;
about 2e-8 is typical), for every output spacing."""
import pytest

import product_cases as pc
import ztswn_chain as zc

TOL = 1e-6


@pytest.mark.parametrize("sa,sb", pc.SPACING_PAIRS)
def test_oracle_ww_chain_matches_vv(oracle_lib, sa, sb):
    x = pc.build(zc.spec())
    h = pc.handles(x)
    ww, _ = zc.chain("oracle", x, h, sa, sb)
    vv = pc.run("oracle", "An_ZtSWn_Yt_vv", h, sa, sb)
    assert ww.shape == vv.shape
    assert zc.rel_err(ww, vv) < TOL
