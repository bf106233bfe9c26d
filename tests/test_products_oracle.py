"""The C restatement of AtTAn_vv, At_T_YnWt_S_Zn_vv and An_ZtSWn_Yt_vv
(oracle/lak_oracle.c) reproduces the reference's own outputs bit for bit on
every committed fixture (tests/golden/kernels_products.npz)."""
import numpy as np
import pytest

import product_cases as pc

CASES = pc.load_golden()


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_reference_products(oracle_lib, name):
    ins, outs = CASES[name]
    h = pc.handles(ins)
    for kind, sa, sb in pc.keys():
        want = outs[pc.key_name(kind, sa, sb)]
        got = pc.run("oracle", kind, h, sa, sb)
        assert got.shape == want.shape, (kind, sa, sb)
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), (name, kind, sa, sb)


def test_product_fixture_coverage():
    kinds = {k.split("/")[0] for _, outs in CASES.values() for k in outs}
    assert kinds == set(pc.KINDS)
    assert len(CASES) == len(pc.specs())
