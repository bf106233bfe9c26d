"""GPU parity of AtTAn_vv, At_T_YnWt_S_Zn_vv and An_ZtSWn_Yt_vv: the product
library, through the reference's C entry points, reproduces the reference's
outputs bit for bit on the committed fixtures and the C oracle's on a larger
seeded case."""
import numpy as np
import pytest

import product_cases as pc

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
