"""wrap_An_ZtSn_ww__run on the GPU (the masked-AND Gram of the An rows
against the bit planes, then the reference's FP64 combination,
lakcluster_c_gb300/csrc/bitplane.cu) against the C oracle's restatement of
dir_c/An_ZtSn_ww.c:5-108, bit for bit: partial row and column masks, one to
three covariate columns, B_MLT 8 / 16 / 32, every spacing, and row counts
from one to a few thousand (the Gram's small-launch and tensor paths)."""
import ctypes as C

import numpy as np
import pytest

import kernel_cases as kc
from lakcluster_c_gb300 import abi
from lakcluster_c_gb300.abi import L_handle

pytestmark = pytest.mark.gpu

CASES = [  # (rows, SNPs, B_MLT, covariates, masked, spacing_a, spacing_s, seed)
    (1, 1921, 8, 1, False, abi.SPACING_a, abi.SPACING_a, 1),
    (37, 4000, 16, 2, True, abi.SPACING_j, abi.SPACING_b, 2),
    (300, 2000, 32, 1, True, abi.SPACING_b, abi.SPACING_j, 3),
    (1031, 5777, 32, 3, True, abi.SPACING_a, abi.SPACING_a, 4),
    (3000, 16384, 32, 1, False, abi.SPACING_a, abi.SPACING_a, 5),
]


def _call(backend, sa, ss, An, Z, St):
    lib = kc.load_backend(backend)
    out = C.POINTER(L_handle)()
    if backend == "oracle":
        n = lib.lako_An_ZtSn_ww(sa, ss, An.ptr, Z.ptr, St.ptr, C.byref(out))
    else:
        n = lib.wrap_An_ZtSn_ww__run(*kc._thread_args(), sa, ss, An.ptr, None, Z.ptr, St.ptr, C.byref(out))
    return kc._take(out, n)


@pytest.mark.parametrize("n,m,B,nS,masked,sa,ss,seed", CASES)
def test_gpu_an_ztsn_equals_oracle(gpu_lib, n, m, B, nS, masked, sa, ss, seed):
    rng = np.random.default_rng(seed)
    frac = 0.8 if masked else 1.0
    rows, mr_b, mr_j = kc.make_matrix_case(rng, n, m, frac, frac)
    mc_b = (rng.random(m) < frac).astype(np.uint8)
    mc_j = mc_b & (rng.random(m) < frac).astype(np.uint8)
    An = kc.mhandle(rows, mr_b, mr_j, mc_b, mc_j)
    Z = abi.MHandle(kc.random_bits(rng, (nS * (B + 1), m), 0.5))
    Z.s.ncols_per_z, Z.s.min_d, Z.s.mlt_d = B + 1, -2.5 + rng.random(), float(2 ** B) / (3.0 + rng.random())
    St = abi.MHandle(np.ones((nS, 16), np.uint8))
    want = _call("oracle", sa, ss, An, Z, St)
    got = _call("gpu", sa, ss, An, Z, St)
    assert got.size == want.size and got.tobytes() == want.tobytes()
