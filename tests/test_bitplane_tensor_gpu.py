"""GPU parity of the two bit-plane kernels (wrap_At_T_YnWt_S_Zn_ww__run): the
tcgen05 kernel and the CUDA-core kernel give identical whole-solve outputs
(trace and elimination order) for B_MLT = 8, 16 and 32, every tensor-core
wait ends in time, and with either kernel the golden cases still match the
reference.  (The other GPU tests run the default, the tensor-core kernel.)"""
import numpy as np
import pytest

import bcc_cases as bc
from lakcluster_c_gb300 import solve as sv

pytestmark = pytest.mark.gpu

POPCOUNT, TENSOR = 0, 1


@pytest.fixture
def lib(gpu_lib):
    lib = bc.bind_solve(gpu_lib)
    before = (lib.lakgb_bitplane_impl(), lib.lakgb_gram_impl())
    yield lib
    lib.lakgb_set_bitplane_impl(before[0])
    lib.lakgb_set_gram_impl(before[1])


def _solve(lib, d, B_MLT):
    p = sv.Problem(d["A"], d.get("Z"), gamma=d["gamma"], gamma_type=d.get("gamma_type") or 0,
                   A_masks=d.get("A_masks"), Z_masks=d.get("Z_masks"), col_mask=d.get("col_mask"),
                   B_MLT=B_MLT, lib=lib)
    return p.solve()


@pytest.mark.parametrize("name", ["case_control_2bin_300x250x2100", "case_control_3bin_ragged",
                                  "case_control_2bin_masked"])
@pytest.mark.parametrize("B_MLT", [8, 16, 32])
def test_tensor_bitplane_matches_popcount(lib, name, B_MLT):
    d = bc.build(name)
    outs = {}
    for impl in (POPCOUNT, TENSOR):
        lib.lakgb_set_bitplane_impl(impl)
        outs[impl] = _solve(lib, d, B_MLT)
        assert lib.lakgb_device_status() == 0
    for key in ("trace", "xdrop_a", "xdrop_b"):
        assert outs[TENSOR][key] == outs[POPCOUNT][key], key


@pytest.mark.parametrize("name", bc.SMALL)
def test_popcount_kernels_still_match_reference(lib, name):
    """Both CUDA-core kernels (Gram and bit-plane) against the golden traces."""
    golden = bc.load_golden()
    lib.lakgb_set_bitplane_impl(POPCOUNT)
    lib.lakgb_set_gram_impl(POPCOUNT)
    got = bc.solve_in_memory(lib, name)
    for key in ("trace", "xdrop_a", "xdrop_b"):
        assert got[key] == golden[name][key], key


def test_tensor_bitplane_large_case(lib):
    """A case with more SNP pairs than one 128-row tile per covariate column,
    several N tiles and a two-block patient dimension."""
    rng = np.random.default_rng(5)
    A = [(rng.random((2100, 700)) < 0.3).astype(np.uint8)]
    Z = [(rng.random((1900, 700)) < 0.3).astype(np.uint8)]
    d = dict(A=A, Z=Z, gamma=0.2)
    outs = {}
    for impl in (POPCOUNT, TENSOR):
        lib.lakgb_set_bitplane_impl(impl)
        outs[impl] = _solve(lib, d, 32)
        assert lib.lakgb_device_status() == 0
    assert outs[TENSOR] == outs[POPCOUNT]
