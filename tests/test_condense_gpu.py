"""The condense row strategy's kernels on the GPU (lakcluster_c_gb300/csrc/
condense.cu) against the C oracle, bit for bit: M_At_to_L2 / M_An_to_L2 over
ragged sizes, partial masks, both value types, every spacing, with and
without A_ajdk (and into a caller-owned handle longer than the product, which
is zeroed whole); AnZt_mm over tile edges, K = 0 and a Zt with more rows per
column than At.  The whole condense solve is covered by
tests/test_bcc_solve_gpu.py against the reference program's goldens."""
import numpy as np
import pytest

import kernel_cases as kc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("at", [True, False])
@pytest.mark.parametrize("spec", kc.to_l2_specs(), ids=lambda s: s["name"])
def test_gpu_to_l2_equals_oracle(gpu_lib, spec, at):
    M, A_ajdk = kc.build_to_l2(spec, at)
    want, _ = kc.call_m_to_l2("oracle", at, spec["type"], spec["sr"], spec["sc"], M, A_ajdk)
    got, _ = kc.call_m_to_l2("gpu", at, spec["type"], spec["sr"], spec["sc"], M, A_ajdk)
    assert got.tobytes() == want.tobytes()


def test_gpu_to_l2_zeroes_the_whole_handle(gpu_lib):
    spec = kc.to_l2_specs()[4]
    M, A_ajdk = kc.build_to_l2(spec)
    n = kc.call_m_to_l2("oracle", True, spec["type"], spec["sr"], spec["sc"], M, A_ajdk)[0].size
    want, _ = kc.call_m_to_l2("oracle", True, spec["type"], spec["sr"], spec["sc"], M, A_ajdk, out_length=n + 50)
    got, _ = kc.call_m_to_l2("gpu", True, spec["type"], spec["sr"], spec["sc"], M, A_ajdk, out_length=n + 50)
    assert got.tobytes() == want.tobytes() and not np.any(got[n:])


@pytest.mark.parametrize("K,m,n,extra", kc.mm_specs())
def test_gpu_anzt_mm_equals_oracle(gpu_lib, K, m, n, extra):
    A, B, lfA, lfZ = kc.build_mm(K, m, n, extra, seed=K * 7 + m)
    want = kc.call_anzt_mm("oracle", lfA, lfZ)
    got = kc.call_anzt_mm("gpu", lfA, lfZ)
    assert got.size == m * n and got.tobytes() == want.tobytes()


def test_gpu_anzt_mm_large(gpu_lib):
    """A removed-column block of a large bin: 700 SNPs x 3000 x 2500 rows."""
    A, B, lfA, lfZ = kc.build_mm(700, 3000, 2500, 0, seed=5)
    got = kc.call_anzt_mm("gpu", lfA, lfZ)
    want = kc.call_anzt_mm("oracle", lfA, lfZ)
    assert got.tobytes() == want.tobytes()
