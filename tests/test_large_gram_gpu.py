"""The large-configuration Gram pass machinery (operands drawn on the device,
3 bins) at a reduced size: every product identical with both Gram kernels,
sampled entries equal to the host recomputation in block order."""
import pytest

pytestmark = pytest.mark.gpu


def test_large_pass_reduced(gpu_lib):
    from lakcluster_c_gb300.large_pass import LargeGramPass
    lp = LargeGramPass(n_cases=3000, n_controls=2600, ncols=20000, nbins=3, planted=(256, 512), seed=9)
    r = lp.run_checks(samples_per_product=6)
    assert r["products"] == 15
    assert r["tensor_equals_popcount"] == r["products"]
    assert r["sampled_equal_host"] == r["sampled_entries"] == 90
    assert r["device_status"] == 0
