"""Dexcluster (GLOBAL_TEST_TYPE dexcluster_driver) through the GPU library's
.in-file entry point: the out_trace / out_xdrop_a / out_xdrop_b lines equal the
reference program's (tests/golden/dcc_traces.npz) on every dexcluster case."""
import pytest

import bcc_cases as bc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def solve_lib(gpu_lib):
    return bc.bind_solve(gpu_lib)


@pytest.mark.parametrize("name", bc.DCC_CASES)
def test_gpu_dcc_equals_reference(solve_lib, tmp_path, name):
    golden = bc.load_dcc_golden()
    p = bc.write_dcc_case(name, str(tmp_path / "in"), str(tmp_path / "out"))
    assert solve_lib.lakgb_bcc_run_in_file(p.encode()) == 0
    got = bc.read_outputs(str(tmp_path / "out"))
    for k in ("trace", "xdrop_a", "xdrop_b"):
        assert got[k] == golden[name][k], (name, k)
