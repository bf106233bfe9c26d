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


@pytest.mark.parametrize("key", list(bc.DCC_SCOREBOX))
def test_gpu_dcc_scorebox_equals_reference(solve_lib, tmp_path, key):
    import numpy as np
    golden, (sb, _) = bc.load_dcc_golden(), bc.load_dcc_extra_golden()
    name, grid = bc.DCC_SCOREBOX[key]
    p = bc.write_scorebox_case(key, golden[name]["xdrop_a"], str(tmp_path / "in"), str(tmp_path / "out"))
    assert solve_lib.lakgb_bcc_run_in_file(p.encode()) == 0
    got = bc.read_scorebox(str(tmp_path / "out"), grid)
    for a in bc.SCOREBOX_ARRAYS:
        assert np.array_equal(got[a].view(np.uint8), sb[key][a].view(np.uint8)), (key, a)


@pytest.mark.parametrize("key", list(bc.DCC_SCRAMBLE))
def test_gpu_dcc_scramble_equals_reference(solve_lib, tmp_path, key):
    golden, (_, scr) = bc.load_dcc_golden(), bc.load_dcc_extra_golden()
    name, _ = bc.DCC_SCRAMBLE[key]
    p = bc.write_scramble_case(key, golden[name]["xdrop_a"], str(tmp_path / "in"), str(tmp_path / "out"))
    assert solve_lib.lakgb_bcc_run_in_file(p.encode()) == 0
    got = bc.read_outputs(str(tmp_path / "out"))
    for k in ("trace", "xdrop_a", "xdrop_b"):
        assert got[k] == scr[key][k], (key, k)
    assert bc.b16_digests(str(tmp_path / "out")) == scr[key]["b16_sha1"]
