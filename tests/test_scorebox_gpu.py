"""Scorebox and scramble runs through the GPU library's .in-file entry point
(lakgb_bcc_run_in_file), against the reference program's own outputs in
tests/golden/bcc_scorebox.npz: the scorebox grid arrays bit for bit (both
loop orders), and the scrambled solves' traces, elimination orders and
.b16 snapshots."""
import numpy as np
import pytest

import bcc_cases as bc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def solve_lib(gpu_lib):
    return bc.bind_solve(gpu_lib)


@pytest.fixture(scope="module")
def goldens():
    return bc.load_golden(), bc.load_scorebox_golden()


@pytest.mark.parametrize("key", list(bc.SCOREBOX))
def test_gpu_scorebox_equals_reference(solve_lib, goldens, tmp_path, key):
    golden, (sb, _) = goldens
    name, grid = bc.SCOREBOX[key]
    p = bc.write_scorebox_case(key, golden[name]["xdrop_a"], str(tmp_path / "in"), str(tmp_path / "out"))
    assert solve_lib.lakgb_bcc_run_in_file(p.encode()) == 0
    got = bc.read_scorebox(str(tmp_path / "out"), grid)
    for a in bc.SCOREBOX_ARRAYS:
        assert np.array_equal(got[a].view(np.uint8), sb[key][a].view(np.uint8)), (key, a)


@pytest.mark.parametrize("key", list(bc.SCRAMBLE))
def test_gpu_scramble_equals_reference(solve_lib, goldens, tmp_path, key):
    golden, (_, scr) = goldens
    name, _ = bc.SCRAMBLE[key]
    p = bc.write_scramble_case(key, golden[name]["xdrop_a"], str(tmp_path / "in"), str(tmp_path / "out"))
    assert solve_lib.lakgb_bcc_run_in_file(p.encode()) == 0
    got = bc.read_outputs(str(tmp_path / "out"))
    for k in ("trace", "xdrop_a", "xdrop_b"):
        assert got[k] == scr[key][k], (key, k)
    assert bc.b16_digests(str(tmp_path / "out")) == scr[key]["b16_sha1"]
