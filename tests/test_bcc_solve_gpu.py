"""Whole bcc solves on the GPU, checked against the reference's outputs.

Every case's out_trace / out_xdrop lines must equal the golden ones exactly
(the elimination order and the %0.16f-printed mean scores), through both the
.in-file entry point and the in-memory one, twice in a row in one process
(device residency must not leak state between solves).  For the small cases
the per-stage digest of every intermediate product is compared as well, so a
failure names the first stage that diverged.
"""
import os
import subprocess
import sys

import pytest

import bcc_cases as bc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def golden():
    return bc.load_golden()


@pytest.fixture(scope="module")
def solve_lib(gpu_lib):
    return bc.bind_solve(gpu_lib)


@pytest.mark.parametrize("name", list(bc.CASES))
def test_in_memory_solve_matches_reference(solve_lib, golden, name):
    for _ in range(2):
        got = bc.solve_in_memory(solve_lib, name)
        for key in ("trace", "xdrop_a", "xdrop_b"):
            assert got[key] == golden[name][key], key


def test_large_case_control_solve_matches_reference(solve_lib, golden):
    """The 4096 + 4096 x 16384 two-bin workload against the reference program's outputs."""
    name = "case_control_4096x4096x16384"
    got = bc.solve_in_memory(solve_lib, name)
    for key in ("trace", "xdrop_a", "xdrop_b"):
        assert got[key] == golden[name][key], key


@pytest.mark.parametrize("name", bc.SMALL)
def test_in_file_solve_matches_reference(solve_lib, golden, tmp_path, name):
    p = bc.write_case(name, str(tmp_path / "in"), str(tmp_path / "out"))
    rc = solve_lib.lakgb_bcc_run_in_file(p.encode())
    assert rc == 0
    got = bc.read_outputs(str(tmp_path / "out"))
    for key in ("trace", "xdrop_a", "xdrop_b"):
        assert got[key] == golden[name][key], key


@pytest.mark.parametrize("name", ["case_only_200x300", "case_control_2bin_masked", "case_control_2bin_masked_qr_condense"])
def test_stage_digests_match_reference_kernels(gpu_lib, golden, tmp_path, name):
    p = bc.write_case(name, str(tmp_path / "in"), str(tmp_path / "out"))
    tpath = str(tmp_path / "stages.trace")
    code = ("import ctypes,sys; lib=ctypes.CDLL(sys.argv[1]); "
            "lib.lakgb_bcc_run_in_file.argtypes=[ctypes.c_char_p]; "
            "sys.exit(lib.lakgb_bcc_run_in_file(sys.argv[2].encode()))")
    from lakcluster_c_gb300 import build
    r = subprocess.run([sys.executable, "-c", code, build.LIB, p], env=dict(os.environ, LAKBCC_TRACE=tpath),
                       stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    got, want = bc.trace_digest(tpath), golden[name]["stages"]
    for i, (g, w) in enumerate(zip(got, want)):
        assert g == w, "first divergence at line %d: got %r want %r" % (i, g, w)
    assert len(got) == len(want)
