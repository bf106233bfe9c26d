"""Dexcluster (GLOBAL_TEST_TYPE dexcluster_driver, dir_c/dexcluster_driver.c)
without a GPU: the solve driver's dcc mode on the C oracle (oracle/lakbcc_port)
writes exactly the out_trace / out_xdrop_a / out_xdrop_b lines the reference
program wrote for the same inputs (tests/golden/dcc_traces.npz): bins, row and
column masks, gamma_type, GLOBAL_Ireq, covariate columns with kappa."""
import os
import subprocess

import pytest

import bcc_cases as bc

ROOT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..")
PORT = os.path.join(ROOT, "oracle", "lakbcc_port")


@pytest.fixture(scope="module")
def port():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    return PORT


@pytest.fixture(scope="module")
def golden():
    return bc.load_dcc_golden()


@pytest.mark.parametrize("name", bc.DCC_CASES)
def test_port_dcc_equals_reference(port, golden, tmp_path, name):
    p = bc.write_dcc_case(name, str(tmp_path / "in"), str(tmp_path / "out"))
    r = subprocess.run([port, p], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    got = bc.read_outputs(str(tmp_path / "out"))
    for k in ("trace", "xdrop_a", "xdrop_b"):
        assert got[k] == golden[name][k], (name, k)


def test_dcc_differs_from_bcc():
    g, d = bc.load_golden(), bc.load_dcc_golden()
    assert all(g[n]["trace"] != d[n]["trace"] for n in bc.DCC_CASES)


@pytest.fixture(scope="module")
def extra():
    return bc.load_dcc_extra_golden()


@pytest.mark.parametrize("key", list(bc.DCC_SCOREBOX))
def test_port_dcc_scorebox_equals_reference(port, golden, extra, tmp_path, key):
    import numpy as np
    name, grid = bc.DCC_SCOREBOX[key]
    p = bc.write_scorebox_case(key, golden[name]["xdrop_a"], str(tmp_path / "in"), str(tmp_path / "out"))
    r = subprocess.run([port, p], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    got = bc.read_scorebox(str(tmp_path / "out"), grid)
    for a in bc.SCOREBOX_ARRAYS:
        assert np.array_equal(got[a].view(np.uint8), extra[0][key][a].view(np.uint8)), (key, a)


@pytest.mark.parametrize("key", list(bc.DCC_SCRAMBLE))
def test_port_dcc_scramble_equals_reference(port, golden, extra, tmp_path, key):
    name, _ = bc.DCC_SCRAMBLE[key]
    p = bc.write_scramble_case(key, golden[name]["xdrop_a"], str(tmp_path / "in"), str(tmp_path / "out"))
    r = subprocess.run([port, p], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]
    got = bc.read_outputs(str(tmp_path / "out"))
    for k in ("trace", "xdrop_a", "xdrop_b"):
        assert got[k] == extra[1][key][k], (key, k)
    assert bc.b16_digests(str(tmp_path / "out")) == extra[1][key]["b16_sha1"]
