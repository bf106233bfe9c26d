"""Scorebox and scramble runs of the solve driver on the C oracle
(oracle/lakbcc_port: the package's driver linked against the plain-C
restatement of the kernels; builds on every host), against the reference
program's own outputs in tests/golden/bcc_scorebox.npz.

  * scorebox (lakcluster_scorebox, dir_c/lakcluster_scorebox.c:103-271): the
    five grid arrays, integers and the FP64 mean scores bit for bit, for
    both loop orders (rows inner / columns inner);
  * scramble (wrap_bcc_scramble, dir_c/R_init.c:165-290): the scrambled
    solve's trace and elimination order, and the pre / post .b16 snapshots.
"""
import os
import subprocess

import numpy as np
import pytest

import bcc_cases as bc

ROOT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..")
PORT = os.path.join(ROOT, "oracle", "lakbcc_port")


@pytest.fixture(scope="module")
def port():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "port"], check=True)
    return PORT


@pytest.fixture(scope="module")
def goldens():
    return bc.load_golden(), bc.load_scorebox_golden()


def _run(port, p):
    r = subprocess.run([port, p], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:]


def test_golden_covers_every_scorebox_and_scramble_case(goldens):
    _, (sb, scr) = goldens
    assert set(sb) == set(bc.SCOREBOX) and set(scr) == set(bc.SCRAMBLE)
    for key, (_, (rmax, rnum, cmax, cnum)) in bc.SCOREBOX.items():
        assert sb[key]["QR_avg"].shape == (rnum, cnum)
        # the grid reaches row_max + 1 retained rows and col_max + 1 columns first
        assert sb[key]["A_rpop_j_total"][0, 0] == rmax + 1 and sb[key]["A_cpop_j"][0, 0] == cmax + 1


@pytest.mark.parametrize("key", list(bc.SCOREBOX))
def test_port_scorebox_equals_reference(port, goldens, tmp_path, key):
    golden, (sb, _) = goldens
    name, grid = bc.SCOREBOX[key]
    p = bc.write_scorebox_case(key, golden[name]["xdrop_a"], str(tmp_path / "in"), str(tmp_path / "out"))
    _run(port, p)
    got = bc.read_scorebox(str(tmp_path / "out"), grid)
    for a in bc.SCOREBOX_ARRAYS:
        assert np.array_equal(got[a].view(np.uint8), sb[key][a].view(np.uint8)), (key, a)


@pytest.mark.parametrize("key", list(bc.SCRAMBLE))
def test_port_scramble_equals_reference(port, goldens, tmp_path, key):
    golden, (_, scr) = goldens
    name, _ = bc.SCRAMBLE[key]
    p = bc.write_scramble_case(key, golden[name]["xdrop_a"], str(tmp_path / "in"), str(tmp_path / "out"))
    _run(port, p)
    got = bc.read_outputs(str(tmp_path / "out"))
    for k in ("trace", "xdrop_a", "xdrop_b"):
        assert got[k] == scr[key][k], (key, k)
    assert bc.b16_digests(str(tmp_path / "out")) == scr[key]["b16_sha1"]
    assert got["xdrop_a"] != golden[name]["xdrop_a"]   # the scramble changed the solve
