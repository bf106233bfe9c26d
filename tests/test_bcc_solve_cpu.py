"""Whole-solve checks that need no GPU.

* The package's solve driver, linked against the reference's own kernels
  (oracle/_ref/lakbcc_refkernels), reproduces the reference program's output
  files byte for byte, and the committed golden traces.
* The product library loads and exports every entry point its header declares.
* The .b16 writer / reader round trip.
The first group needs the reference built from its sources (x86-64 only) and
is skipped where oracle/_ref is absent.
"""
import ctypes
import os
import re

import numpy as np
import pytest

import bcc_cases as bc
from lakcluster_c_gb300 import infiles

HAVE_REF = os.path.exists(bc.REF_PROGRAM) and os.path.exists(bc.REF_KERNELS_DRIVER)
needs_ref = pytest.mark.skipif(not HAVE_REF, reason="reference build (oracle/_ref) not present")


@pytest.fixture(scope="module")
def golden():
    return bc.load_golden()


def test_golden_covers_every_case(golden):
    assert set(golden) == set(bc.CASES) | set(bc.LARGE_CASES)
    for name in bc.SMALL:
        assert golden[name]["stages"], name


def test_goldens_with_controls_come_from_the_reference_program():
    z = np.load(bc.GOLDEN, allow_pickle=False)
    for name in list(bc.CASES) + list(bc.LARGE_CASES):
        has_controls = (bc.CASES.get(name) or bc.LARGE_CASES.get(name))[1]
        src = str(z[name + "/source"][0])
        assert (src == "reference program") == has_controls, (name, src)


@needs_ref
@pytest.mark.parametrize("name", ["case_only_200x300", "case_control_1bin_gamma_lin"])
def test_driver_on_reference_kernels_matches_golden(tmp_path, golden, name):
    p = bc.write_case(name, str(tmp_path / "in"), str(tmp_path / "out"))
    bc.run_refkernels(p)
    got = bc.read_outputs(str(tmp_path / "out"))
    for key in ("trace", "xdrop_a", "xdrop_b"):
        assert got[key] == golden[name][key], key


@needs_ref
@pytest.mark.parametrize("name", ["case_only_200x300", "case_control_2bin_masked"])
def test_stage_digest_golden_is_current(tmp_path, golden, name):
    """The committed per-stage digests (what the GPU solve's LAKBCC_TRACE is
    compared with) are those of the current driver on the reference's kernels,
    so a driver change that adds or reorders a stage shows up here first."""
    p = bc.write_case(name, str(tmp_path / "in"), str(tmp_path / "out"))
    tpath = str(tmp_path / "stages.trace")
    bc.run_refkernels(p, env=dict(os.environ, LAKBCC_TRACE=tpath))
    assert bc.trace_digest(tpath) == golden[name]["stages"]


@needs_ref
def test_driver_reproduces_reference_program_on_case_control(tmp_path):
    name = "case_control_1bin_gamma_lin"
    p = bc.write_case(name, str(tmp_path / "in"), str(tmp_path / "ref"), "ref.in")
    q = bc.write_case(name, str(tmp_path / "in"), str(tmp_path / "rk"), "rk.in")
    bc.run_reference(p)
    bc.run_refkernels(q)
    assert bc.read_outputs(str(tmp_path / "ref")) == bc.read_outputs(str(tmp_path / "rk"))


@needs_ref
def test_driver_reproduces_reference_program_without_controls(tmp_path):
    """Without controls the reference adds a constant it reads past an empty
    buffer; with that constant injected, the driver matches it exactly."""
    name = "case_only_200x300"
    p = bc.write_case(name, str(tmp_path / "in"), str(tmp_path / "ref"), "ref.in")
    q = bc.write_case(name, str(tmp_path / "in"), str(tmp_path / "rk"), "rk.in")
    bc.run_reference(p)
    raw = open(str(tmp_path / "ref" / "AZ_rsum.mda"), "rb").read()
    az = np.frombuffer(raw[12:], np.float64)
    k = az - bc.build(name)["A"][0].sum(0)
    assert np.all(k == k[0])
    bc.run_refkernels(q, env=dict(os.environ, LAKREF_EMPTY_Z_ROWSUM=repr(float(k[0]))))
    assert bc.read_outputs(str(tmp_path / "ref")) == bc.read_outputs(str(tmp_path / "rk"))


def test_library_exports_every_declared_entry_point():
    from lakcluster_c_gb300 import build
    lib_path = build.build_lib()
    lib = ctypes.CDLL(lib_path)
    hdr = open(os.path.join(bc.ROOT, "include", "lakcluster_gb300.h")).read()
    hdr = re.sub(r"/\*.*?\*/", "", hdr, flags=re.S)
    names = re.findall(r"^\s*(?:int|void|double|unsigned long long|long long|lakgb_\w+|struct \w+)\s*\**\s*(\w+)\s*\(",
                       hdr, flags=re.M)
    assert "lakgb_gram_group_create" in names and "lakgb_server_create" in names
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_b16_round_trip(tmp_path):
    rng = np.random.default_rng(0)
    for shape in [(1, 1), (3, 15), (5, 16), (7, 17), (2, 1921)]:
        x = (rng.random(shape) < 0.5).astype(np.uint8)
        p = str(tmp_path / ("m_%d_%d.b16" % shape))
        infiles.write_b16(p, x)
        assert np.array_equal(infiles.read_b16(p), x)
        hdr = np.fromfile(p, dtype=np.int32, count=3)
        assert list(hdr) == [16, shape[1], shape[0]]


@pytest.fixture(scope="module")
def port_driver():
    import subprocess
    subprocess.run(["make", "-s", "-C", os.path.join(bc.ROOT, "oracle"), "port"], check=True)
    return os.path.join(bc.ROOT, "oracle", "lakbcc_port")


@pytest.mark.parametrize("name", list(bc.CASES))
def test_oracle_port_solve_matches_golden(tmp_path, golden, port_driver, name):
    """The driver on the plain-C oracle kernels: a whole solve that builds on
    every machine, pinned to the reference's outputs."""
    import subprocess
    p = bc.write_case(name, str(tmp_path / "in"), str(tmp_path / "out"))
    r = subprocess.run([port_driver, p], stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    assert r.returncode == 0, r.stdout[-2000:]
    got = bc.read_outputs(str(tmp_path / "out"))
    for key in ("trace", "xdrop_a", "xdrop_b"):
        assert got[key] == golden[name][key], key
