"""Build liblakgb300.so (the product library) and the test oracle in-tree.

The CUDA sources are compiled for sm_103a only, in parallel, one object per
translation unit, then linked into a shared library next to this file.  Host
code is compiled with FP contraction off so FP64 expressions round exactly as
the reference's (x86-64 gcc -O2 without -mfma evaluates a*b+c as two roundings;
gcc on aarch64 would otherwise fuse them).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "liblakgb300.so")

CU_SOURCES = ["lakgb_runtime.cu", "gram.cu", "gram_tc.cu", "rowvec.cu", "abi_kernels.cu", "xcalc.cu", "bitplane.cu",
              "bitplane_tc.cu", "loopsum.cu", "lmirror.cu",
              "vv_kernels.cu", "transpose.cu", "bed.cu", "condense.cu"]
# Host-only translation units (the solve driver and its input reader).
CPP_SOURCES = ["bcc_model.cpp", "bcc_sort.cpp", "bcc_driver.cpp", "bcc_io.cpp", "bcc_abi.cpp", "bcc_server.cpp"]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-pthread", "-I" + os.path.join(ROOT, "include")]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2",
    "-I" + os.path.join(ROOT, "include"),
]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblakgb300.so")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return False
    t = os.path.getmtime(target)
    return all(os.path.getmtime(d) <= t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        sys.stderr.write(r.stdout)
        raise RuntimeError("build step failed: " + " ".join(cmd))


def build_lib(force: bool = False, verbose: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    headers.append(os.path.join(ROOT, "include", "lakcluster_gb300.h"))
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append([nvcc] + NVCC_FLAGS + ["-c", s, "-o", o])
    cxx = shutil.which("g++") or "g++"
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src.replace(".cpp", ".o"))
        objs.append(o)
        if force or not _newer(o, [s] + headers):
            jobs.append([cxx] + CXX_FLAGS + ["-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            list(ex.map(_run, jobs))
    if force or jobs or not _newer(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart", "-lpthread"])
    if verbose:
        print("built", LIB)
    return LIB


def build_oracle(force: bool = False) -> str:
    """Compile the plain-C oracle, and the reference where oracle/Makefile
    finds its sources (LAK_REFERENCE_DIR overrides the Makefile's REF)."""
    odir = os.path.join(ROOT, "oracle")
    ref = os.environ.get("LAK_REFERENCE_DIR")
    _run(["make", "-s", "-C", odir] + (["REF=" + ref] if ref else []) + (["-B"] if force else [])
         + ["oracle", "ref-if-present"])
    return os.path.join(odir, "liblakoracle.so")


if __name__ == "__main__":
    build_lib(force="--force" in sys.argv, verbose=True)
    build_oracle()
