"""The solve driver's host sorts and mask index lists against restatements of
the reference's own algorithms (CPU only).

`lakcluster_c_gb300/csrc/bcc_sort.cpp` sorts the row and column scores of
every iteration: a radix sort when the scores are all distinct, else the
reference's quicksort.  `bcc_model.cpp` builds the index lists of the
retained rows and columns 64 elements at a time.  Both are compiled here on
their own with a small harness and compared with the pure-Python
restatements below on seeded inputs: distinct values, many ties, signed
zeros, NaNs, infinities, sorted inputs and small recursion limits.
"""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "lakcluster_c_gb300", "csrc")

HARNESS = r"""
#include <stdio.h>
#include <stdint.h>
#include <string.h>
#include <vector>
#include "bcc_model.h"
#include "bcc_sort.h"
using namespace lakbcc;

template <typename T> static T get(FILE *f) { T v; if (fread(&v, sizeof v, 1, f) != 1) v = T(); return v; }

int main(int argc, char **argv) {
  if (argc != 4) return 2;
  FILE *in = fopen(argv[2], "rb"), *out = fopen(argv[3], "wb");
  if (!in || !out) return 3;
  const int ncases = get<int32_t>(in);
  for (int c = 0; c < ncases; ++c) {
    if (!strcmp(argv[1], "sort")) {
      const int kind = get<int32_t>(in), n = get<int32_t>(in);
      const unsigned limit = get<uint32_t>(in);
      const int stride = get<int32_t>(in);
      std::vector<double> d((size_t)n * stride + 1);
      if (n) fread(d.data(), sizeof(double), (size_t)n * stride, in);
      std::vector<int> idx(n + 1);
      for (int k = 0; k < n; ++k) idx[k] = k;
      if (kind == 0) quicksort_xij(limit, d.data(), idx.data(), nullptr, nullptr, nullptr, nullptr, nullptr, 0, n - 1);
      else dquicksort_strided(limit, d.data(), stride, 0, n - 1);
      if (n) fwrite(d.data(), sizeof(double), (size_t)n * stride, out);
      if (n) fwrite(idx.data(), sizeof(int), (size_t)n, out);
    } else {
      const int n = get<int32_t>(in), len = get<int32_t>(in);
      MH *M = mh_make_owned(n, 1);
      if (len != (int)M->h.mr_length) return 4;
      fread(M->mr_b.data(), 1, (size_t)len, in);
      fread(M->mr_j.data(), 1, (size_t)len, in);
      std::vector<unsigned> a(n + 1, 0xFFFFFFFFu), b(n + 1, 0xFFFFFFFFu);
      M->h.m_a_ = a.data();
      M->h.m_b_ = b.data();
      mh_mxget(M);
      const long long pb = M->h.rpop_b, pj = M->h.rpop_j;
      fwrite(&pb, 8, 1, out);
      fwrite(&pj, 8, 1, out);
      fwrite(a.data(), 4, (size_t)n, out);
      fwrite(b.data(), 4, (size_t)n, out);
      delete M;
    }
  }
  fclose(out);
  return 0;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("host_sort")
    src = d / "harness.cpp"
    src.write_text(HARNESS)
    exe = d / "harness"
    subprocess.run(["g++", "-O2", "-std=c++17", "-I", CSRC, str(src), os.path.join(CSRC, "bcc_sort.cpp"),
                    os.path.join(CSRC, "bcc_model.cpp"), "-o", str(exe)], check=True)
    return str(exe), d


# --- restatements ----------------------------------------------------------


def _partition(d, idx, stride, l, r):
    """dPartition_xij / dPartition (dir_c/Quicksort.c:83-110): first element as
    pivot, i up over values <= pivot, j down over values > pivot, swap."""
    pivot = d[stride * l]
    i, j = l, r + 1
    while True:
        i += 1
        while i <= r and d[stride * i] <= pivot:
            i += 1
        j -= 1
        while d[stride * j] > pivot:
            j -= 1
        if i >= j:
            break
        d[stride * i], d[stride * j] = d[stride * j], d[stride * i]
        if idx is not None:
            idx[i], idx[j] = idx[j], idx[i]
    d[stride * l], d[stride * j] = d[stride * j], d[stride * l]
    if idx is not None:
        idx[l], idx[j] = idx[j], idx[l]
    return j


def ref_quicksort_xij(d, idx, limit):
    """dQuickSort_xij (dir_c/Quicksort.c:111-141): partition, then recurse on
    both sides while nn < GLOBAL_recursion_limit."""
    stack = [(0, len(d) - 1, 0)]
    while stack:
        l, r, nn = stack.pop()
        if l < r:
            j = _partition(d, idx, 1, l, r)
            if nn < limit:
                stack.append((l, j - 1, nn + 1))
                stack.append((j + 1, r, nn + 1))


def ref_dquicksort(d, stride, n, limit):
    """dQuickSort (dir_c/Quicksort.c:43-81): the limit is checked before the
    partition."""
    stack = [(0, n - 1, 0)]
    while stack:
        l, r, nn = stack.pop()
        if l < r and nn < limit:
            j = _partition(d, None, stride, l, r)
            stack.append((l, j - 1, nn + 1))
            stack.append((j + 1, r, nn + 1))


def ref_mxget(n, mb, mj):
    """M_mxget_excerpt (dir_c/M_init.c:244-271): popcounts of the whole masks;
    every bit on in mb takes the next b index, those also on in mj are listed
    with their a and b indices (bit 7 of a byte first)."""
    bits_b = np.unpackbits(mb)
    bits_j = np.unpackbits(mj)
    a_, b_ = [], []
    b = 0
    for a in range(n):
        if bits_b[a]:
            if bits_j[a]:
                a_.append(a)
                b_.append(b)
            b += 1
    return int(bits_b.sum()), int(bits_j.sum()), a_, b_


def bsize(n):
    n16 = n + (16 - n % 16) % 16
    return (n16 + 1919) // 1920 * 1920 // 8


# --- cases -------------------------------------------------------------------


def _values(rng, mode, n):
    if mode == "distinct":
        return rng.standard_normal(n)
    if mode == "ties":
        return rng.integers(0, 10, n).astype(np.float64)
    if mode == "zeros":
        v = rng.standard_normal(n)
        v[rng.random(n) < 0.3] = 0.0
        v[rng.random(n) < 0.05] = -0.0
        return v
    if mode == "nan":
        v = rng.standard_normal(n)
        v[rng.random(n) < 0.02] = np.nan
        return v
    if mode == "inf":
        v = np.ldexp(rng.standard_normal(n), rng.integers(-1000, 1000, n))
        v[rng.random(n) < 0.03] = np.inf
        v[rng.random(n) < 0.03] = -np.inf
        return v
    if mode == "sorted":
        return np.sort(rng.standard_normal(n))
    raise ValueError(mode)


def _sort_cases():
    rng = np.random.default_rng(20240611)
    cases = []
    modes = ["distinct", "ties", "zeros", "nan", "inf", "sorted"]
    for t in range(240):
        mode = modes[t % len(modes)]
        n = int(rng.integers(0, 300))
        limit = int(rng.integers(0, 12)) if t % 5 == 0 else 32768
        cases.append((0, _values(rng, mode, n), limit, 1))
    for mode in ("distinct", "ties", "zeros"):
        cases.append((0, _values(rng, mode, 2000), 32768, 1))
    cases.append((0, _values(rng, "sorted", 600), 300, 1))   # more values than the limit
    cases.append((0, _values(rng, "distinct", 600), 300, 1))
    for t in range(40):
        n = int(rng.integers(1, 12))
        cases.append((1, _values(rng, modes[t % 3], n * 3), int(rng.integers(0, 5)) if t % 4 == 0 else 32768, 3))
    return cases


def _run(harness, cmd, payload):
    exe, d = harness
    fin, fout = d / (cmd + ".in"), d / (cmd + ".out")
    fin.write_bytes(payload)
    subprocess.run([exe, cmd, str(fin), str(fout)], check=True)
    return fout.read_bytes()


def test_sorts_match_reference_quicksort(harness):
    cases = _sort_cases()
    buf = [struct.pack("<i", len(cases))]
    for kind, v, limit, stride in cases:
        n = len(v) // stride
        buf.append(struct.pack("<iiIi", kind, n, limit, stride))
        buf.append(np.ascontiguousarray(v, dtype="<f8").tobytes())
    out = _run(harness, "sort", b"".join(buf))
    off = 0
    fast = 0
    for c, (kind, v, limit, stride) in enumerate(cases):
        n = len(v) // stride
        got_d = np.frombuffer(out, "<f8", n * stride, off)
        off += 8 * n * stride
        got_i = np.frombuffer(out, "<i4", n, off)
        off += 4 * n
        d = [float(x) for x in v]
        idx = list(range(n))
        if kind == 0:
            ref_quicksort_xij(d, idx, limit)
            assert list(got_i) == idx, "case %d: index order" % c
        else:
            ref_dquicksort(d, stride, n, limit)
        # bitwise: signed zeros and NaNs must land where the quicksort puts them
        assert np.array_equal(np.asarray(d, dtype="<f8").view("<u8"), got_d.view("<u8")), "case %d: values" % c
        if kind == 0 and len(set(d)) == n and not np.isnan(d).any():
            fast += 1
    assert off == len(out)
    assert fast > 40  # the radix path ran on many of the cases


def test_mask_index_lists_match_reference_walk(harness):
    rng = np.random.default_rng(77)
    cases = []
    for t in range(300):
        n = int(rng.integers(0, 2500))
        L = bsize(n)
        kind = t % 4
        if kind == 0:      # every element retained, a few removed
            mb = np.full(L, 255, np.uint8)
            mj = mb.copy()
            for k in rng.integers(0, max(1, n), 5):
                mj[k // 8] &= ~np.uint8(1 << (7 - k % 8))
        elif kind == 1:    # sparse masks (elements just removed)
            mb = np.full(L, 255, np.uint8)
            mj = np.zeros(L, np.uint8)
            for k in rng.integers(0, max(1, n), 7):
                mj[k // 8] |= np.uint8(1 << (7 - k % 8))
        else:              # random densities, bits past n included
            pb, pj = rng.random(), rng.random()
            mb = np.packbits(rng.random(8 * L) < pb)
            mj = np.packbits(rng.random(8 * L) < pj)
        cases.append((n, mb, mj))
    buf = [struct.pack("<i", len(cases))]
    for n, mb, mj in cases:
        buf.append(struct.pack("<ii", n, len(mb)))
        buf.append(mb.tobytes())
        buf.append(mj.tobytes())
    out = _run(harness, "mxget", b"".join(buf))
    off = 0
    for c, (n, mb, mj) in enumerate(cases):
        pb, pj = struct.unpack_from("<qq", out, off)
        off += 16
        a = np.frombuffer(out, "<u4", n, off)
        off += 4 * n
        b = np.frombuffer(out, "<u4", n, off)
        off += 4 * n
        rpb, rpj, ra, rb = ref_mxget(n, mb, mj)
        assert (pb, pj) == (rpb, rpj), "case %d: popcounts" % c
        k = len(ra)
        assert list(a[:k]) == ra and list(b[:k]) == rb, "case %d: index lists" % c
        assert (a[k:] == 0xFFFFFFFF).all() and (b[k:] == 0xFFFFFFFF).all(), "case %d: wrote past the list" % c
    assert off == len(out)
