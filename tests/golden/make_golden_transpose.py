"""Generate the golden fixtures of the .b16 transpose from the reference's own
wrap_transpose (dir_c/binary_read.c:174), compiled from the reference sources
by ``make -C oracle ref`` into oracle/_ref/liblakref.so: for every case of
tests/transpose_cases.py, the input file's bytes and the reference's output
file's bytes (with two workspace chunk sizes, which must agree), saved to
tests/golden/b16_transpose.npz.

Usage (x86-64 container with the reference tree present):
    make -C oracle ref && python tests/golden/make_golden_transpose.py
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

import transpose_cases as tc  # noqa: E402


def main():
    store = {}
    with tempfile.TemporaryDirectory() as td:
        for i, shape in enumerate(tc.SHAPES):
            src = os.path.join(td, "in_%d.b16" % i)
            raw = tc.write_file(src, tc.matrix(i, shape))
            outs = [tc.file_transpose("ref", src, os.path.join(td, "out_%d_%d.b16" % (i, k)), k)
                    for k in (8, 4096)]
            assert outs[0] == outs[1], shape
            store["case%02d/in" % i] = np.frombuffer(raw, np.uint8)
            store["case%02d/out" % i] = np.frombuffer(outs[0], np.uint8)
    np.savez_compressed(tc.GOLDEN, **store)
    print("wrote", tc.GOLDEN, len(store), "arrays", os.path.getsize(tc.GOLDEN), "bytes")


if __name__ == "__main__":
    main()
