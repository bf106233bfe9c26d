"""Generate the golden fixtures of the SNP x SNP and element-wise loop
products (AtTAn_vv, At_T_YnWt_S_Zn_vv, An_ZtSWn_Yt_vv) from the reference's
own wrap_* kernels, compiled from the reference sources by
``make -C oracle ref`` into oracle/_ref/liblakref.so.  Saves every case's
inputs and outputs to tests/golden/kernels_products.npz.

Usage (x86-64 container with the reference tree present):
    make -C oracle ref && python tests/golden/make_golden_products.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
sys.path.insert(0, os.path.dirname(HERE))

import product_cases as pc  # noqa: E402


def main():
    store = {}
    for spec in pc.specs():
        x = pc.build(spec)
        for k, v in x.items():
            store[f"{spec['name']}/in/{k}"] = v
        h = pc.handles(x)
        for kind, sa, sb in pc.keys():
            store[f"{spec['name']}/{pc.key_name(kind, sa, sb)}"] = pc.run("ref", kind, h, sa, sb)
    path = os.path.join(HERE, "kernels_products.npz")
    np.savez_compressed(path, **store)
    print("wrote", path, len(store), "arrays", os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
