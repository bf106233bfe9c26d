"""Generate the kernel-level golden fixtures from the reference itself.

Runs the reference's own wrap_* kernels -- compiled from the reference sources
by ``make -C oracle ref`` into oracle/_ref/liblakref.so -- on seeded inputs and
saves inputs and outputs to tests/golden/kernels_gram.npz.  The fixtures pin
both the C restatement (oracle/lak_oracle.c) and the GPU library.

Usage (x86-64 container with the reference tree present):
    make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.dirname(HERE))

from lakcluster_c_gb300 import abi  # noqa: E402
import kernel_cases as kc  # noqa: E402

SPACING_COMBOS = [(abi.SPACING_a, abi.SPACING_a), (abi.SPACING_j, abi.SPACING_j),
                  (abi.SPACING_b, abi.SPACING_a)]


def ref_calc_ajdk(A_p: np.ndarray) -> np.ndarray:
    lib = kc.load_backend("ref")
    out = np.zeros(abi.AJDK_TOT * A_p.size, np.float64)
    p = C.c_void_p(out.ctypes.data)
    lib.calc_A_ajdk(A_p.ctypes.data_as(C.POINTER(C.c_double)), A_p.size, C.byref(p))
    return out


def main():
    store: dict[str, np.ndarray] = {}
    for spec in kc.gram_case_specs():
        name = spec["name"]
        x = kc.build_gram_inputs(spec)
        for k, v in x.items():
            if v is not None:
                store[f"{name}/in/{k}"] = v
        MA = kc.mhandle(x["A"], x["ar_b"], x["ar_j"], x["mc_b"], x["mc_j"])
        MZ = kc.mhandle(x["Z"], x["zr_b"], x["zr_j"], x["mc_b"], x["mc_j"])
        A_ajdk = lfA = lfZ = None
        if x["A_p"] is not None:
            A_ajdk = ref_calc_ajdk(x["A_p"])
            store[f"{name}/A_ajdk"] = A_ajdk
            vA = kc.call_an_ajdk("ref", abi.TYPE_pm, abi.SPACING_a, MA, A_ajdk)
            vZ = kc.call_an_ajdk("ref", abi.TYPE_pm, abi.SPACING_a, MZ, A_ajdk)
            store[f"{name}/lf_An_ajdk"] = vA
            store[f"{name}/lf_Zn_ajdk"] = vZ
            lfA = kc.lhandle_from(vA, MA.nrows, abi.AJDK_TOT, abi.SPACING_a)
            lfZ = kc.lhandle_from(vZ, MZ.nrows, abi.AJDK_TOT, abi.SPACING_a)
            for spr in (abi.SPACING_a, abi.SPACING_b, abi.SPACING_j):
                store[f"{name}/An_ajdk/{spr}"] = kc.call_an_ajdk("ref", abi.TYPE_pm, spr, MA, A_ajdk)
        for t in (abi.TYPE_pm, abi.TYPE_00):
            for spr in (abi.SPACING_a, abi.SPACING_b, abi.SPACING_j):
                store[f"{name}/An_v/{t}/{spr}"] = kc.call_an_v("ref", t, spr, MA)
            for spr, spc in SPACING_COMBOS:
                store[f"{name}/AnZt/{t}/{spr}{spc}"] = kc.call_gram("ref", False, t, spr, spc, MA, MZ, A_ajdk, lfA, lfZ)
                store[f"{name}/AnAt/{t}/{spr}{spc}"] = kc.call_gram("ref", True, t, spr, spc, MA, MA, A_ajdk, lfA, lfA)
    path = os.path.join(HERE, "kernels_gram.npz")
    np.savez_compressed(path, **store)
    print("wrote", path, len(store), "arrays", os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
