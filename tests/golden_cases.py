"""Load the committed kernel fixtures (made by tests/golden/make_golden.py from
the reference's own kernels) back into reference structs."""
from __future__ import annotations

import os

import numpy as np

import kernel_cases as kc
from lakcluster_c_gb300 import abi

HERE = os.path.dirname(os.path.abspath(__file__))
GRAM_NPZ = os.path.join(HERE, "golden", "kernels_gram.npz")


class GramFixture:
    def __init__(self, npz, name):
        g = lambda k: npz[f"{name}/{k}"] if f"{name}/{k}" in npz.files else None  # noqa: E731
        self.name = name
        x = {k: g(f"in/{k}") for k in ("A", "ar_b", "ar_j", "Z", "zr_b", "zr_j", "mc_b", "mc_j", "A_p")}
        self.MA = kc.mhandle(x["A"], x["ar_b"], x["ar_j"], x["mc_b"], x["mc_j"])
        self.MZ = kc.mhandle(x["Z"], x["zr_b"], x["zr_j"], x["mc_b"], x["mc_j"])
        self.A_ajdk = g("A_ajdk")
        self.lfA = self.lfZ = None
        if self.A_ajdk is not None:
            self.lfA = kc.lhandle_from(g("lf_An_ajdk"), self.MA.nrows, abi.AJDK_TOT, abi.SPACING_a)
            self.lfZ = kc.lhandle_from(g("lf_Zn_ajdk"), self.MZ.nrows, abi.AJDK_TOT, abi.SPACING_a)
        self.npz = npz
        self.prefix = name

    def expected(self, key):
        return self.npz[f"{self.prefix}/{key}"]

    def keys(self, kind):
        pre = f"{self.prefix}/{kind}/"
        return [k[len(self.prefix) + 1:] for k in self.npz.files if k.startswith(pre)]


def load_gram_fixtures():
    npz = np.load(GRAM_NPZ)
    names = sorted({k.split("/")[0] for k in npz.files})
    return [GramFixture(npz, n) for n in names]


def run_key(backend, fx: GramFixture, key):
    parts = key.split("/")
    kind = parts[0]
    if kind in ("AnZt", "AnAt"):
        t = int(parts[1]); spr, spc = int(parts[2][0]), int(parts[2][1])
        sym = kind == "AnAt"
        MZ = fx.MA if sym else fx.MZ
        lfZ = fx.lfA if sym else fx.lfZ
        return kc.call_gram(backend, sym, t, spr, spc, fx.MA, MZ, fx.A_ajdk, fx.lfA, lfZ)
    if kind == "An_v":
        return kc.call_an_v(backend, int(parts[1]), int(parts[2]), fx.MA)
    if kind == "An_ajdk":
        return kc.call_an_ajdk(backend, abi.TYPE_pm, int(parts[1]), fx.MA, fx.A_ajdk)
    raise KeyError(key)


def all_keys(fx: GramFixture):
    keys = []
    for kind in ("AnZt", "AnAt", "An_v", "An_ajdk"):
        keys += fx.keys(kind)
    return keys
