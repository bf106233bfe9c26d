"""Parity cases for the SNP x SNP and element-wise loop products and the
bit-plane form of the last: AtTAn_vv, At_T_YnWt_S_Zn_vv, An_ZtSWn_Yt_vv and
An_ZtSWn_Yt_ww (dir_c/AtTAn_vv.c, dir_c/At_T_YnWt_S_Zn_vv.c,
dir_c/An_ZtSWn_Yt_vv.c, dir_c/An_ZtSWn_Yt_ww.c).

``build(spec)`` makes seeded inputs (bit matrices with ragged row and column
masks, allele weights, FP64 score matrices); ``run(backend, name, x, ...)``
calls one backend with the reference's argument lists:

  ``ref``    the reference's own wrap_* kernels (oracle/_ref/liblakref.so)
  ``oracle`` the plain-C restatement (oracle/liblakoracle.so, lako_*)
  ``gpu``    the product library (wrap_*)
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

import kernel_cases as kc
from lakcluster_c_gb300 import abi
from lakcluster_c_gb300.abi import LHandle, L_handle

SPACINGS = [abi.SPACING_a, abi.SPACING_b, abi.SPACING_j]


def specs():
    """name, sizes and seed of every case (small: the reference and the C
    oracle run these in well under a second)."""
    out = []
    shapes = [(5, 7, 9, 2), (33, 70, 41, 1), (64, 130, 90, 3), (20, 250, 200, 2)]
    for i, (nsnp, npat, nctl, nt) in enumerate(shapes):
        for masked in (False, True):
            out.append(dict(name=f"p{i}_{int(masked)}", nsnp=nsnp, npat=npat, nctl=nctl, nt=nt,
                            masked=masked, seed=5000 + 31 * i + int(masked), ww_b_index=i))
    return out


def _mask(rng, n, frac):
    b = (rng.random(n) < frac).astype(np.uint8)
    j = b & (rng.random(n) < frac).astype(np.uint8)
    if not j.any():
        b[0] = j[0] = 1
    return b, j


def build(spec):
    rng = np.random.default_rng(spec["seed"])
    frac = 0.85 if spec["masked"] else 1.0
    nsnp, npat, nctl, nt = spec["nsnp"], spec["npat"], spec["nctl"], spec["nt"]
    x = {}
    # SNP-major matrices: At (SNPs x patients), Zt (SNPs x controls)
    x["At"] = (rng.random((nsnp, npat)) < 0.4).astype(np.uint8)
    x["Zt"] = (rng.random((nsnp, nctl)) < 0.4).astype(np.uint8)
    x["Tt"] = (rng.random((nt, npat)) < 0.6).astype(np.uint8)
    x["St"] = (rng.random((nt, nctl)) < 0.6).astype(np.uint8)
    x["snp_b"], x["snp_j"] = _mask(rng, nsnp, frac)
    x["pat_b"], x["pat_j"] = _mask(rng, npat, frac)
    x["ctl_b"], x["ctl_j"] = _mask(rng, nctl, frac)
    x["t_b"], x["t_j"] = _mask(rng, nt, 1.0)
    # patient-major matrices for An_ZtSWn_Yt: An (patients x SNPs), Yn (patients x SNPs of Y)
    x["An"] = (rng.random((npat, nsnp)) < 0.4).astype(np.uint8)
    x["Yn"] = (rng.random((npat, nsnp + 3)) < 0.4).astype(np.uint8)
    x["ysnp_b"], x["ysnp_j"] = _mask(rng, nsnp + 3, frac)
    x["A_p"] = 0.05 + 0.9 * rng.random(abi.psize(nsnp))
    x["Y_p"] = 0.05 + 0.9 * rng.random(abi.psize(nsnp + 3))
    # integer-valued per-(SNP, covariate) sums, as AtTn holds them
    x["lf_AtTn"] = rng.integers(-npat, npat + 1, (nsnp, nt)).astype(np.float64)
    x["lf_YnWt"] = rng.standard_normal((npat, nctl))
    x["lf_ZtSWn"] = rng.standard_normal((nsnp, nsnp + 3, nt))
    # An_ZtSWn_Yt_ww: Wt (Y SNPs x controls; its retained rows index the
    # planes) and, per covariate row, one set of bit planes with its own
    # min / mlt (drawn after everything above, so earlier inputs keep their values)
    x["Wt"] = (rng.random((nsnp + 3, nctl)) < 0.4).astype(np.uint8)
    B = (3, 32, 8, 16)[spec.get("ww_b_index", 0) % 4] if "ww_b_index" in spec else 8
    nwj = int(x["ysnp_j"].sum())
    mcl = abi.bsize(nsnp)
    x["ww_B"] = np.array([B], np.int32)
    x["ww_planes"] = rng.integers(0, 256, (nt, (B + 1) * nwj, mcl), dtype=np.uint8)
    x["ww_min"] = -5.0 * rng.random(nt)
    x["ww_mlt"] = float(2 ** B) / (1.0 + 10.0 * rng.random(nt))
    return x


def handles(x):
    """Reference M_handle / L_handle structs for a case (kept alive in the dict)."""
    h = {}
    h["At"] = kc.mhandle(x["At"], x["snp_b"], x["snp_j"], x["pat_b"], x["pat_j"])
    h["Zt"] = kc.mhandle(x["Zt"], x["snp_b"], x["snp_j"], x["ctl_b"], x["ctl_j"])
    h["Tt"] = kc.mhandle(x["Tt"], x["t_b"], x["t_j"], x["pat_b"], x["pat_j"])
    h["St"] = kc.mhandle(x["St"], x["t_b"], x["t_j"], x["ctl_b"], x["ctl_j"])
    h["An"] = kc.mhandle(x["An"], x["pat_b"], x["pat_j"], x["snp_b"], x["snp_j"])
    h["Yn"] = kc.mhandle(x["Yn"], x["pat_b"], x["pat_j"], x["ysnp_b"], x["ysnp_j"])
    h["A_ajdk"] = abi.calc_A_ajdk(x["A_p"])
    h["Y_ajdk"] = abi.calc_A_ajdk(x["Y_p"])
    lt = LHandle.from_matrix(x["lf_AtTn"])
    h["lf_AtTn"] = lt
    h["lf_YnWt"] = LHandle.from_matrix(x["lf_YnWt"])
    z = x["lf_ZtSWn"]
    lz = LHandle(z.size)
    lz.buf[: z.size] = z.transpose(2, 1, 0).ravel()  # lf[na + ny*rs + s*rs*cs]
    lz.s.row_stride, lz.s.col_stride, lz.s.lyr_stride = z.shape
    lz.s.spacing_row = lz.s.spacing_col = lz.s.spacing_lyr = abi.SPACING_a
    h["lf_ZtSWn"] = lz
    h["Wt"] = kc.mhandle(x["Wt"], x["ysnp_b"], x["ysnp_j"], x["ctl_b"], x["ctl_j"])
    B = int(x["ww_B"][0])
    planes = []
    for s in range(x["ww_planes"].shape[0]):
        w = x["ww_planes"][s]
        m = abi.MHandle(None, nrows=w.shape[0], ncols=x["An"].shape[1], wX=w)
        m.s.ncols_per_z = B + 1
        m.s.min_d, m.s.mlt_d = float(x["ww_min"][s]), float(x["ww_mlt"][s])
        planes.append(m)
    h["ww_planes"] = planes
    h["ww_arr"] = (C.POINTER(abi.M_handle) * len(planes))(*[C.pointer(m.s) for m in planes])
    return h


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def _take(out, n):
    return kc._take(out, n)


def run(backend, kind, h, sa, sb, st=abi.SPACING_a):
    """One product on one backend; returns the output as a float64 array."""
    lib = kc.load_backend(backend)
    out = C.POINTER(L_handle)()
    if kind == "AtTAn":
        args = (sa, sb, st, h["At"].ptr, h["Tt"].ptr, h["At"].ptr, _dptr(h["A_ajdk"]), _dptr(h["A_ajdk"]),
                h["lf_AtTn"].ptr, h["lf_AtTn"].ptr, C.byref(out))
        n = lib.lako_AtTAn_vv(*args) if backend == "oracle" else lib.wrap_AtTAn_vv__run(*kc._thread_args(), *args)
    elif kind == "At_T_YnWt_S_Zn_vv":
        args = (sa, sb, h["At"].ptr, h["Tt"].ptr, h["St"].ptr, h["Zt"].ptr, _dptr(h["A_ajdk"]),
                h["lf_YnWt"].ptr, C.byref(out))
        n = (lib.lako_At_T_YnWt_S_Zn_vv(*args) if backend == "oracle"
             else lib.wrap_At_T_YnWt_S_Zn_vv__run(*kc._thread_args(), *args))
    elif kind == "An_ZtSWn_Yt_vv":
        args = (sa, sb, h["An"].ptr, h["St"].ptr, h["Yn"].ptr, _dptr(h["A_ajdk"]), _dptr(h["Y_ajdk"]),
                h["lf_ZtSWn"].ptr, C.byref(out))
        n = (lib.lako_An_ZtSWn_Yt_vv(*args) if backend == "oracle"
             else lib.wrap_An_ZtSWn_Yt_vv__run(*kc._thread_args(), *args))
    elif kind == "An_ZtSWn_Yt_ww":
        args = (sa, sb, h["An"].ptr, h["St"].ptr, h["ww_arr"], h["Wt"].ptr, h["Yn"].ptr, _dptr(h["A_ajdk"]),
                _dptr(h["Y_ajdk"]), C.byref(out))
        n = (lib.lako_An_ZtSWn_Yt_ww(*args) if backend == "oracle"
             else lib.wrap_An_ZtSWn_Yt_ww__run(*kc._thread_args(), *args))
    else:
        raise ValueError(kind)
    return _take(out, n)


KINDS = ["AtTAn", "At_T_YnWt_S_Zn_vv", "An_ZtSWn_Yt_vv", "An_ZtSWn_Yt_ww"]
SPACING_PAIRS = [(abi.SPACING_a, abi.SPACING_a), (abi.SPACING_j, abi.SPACING_b), (abi.SPACING_b, abi.SPACING_j)]


def keys():
    """(kind, spacing_a, spacing_b) combinations stored per case."""
    return [(k, sa, sb) for k in KINDS for sa, sb in SPACING_PAIRS]


def key_name(kind, sa, sb):
    return f"{kind}/{sa}{sb}"


GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "kernels_products.npz")


def load_golden():
    """{case name: (inputs dict, {key name: expected output})}."""
    d = np.load(GOLDEN)
    cases = {}
    for k in d.files:
        name, rest = k.split("/", 1)
        ins, outs = cases.setdefault(name, ({}, {}))
        if rest.startswith("in/"):
            ins[rest[3:]] = d[k]
        else:
            outs[rest] = d[k]
    return cases
