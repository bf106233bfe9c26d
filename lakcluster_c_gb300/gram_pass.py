"""The bcc Gram pass (bcc_lf_YnWt, dir_c/bcc_lf.c:223-270) over all bin pairs.

For bins nb1, nb2 the reference computes, all with the +/-1 centred D-weighted
Gram of wrap_AnZt_vv__run / wrap_AnAt_vv__run at SPACING_b:
    lf_AnZt[nb1,nb2] = A_nb1 x Z_nb2          (every pair)
    lf_AnAt[nb1,nb1] = A_nb1 x A_nb1          (symmetric kernel)
    lf_AnAt[nb1,nb2] = A_nb1 x A_nb2          (nb1 < nb2; nb1 > nb2 is its transpose)

Two ways to run it are provided:
  ``GramPassDevice``  inputs already resident in HBM, one lakgb_gram_device
                      launch per product (the throughput measured as `value`)
  ``gram_pass_host``  the reference-facing C entry points on host buffers,
                      host<->device copies included (the `e2e` measurement)

Work is counted as the reference's own Gram kernels define it: rows_A x rows_Z
x retained columns per product (the full square for the symmetric one).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from ._lib import load
from .abi import MHandle
from .synth import BccInstance

AJDK_0_1, AJDK_1_1, AJDK_2_1 = 5, 6, 7


class GramArgs(C.Structure):
    _fields_ = [
        ("wA", C.c_void_p), ("a_rowb", C.c_void_p), ("nA", C.c_int), ("a_row_bytes", C.c_longlong),
        ("wZ", C.c_void_p), ("z_rowb", C.c_void_p), ("nZ", C.c_int), ("z_row_bytes", C.c_longlong),
        ("mask", C.c_void_p), ("P", C.c_int),
        ("D", C.c_void_p), ("type_flag", C.c_int),
        ("a0d1", C.c_double), ("a2d1", C.c_double),
        ("lfA", C.c_void_p), ("lfZ", C.c_void_p),
        ("out_r", C.c_void_p), ("out_c", C.c_void_p),
        ("out_r2", C.c_void_p), ("out_c2", C.c_void_p),
        ("out_stride", C.c_longlong), ("out", C.c_void_p),
        ("symmetric", C.c_int),
        ("stream", C.c_void_p),
    ]


def block_allele_freq(inst: BccInstance) -> np.ndarray:
    """Per-1920-column-block frequency of the minor allele over all case rows
    (the quantity bcc_load_A_p turns into alpha and D)."""
    P = abi.psize(inst.ncols)
    A = np.concatenate(inst.A_bins, axis=0)
    s = A.sum(axis=0).astype(np.float64)
    out = np.full(P, 0.5)
    for b in range(P):
        lo, hi = b * abi.POPLENGTH, min((b + 1) * abi.POPLENGTH, inst.ncols)
        if hi > lo:
            out[b] = s[lo:hi].sum() / max(1, (hi - lo) * A.shape[0])
    return out


def products(nbins: int):
    """(kind, nb1, nb2, symmetric) for every Gram launch of the pass."""
    out = []
    for nb1 in range(nbins):
        for nb2 in range(nbins):
            out.append(("AnZt", nb1, nb2, False))
            if nb1 == nb2:
                out.append(("AnAt", nb1, nb2, True))
            elif nb1 < nb2:
                out.append(("AnAt", nb1, nb2, False))
    return out


class GramPassHost:
    """Reference structs for every bin (host buffers)."""

    def __init__(self, inst: BccInstance):
        self.inst = inst
        self.MA = [MHandle(a) for a in inst.A_bins]
        self.MZ = [MHandle(z) if z.shape[0] > 0 else None for z in inst.Z_bins]
        self.A_p = block_allele_freq(inst)
        self.A_ajdk = abi.calc_A_ajdk(self.A_p)
        self.P = abi.psize(inst.ncols)
        self.cpop = inst.ncols
        lib = load()
        self.lf = {}
        for b in range(inst.nbins):
            for key, M in (("A", self.MA[b]), ("Z", self.MZ[b])):
                if M is None:
                    continue
                out = C.POINTER(abi.L_handle)()
                lib.wrap_An_ajdk_v(C.byref(C.c_int(0)), None, None, abi.TYPE_pm, abi.SPACING_b, M.ptr,
                                   self.A_ajdk.ctypes.data_as(C.POINTER(C.c_double)), C.byref(out))
                L = out.contents
                n = M.rpop_b * abi.AJDK_TOT
                v = np.ctypeslib.as_array(C.cast(L.lf, C.POINTER(C.c_double)), shape=(n,)).copy()
                self.lf[(key, b)] = v

    def work_bitops(self) -> float:
        w = 0.0
        for kind, nb1, nb2, sym in products(self.inst.nbins):
            MA = self.MA[nb1]
            MZ = self.MZ[nb2] if kind == "AnZt" else self.MA[nb2]
            if MZ is None:
                continue
            w += float(MA.rpop_j) * float(MZ.rpop_j) * float(self.cpop)
        return w

    def mask_sums(self):
        mc = self.MA[0].mc_j
        a0 = a2 = 0.0
        for nc in range(self.P):
            c = float(np.unpackbits(mc[nc * 240:(nc + 1) * 240]).sum())
            a0 += self.A_ajdk[nc + AJDK_0_1 * self.P] * c
            a2 += self.A_ajdk[nc + AJDK_2_1 * self.P] * c
        return a0, a2


def gram_pass_host(gp: GramPassHost, outputs: dict | None = None) -> int:
    """Run every product through the reference-facing C entry points on host
    buffers.  Returns the number of output bytes copied back to the host."""
    lib = load()
    aj = gp.A_ajdk.ctypes.data_as(C.POINTER(C.c_double))
    nbytes = 0
    for kind, nb1, nb2, sym in products(gp.inst.nbins):
        MA = gp.MA[nb1]
        if kind == "AnZt":
            MZ, lfZ_key = gp.MZ[nb2], ("Z", nb2)
        else:
            MZ, lfZ_key = gp.MA[nb2], ("A", nb2)
        if MZ is None:
            continue
        lfA = _lh(gp.lf[("A", nb1)], MA)
        lfZ = _lh(gp.lf[lfZ_key], MZ)
        key = (kind, nb1, nb2)
        out = outputs.get(key) if outputs is not None else None
        if out is None:
            out = C.POINTER(abi.L_handle)()
            if outputs is not None:
                outputs[key] = out
        fn = lib.wrap_AnAt_vv__run if sym else lib.wrap_AnZt_vv__run
        n = fn(C.byref(C.c_int(0)), None, None, abi.TYPE_pm, abi.SPACING_b, abi.SPACING_b,
               MA.ptr, MZ.ptr, aj, lfA.ptr, lfZ.ptr, C.byref(out))
        nbytes += 8 * n
    return nbytes


def _lh(vec: np.ndarray, M: MHandle):
    h = abi.LHandle(vec.size)
    h.buf[:] = vec
    h.s.row_stride, h.s.col_stride = M.rpop_b, abi.AJDK_TOT
    h.s.spacing_row, h.s.spacing_col = abi.SPACING_b, abi.SPACING_a
    return h


class GramPassDevice:
    """Every operand of the pass resident in HBM (torch tensors as plumbing);
    ``run(stream)`` enqueues one Gram launch per product."""

    def __init__(self, gp: GramPassHost, device="cuda"):
        import torch
        self.torch = torch
        self.gp = gp
        t = lambda a, dt=None: torch.from_numpy(np.ascontiguousarray(a)).to(device)  # noqa: E731
        self.w = {}
        self.rows = {}
        self.lf11 = {}
        for b in range(gp.inst.nbins):
            for key, M in (("A", gp.MA[b]), ("Z", gp.MZ[b])):
                if M is None:
                    continue
                self.w[(key, b)] = t(M.wX)
                self.rows[(key, b)] = t(M.m_b_[: M.rpop_j].astype(np.int32))
                lf = gp.lf[(key, b)]
                self.lf11[(key, b)] = t(lf[M.m_b_[: M.rpop_j].astype(np.int64) + AJDK_1_1 * M.rpop_b])
        self.mask = t(gp.MA[0].mc_j)
        self.D = t(gp.A_ajdk[AJDK_0_1 * gp.P:(AJDK_0_1 + 1) * gp.P])
        self.a0d1, self.a2d1 = gp.mask_sums()
        self.args = []
        self.out = {}
        for kind, nb1, nb2, sym in products(gp.inst.nbins):
            zkey = ("Z", nb2) if kind == "AnZt" else ("A", nb2)
            if zkey not in self.w:
                continue
            MA = gp.MA[nb1]
            MZ = gp.MZ[nb2] if kind == "AnZt" else gp.MA[nb2]
            out = torch.zeros(MA.rpop_b * MZ.rpop_b, dtype=torch.float64, device=device)
            self.out[(kind, nb1, nb2)] = out
            a = GramArgs()
            a.wA = self.w[("A", nb1)].data_ptr(); a.a_rowb = self.rows[("A", nb1)].data_ptr()
            a.nA = MA.rpop_j; a.a_row_bytes = MA.mc_length
            a.wZ = self.w[zkey].data_ptr(); a.z_rowb = self.rows[zkey].data_ptr()
            a.nZ = MZ.rpop_j; a.z_row_bytes = MZ.mc_length
            a.mask = self.mask.data_ptr(); a.P = gp.P
            a.D = self.D.data_ptr(); a.type_flag = abi.TYPE_pm
            a.a0d1, a.a2d1 = self.a0d1, self.a2d1
            a.lfA = self.lf11[("A", nb1)].data_ptr(); a.lfZ = self.lf11[zkey].data_ptr()
            # SPACING_b with all rows retained: output index = wX row
            a.out_r = self.rows[("A", nb1)].data_ptr(); a.out_c = self.rows[zkey].data_ptr()
            a.out_r2 = self.rows[zkey].data_ptr(); a.out_c2 = self.rows[("A", nb1)].data_ptr()
            a.out_stride = MA.rpop_b; a.out = out.data_ptr(); a.symmetric = int(sym)
            self.args.append(a)
        self.lib = load()
        self.lib.lakgb_gram_device.argtypes = [C.POINTER(GramArgs)]
        self.lib.lakgb_gram_device.restype = C.c_int

    def run(self, stream_handle: int = 0) -> int:
        for a in self.args:
            a.stream = stream_handle
            rc = self.lib.lakgb_gram_device(C.byref(a))
            if rc != 0:
                raise RuntimeError("lakgb_gram_device failed")
        return len(self.args)

    def run_grouped(self, stream_handle: int = 0) -> int:
        """The whole pass as one grouped persistent launch of the tensor-core
        kernel (lakgb_gram_group_run): same outputs, one tile list over all
        products instead of one launch per product."""
        if getattr(self, "_group", None) is None:
            arr = (GramArgs * len(self.args))(*self.args)
            self._group_args = arr
            self._group = self.lib.lakgb_gram_group_create(C.cast(arr, C.c_void_p), len(self.args))
            if not self._group:
                raise RuntimeError("lakgb_gram_group_create failed")
        if self.lib.lakgb_gram_group_run(self._group, C.c_void_p(stream_handle or None)) != 0:
            raise RuntimeError("lakgb_gram_group_run failed")
        return 1

    def close(self):
        if getattr(self, "_group", None):
            self.lib.lakgb_gram_group_destroy(self._group)
            self._group = None


def main(argv=None):
    """Run the case/control Gram pass on the GPU a few times, per product or as
    one grouped launch (for profiling a single form of the pass)."""
    import argparse
    import time

    ap = argparse.ArgumentParser(description="Run the case/control Gram pass (4096 + 4096 x 16384, 2 bins).")
    ap.add_argument("--grouped", action="store_true", help="one grouped launch per pass")
    ap.add_argument("--reps", type=int, default=3)
    args = ap.parse_args(argv)
    import torch
    from . import synth
    gp = GramPassHost(synth.case_control(seed=2))
    dev = GramPassDevice(gp)
    for r in range(args.reps):
        t0 = time.perf_counter()
        (dev.run_grouped if args.grouped else dev.run)(0)
        torch.cuda.synchronize()
        print("pass %d (%s): %.3f ms" % (r, "grouped" if args.grouped else "per product",
                                         1e3 * (time.perf_counter() - t0)), flush=True)
    dev.close()


if __name__ == "__main__":
    main()
