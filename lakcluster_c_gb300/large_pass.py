"""The Gram pass of the large single-solve configuration on one GPU:
cases 32768 and controls 32768 x 131072 SNPs, MAF U[0.01, 0.5], a
2048 x 4096 planted bicluster with 5 % flips, rows in 3 covariate bins.

At this size the 0/1 matrices (4.3 G entries each) never exist: the packed
rows are drawn on the device, chunk by chunk (torch as plumbing: a seeded
generator, comparisons, an MSB-first bit pack).  The pass is the reference's
bcc_lf_YnWt Gram pass (dir_c/bcc_lf.c:223-270): AnZt for every bin pair and
AnAt for nb1 <= nb2, D-weighted, with the AJDK_1_1 row terms.  The row terms
come from the library's own wrap_An_ajdk_v on host copies of the packed bins.

``run_checks`` runs every product with both Gram kernels and compares the
outputs bit for bit, and recomputes sampled entries on the host from the
packed bits (XOR popcounts per 1920-column block and the FP64 fold in block
order, in Python floats, which are IEEE binary64).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import abi
from ._lib import load
from .gram_pass import AJDK_0_1, AJDK_1_1, AJDK_2_1, GramArgs, products

TENSOR, POPCOUNT = 1, 0


def _pack_rows(bits, row_bytes):
    """(rows, m) bool tensor -> (rows, row_bytes) uint8, MSB first, zero padded."""
    import torch
    rows, m = bits.shape
    pad = row_bytes * 8 - m
    if pad:
        bits = torch.cat([bits, torch.zeros(rows, pad, dtype=torch.bool, device=bits.device)], dim=1)
    w = torch.tensor([128, 64, 32, 16, 8, 4, 2, 1], dtype=torch.uint8, device=bits.device)
    return (bits.view(rows, row_bytes, 8).to(torch.uint8) * w).sum(dim=2, dtype=torch.uint8)


class LargeGramPass:
    def __init__(self, n_cases=32768, n_controls=32768, ncols=131072, nbins=3, planted=(2048, 4096),
                 flip=0.05, maf=(0.01, 0.5), seed=3, device="cuda", chunk_rows=2048):
        import torch
        self.torch = torch
        self.ncols, self.nbins = ncols, nbins
        self.P = abi.psize(ncols)
        self.row_bytes = abi.bsize(ncols)
        g = torch.Generator(device=device)
        g.manual_seed(seed)
        p = maf[0] + (maf[1] - maf[0]) * torch.rand(ncols, generator=g, device=device)
        pr, pc = planted
        pattern = torch.rand(pc, generator=g, device=device) < 0.5
        # bin of every row (uniform), cases then controls
        bin_a = torch.randint(0, nbins, (n_cases,), generator=g, device=device)
        bin_z = torch.randint(0, nbins, (n_controls,), generator=g, device=device)
        self.A = [[] for _ in range(nbins)]
        self.Z = [[] for _ in range(nbins)]
        colsum = torch.zeros(ncols, dtype=torch.float64, device=device)
        for side, n, bins, store in (("A", n_cases, bin_a, self.A), ("Z", n_controls, bin_z, self.Z)):
            for r0 in range(0, n, chunk_rows):
                r1 = min(n, r0 + chunk_rows)
                bits = torch.rand(r1 - r0, ncols, generator=g, device=device) < p
                if side == "A" and r0 < pr:
                    k = min(r1, pr) - r0
                    noise = torch.rand(k, pc, generator=g, device=device) < flip
                    bits[:k, :pc] = pattern ^ noise
                if side == "A":
                    colsum += bits.sum(dim=0, dtype=torch.float64)
                packed = _pack_rows(bits, self.row_bytes)
                b = bins[r0:r1]
                for nb in range(nbins):
                    store[nb].append(packed[b == nb])
                del bits
        self.A = [torch.cat(x) for x in self.A]
        self.Z = [torch.cat(x) for x in self.Z]
        # per-block allele frequency over all case rows (bcc_load_A_p)
        A_p = np.full(self.P, 0.5)
        cs = colsum.cpu().numpy()
        for blk in range(self.P):
            lo, hi = blk * abi.POPLENGTH, min((blk + 1) * abi.POPLENGTH, ncols)
            if hi > lo:
                A_p[blk] = cs[lo:hi].sum() / max(1, (hi - lo) * n_cases)
        self.A_ajdk = abi.calc_A_ajdk(A_p)
        mask = np.zeros(self.row_bytes, np.uint8)
        mask[: ncols // 8] = 0xFF
        if ncols % 8:
            mask[ncols // 8] = (0xFF << (8 - ncols % 8)) & 0xFF
        self.mask_host = mask
        self.mask = torch.from_numpy(mask).to(device)
        self.D = torch.from_numpy(self.A_ajdk[AJDK_0_1 * self.P:(AJDK_0_1 + 1) * self.P].copy()).to(device)
        a0 = a2 = 0.0
        for nc in range(self.P):
            c = float(np.unpackbits(mask[nc * 240:(nc + 1) * 240]).sum())
            a0 += self.A_ajdk[nc + AJDK_0_1 * self.P] * c
            a2 += self.A_ajdk[nc + AJDK_2_1 * self.P] * c
        self.a0d1, self.a2d1 = a0, a2
        self.lib = load()
        self.lib.lakgb_gram_device.argtypes = [C.POINTER(GramArgs)]
        self.lib.lakgb_gram_device.restype = C.c_int
        self.lf11 = {}
        self.lf11_host = {}
        for nb in range(nbins):
            for key, W in (("A", self.A[nb]), ("Z", self.Z[nb])):
                v = self._row_terms(W)
                self.lf11_host[(key, nb)] = v
                self.lf11[(key, nb)] = torch.from_numpy(v).to(device)
        self.rows = {}
        for nb in range(nbins):
            for key, W in (("A", self.A[nb]), ("Z", self.Z[nb])):
                self.rows[(key, nb)] = torch.arange(W.shape[0], dtype=torch.int32, device=device)
        self.args = []
        for kind, nb1, nb2, sym in products(nbins):
            W1 = self.A[nb1]
            zkey = ("Z", nb2) if kind == "AnZt" else ("A", nb2)
            W2 = self.Z[nb2] if kind == "AnZt" else self.A[nb2]
            a = GramArgs()
            a.wA = W1.data_ptr(); a.a_rowb = self.rows[("A", nb1)].data_ptr()
            a.nA = W1.shape[0]; a.a_row_bytes = self.row_bytes
            a.wZ = W2.data_ptr(); a.z_rowb = self.rows[zkey].data_ptr()
            a.nZ = W2.shape[0]; a.z_row_bytes = self.row_bytes
            a.mask = self.mask.data_ptr(); a.P = self.P
            a.D = self.D.data_ptr(); a.type_flag = abi.TYPE_pm
            a.a0d1, a.a2d1 = self.a0d1, self.a2d1
            a.lfA = self.lf11[("A", nb1)].data_ptr(); a.lfZ = self.lf11[zkey].data_ptr()
            a.out_r = self.rows[("A", nb1)].data_ptr(); a.out_c = self.rows[zkey].data_ptr()
            a.out_r2 = self.rows[zkey].data_ptr(); a.out_c2 = self.rows[("A", nb1)].data_ptr()
            a.out_stride = W1.shape[0]; a.symmetric = int(sym)
            self.args.append(((kind, nb1, nb2, sym), a, W1.shape[0] * W2.shape[0]))
        self.max_out = max(n for _, _, n in self.args)
        self.out = torch.empty(self.max_out, dtype=torch.float64, device=device)
        self.out2 = None

    def _row_terms(self, W):
        """AJDK_1_1 row terms of packed rows W through wrap_An_ajdk_v."""
        lib = self.lib
        w = W.cpu().numpy()
        M = abi.MHandle(None, wX=w, nrows=w.shape[0], ncols=self.ncols)
        out = C.POINTER(abi.L_handle)()
        lib.wrap_An_ajdk_v(C.byref(C.c_int(0)), None, None, abi.TYPE_pm, abi.SPACING_b, M.ptr,
                           self.A_ajdk.ctypes.data_as(C.POINTER(C.c_double)), C.byref(out))
        n = M.rpop_b * abi.AJDK_TOT
        v = np.ctypeslib.as_array(C.cast(out.contents.lf, C.POINTER(C.c_double)), shape=(n,)).copy()
        return np.ascontiguousarray(v[np.arange(M.rpop_b) + AJDK_1_1 * M.rpop_b])

    def work_bitops(self) -> float:
        return float(sum(n for _, _, n in self.args)) * float(self.ncols)

    def run(self, stream_handle=0, out=None):
        """One pass; every product writes into the same output buffer."""
        out = self.out if out is None else out
        for _, a, _ in self.args:
            a.stream = stream_handle
            a.out = out.data_ptr()
            if self.lib.lakgb_gram_device(C.byref(a)) != 0:
                raise RuntimeError("lakgb_gram_device failed")

    def _host_entry(self, kind, nb1, nb2, i, k):
        """One output entry recomputed on the host (reference order)."""
        ra = self.A[nb1][i].cpu().numpy()
        rz = (self.Z[nb2] if kind == "AnZt" else self.A[nb2])[k].cpu().numpy()
        x = np.unpackbits(ra ^ rz) & np.unpackbits(self.mask_host)
        acc = 0.0
        D = self.A_ajdk[AJDK_0_1 * self.P:(AJDK_0_1 + 1) * self.P]
        for b in range(self.P):
            c = float(x[b * 1920:(b + 1) * 1920].sum())
            acc = acc + float(D[b]) * c
        zkey = ("Z", nb2) if kind == "AnZt" else ("A", nb2)
        o = self.a0d1 - 2.0 * acc
        return o - ((float(self.lf11_host[("A", nb1)][i]) + float(self.lf11_host[zkey][k])) - self.a2d1)

    def run_checks(self, samples_per_product=4, seed=0):
        """Both kernels on every product: identical outputs; sampled entries
        equal to the host recomputation.  Returns a summary dict."""
        torch = self.torch
        rng = np.random.default_rng(seed)
        self.lib.lakgb_set_gram_impl.argtypes = [C.c_int]
        self.lib.lakgb_gram_impl.restype = C.c_int
        self.lib.lakgb_device_status.restype = C.c_int
        before = self.lib.lakgb_gram_impl()
        out_t = torch.empty(self.max_out, dtype=torch.float64, device=self.out.device)
        out_p = torch.empty_like(out_t)
        identical, sampled, sample_ok = 0, 0, 0
        try:
            for (kind, nb1, nb2, sym), a, n in self.args:
                res = {}
                for impl, buf in ((TENSOR, out_t), (POPCOUNT, out_p)):
                    buf.zero_()
                    self.lib.lakgb_set_gram_impl(impl)
                    a.stream = 0
                    a.out = buf.data_ptr()
                    if self.lib.lakgb_gram_device(C.byref(a)) != 0:
                        raise RuntimeError("lakgb_gram_device failed")
                torch.cuda.synchronize()
                if torch.equal(out_t[:n].view(torch.int64), out_p[:n].view(torch.int64)):
                    identical += 1
                nA = a.nA
                for _ in range(samples_per_product):
                    i = int(rng.integers(0, a.nA))
                    k = int(rng.integers(i if sym else 0, a.nZ))
                    got = float(out_t[i + k * nA].item())
                    want = self._host_entry(kind, nb1, nb2, i, k)
                    sampled += 1
                    sample_ok += int(np.float64(got).view(np.uint64) == np.float64(want).view(np.uint64))
        finally:
            self.lib.lakgb_set_gram_impl(before)
        return {"products": len(self.args), "tensor_equals_popcount": identical, "sampled_entries": sampled,
                "sampled_equal_host": sample_ok, "device_status": self.lib.lakgb_device_status()}


class LargeGramPassHost:
    """The same pass through the reference-facing C entry points
    (wrap_AnZt_vv__run / wrap_AnAt_vv__run) on host buffers: the packed bins
    of a LargeGramPass copied once into pinned host memory, M_handles over
    them (every row and SNP retained), the full AJDK row-term handles from
    wrap_An_ajdk_v, and FP64 outputs in host L_handles the library allocates
    on the first call and refills on every later one (the reference's
    zero-then-fill contract) -- or, with ``pinned_outputs``, in caller-owned
    output handles over page-locked host memory (the reference's callers
    may pass pre-allocated outputs; the callee checks their length and fills
    them).

    ``run`` makes one call per product.  With residency on, each packed bin
    is uploaded by the first call that reads it and reused by the others of
    the same pass; ``forget_inputs`` drops those copies so that the next pass
    uploads every bin again (the per-step host-to-device copy)."""

    def __init__(self, lp: LargeGramPass, pinned_outputs: bool = False):
        import torch
        self.lp = lp
        self.lib = lp.lib
        self.lib.wrap_An_ajdk_v.restype = C.c_int
        self.M = {}
        self._pinned = []
        for nb in range(lp.nbins):
            for key, W in (("A", lp.A[nb]), ("Z", lp.Z[nb])):
                h = torch.empty(tuple(W.shape), dtype=torch.uint8, pin_memory=True)
                h.copy_(W)
                self._pinned.append(h)
                self.M[(key, nb)] = abi.MHandle(None, wX=h.numpy(), nrows=W.shape[0], ncols=lp.ncols)
        self.lf = {}
        for k, M in self.M.items():
            out = C.POINTER(abi.L_handle)()
            self.lib.wrap_An_ajdk_v(C.byref(C.c_int(0)), None, None, abi.TYPE_pm, abi.SPACING_b, M.ptr,
                                    lp.A_ajdk.ctypes.data_as(C.POINTER(C.c_double)), C.byref(out))
            n = M.rpop_b * abi.AJDK_TOT
            v = np.ctypeslib.as_array(C.cast(out.contents.lf, C.POINTER(C.c_double)), shape=(n,)).copy()
            h = abi.LHandle(n)
            h.buf[:] = v
            h.s.row_stride, h.s.col_stride = M.rpop_b, abi.AJDK_TOT
            h.s.spacing_row, h.s.spacing_col = abi.SPACING_b, abi.SPACING_a
            self.lf[k] = h
        self.outputs = {}
        self._out_bufs = []
        if pinned_outputs:
            for key, ka, kz in self.calls():
                n = self.M[ka].rpop_b * self.M[kz].rpop_b
                buf = torch.empty(n, dtype=torch.float64, pin_memory=True)
                L = abi.L_handle()
                L.length, L.lf = n, buf.data_ptr()
                self._out_bufs.append((buf, L))
                self.outputs[key] = C.pointer(L)

    def calls(self):
        for kind, nb1, nb2, sym in products(self.lp.nbins):
            zkey = ("Z", nb2) if kind == "AnZt" else ("A", nb2)
            yield (kind, nb1, nb2, sym), ("A", nb1), zkey

    def forget_inputs(self):
        for M in self.M.values():
            self.lib.lakgb_forget_host_buffer(C.c_void_p(M.wX.ctypes.data))

    def h2d_bytes(self) -> int:
        """Bytes one pass copies host to device: every packed bin once, and
        per call the column mask, the row-index and output-index lists, the
        block weights and the row terms it reads."""
        n = sum(M.wX.nbytes for M in self.M.values())
        P = self.lp.P
        for (kind, nb1, nb2, sym), ka, kz in self.calls():
            nA, nZ = self.M[ka].rpop_j, self.M[kz].rpop_j
            n += self.M[ka].mc_length + 8 * P + 4 * 2 * (nA + nZ) * (2 if sym else 1) + 8 * (nA + nZ)
        return n

    def run(self) -> int:
        """One pass; returns the FP64 output bytes copied back to the host."""
        aj = self.lp.A_ajdk.ctypes.data_as(C.POINTER(C.c_double))
        nbytes = 0
        for key, ka, kz in self.calls():
            out = self.outputs.get(key)
            if out is None:
                out = self.outputs[key] = C.POINTER(abi.L_handle)()
            fn = self.lib.wrap_AnAt_vv__run if key[3] else self.lib.wrap_AnZt_vv__run
            n = fn(C.byref(C.c_int(0)), None, None, abi.TYPE_pm, abi.SPACING_b, abi.SPACING_b,
                   self.M[ka].ptr, self.M[kz].ptr, aj, self.lf[ka].ptr, self.lf[kz].ptr, C.byref(out))
            nbytes += 8 * n
        return nbytes

    def run_timed(self) -> list:
        """One pass as ``run``, returning each call's wall time (s)."""
        import time
        aj = self.lp.A_ajdk.ctypes.data_as(C.POINTER(C.c_double))
        out_s = []
        for key, ka, kz in self.calls():
            out = self.outputs.get(key)
            if out is None:
                out = self.outputs[key] = C.POINTER(abi.L_handle)()
            fn = self.lib.wrap_AnAt_vv__run if key[3] else self.lib.wrap_AnZt_vv__run
            t0 = time.perf_counter()
            fn(C.byref(C.c_int(0)), None, None, abi.TYPE_pm, abi.SPACING_b, abi.SPACING_b,
               self.M[ka].ptr, self.M[kz].ptr, aj, self.lf[ka].ptr, self.lf[kz].ptr, C.byref(out))
            out_s.append(time.perf_counter() - t0)
        return out_s

    def output(self, key) -> np.ndarray:
        L = self.outputs[key].contents
        return np.ctypeslib.as_array(C.cast(L.lf, C.POINTER(C.c_double)), shape=(int(L.length),))


def host_rows(n_rows, ncols, maf=(0.01, 0.5), planted=(2048, 4096), flip=0.05, seed=3, chunk=512):
    """Packed rows (n_rows x bsize(ncols) bytes) drawn on the host with the
    large configuration's distributions: per-SNP MAF U[maf], Bernoulli bits,
    and the first planted[0] rows sharing a random pattern on the first
    planted[1] SNPs with `flip` noise (a numpy PCG64 stream; for CPU timing
    samples, which need the shapes and distributions, not the device bits)."""
    rng = np.random.default_rng(seed)
    p = (maf[0] + (maf[1] - maf[0]) * rng.random(ncols)).astype(np.float32)
    pr, pc = planted
    pattern = rng.random(pc) < 0.5
    row_bytes = abi.bsize(ncols)
    out = np.zeros((n_rows, row_bytes), np.uint8)
    for r0 in range(0, n_rows, chunk):
        r1 = min(n_rows, r0 + chunk)
        bits = rng.random((r1 - r0, ncols), dtype=np.float32) < p
        if r0 < pr:
            k = min(r1, pr) - r0
            bits[:k, :pc] = pattern ^ (rng.random((k, pc)) < flip)
        out[r0:r1, : (ncols + 7) // 8] = np.packbits(bits, axis=1, bitorder="big")
    return out


class GroupedGramPasses:
    """The Gram passes of several independent problems (e.g. label-shuffled
    null instances), each product with its own output buffer, run either one
    launch per product (``run_plain``) or as one grouped persistent launch of
    the tensor-core kernel (``run_grouped``, lakgb_gram_group_run), which
    gives the same outputs bit for bit."""

    def __init__(self, passes):
        import torch
        self.torch = torch
        self.passes = passes
        self.lib = passes[0].lib
        self.items = []
        for ps in passes:
            for key, a, n in ps.args:
                out = torch.empty(n, dtype=torch.float64, device=ps.out.device)
                a.out = out.data_ptr()
                self.items.append((ps, key, a, out))
        self.n = len(self.items)
        arr = (GramArgs * self.n)()
        for i, (_, _, a, _) in enumerate(self.items):
            arr[i] = a
        self._arr = arr
        self.group = self.lib.lakgb_gram_group_create(C.cast(arr, C.c_void_p), self.n)
        if not self.group:
            raise RuntimeError("lakgb_gram_group_create failed")

    def work_bitops(self) -> float:
        return float(sum(ps.work_bitops() for ps in self.passes))

    def outputs(self):
        return [out for _, _, _, out in self.items]

    def run_plain(self, stream_handle=0):
        for _, _, a, _ in self.items:
            a.stream = stream_handle
            if self.lib.lakgb_gram_device(C.byref(a)) != 0:
                raise RuntimeError("lakgb_gram_device failed")

    def run_grouped(self, stream_handle=0):
        if self.lib.lakgb_gram_group_run(self.group, C.c_void_p(stream_handle or None)) != 0:
            raise RuntimeError("lakgb_gram_group_run failed")

    def close(self):
        if self.group:
            self.lib.lakgb_gram_group_destroy(self.group)
            self.group = None


def main(argv=None):
    """Run a large-configuration Gram pass on the GPU a few times (for
    profiling one form of it on a chosen size)."""
    import argparse
    import time

    ap = argparse.ArgumentParser(description="Gram pass of the large configuration, or a smaller one of its shape.")
    ap.add_argument("--cases", type=int, default=32768)
    ap.add_argument("--controls", type=int, default=32768)
    ap.add_argument("--snps", type=int, default=131072)
    ap.add_argument("--bins", type=int, default=3)
    ap.add_argument("--grouped", action="store_true", help="one grouped launch per pass")
    ap.add_argument("--reps", type=int, default=2)
    args = ap.parse_args(argv)
    import torch
    lp = LargeGramPass(n_cases=args.cases, n_controls=args.controls, ncols=args.snps, nbins=args.bins)
    g = GroupedGramPasses([lp]) if args.grouped else None
    print("products %d, bit-ops per pass %.6e" % (len(lp.args), lp.work_bitops()), flush=True)
    for r in range(args.reps):
        t0 = time.perf_counter()
        if g is not None:
            g.run_grouped(0)
        else:
            lp.run(0)
        torch.cuda.synchronize()
        print("pass %d (%s): %.3f ms" % (r, "grouped" if g else "per product", 1e3 * (time.perf_counter() - t0)),
              flush=True)
    if g is not None:
        g.close()


if __name__ == "__main__":
    main()
