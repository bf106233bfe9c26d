"""The large single-solve configuration against the C oracle, stage by stage.

Cases 32768 and controls 32768 x 131072 SNPs (MAF U[0.01,0.5], a 2048 x 4096
planted bicluster with 5% flips, rows in 3 bins), packed rows drawn on the
GPU (lakcluster_c_gb300.large_pass); the oracle reads host copies of the same
bits.  Compared bit for bit:

  * An_ajdk (dir_c/An_ajdk_v.c:272-363) of all six bins, all 15 row-term
    columns: wrap_An_ajdk_v against lako_An_ajdk_v;
  * every one of the pass's 15 Gram products (dir_c/AnZt_vv.c:5-183,
    dir_c/AnAt_vv.c:5-155), in full, from the pass's one grouped tensor-core
    launch (the form the benchmark times) against lako_AnZt_vv / lako_AnAt_vv
    with the oracle's own row terms;
  * xcalc (dir_c/xcalc.c:41-246) of the bin-0 x bin-0 AnZt scores
    (about 10900 x 10900): planes, min, max and mlt;
  * the bit-plane loop product At_T_YnWt_S_Zn_ww (dir_c/At_T_YnWt_S_Zn_ww.c)
    on those planes for a fixed subset of SNPs (the first 256 and 256 more
    drawn uniformly with seed 5), every patient and control of bin 0.

The oracle side takes a few minutes on the host cores (the Gram pass is
2.35e14 bit pairs).
"""
import ctypes as C
import os

import numpy as np
import pytest

import kernel_cases as kc
from lakcluster_c_gb300 import abi

pytestmark = pytest.mark.gpu

SUBSET_SNPS = 512


@pytest.fixture(scope="module")
def large(gpu_lib, oracle_lib):
    from lakcluster_c_gb300.large_pass import GroupedGramPasses, LargeGramPass
    oracle_lib.lako_set_threads(os.cpu_count() or 1)
    lp = LargeGramPass()
    g = GroupedGramPasses([lp])
    g.run_grouped(0)
    import torch
    torch.cuda.synchronize()
    host = {}
    for nb in range(lp.nbins):
        for key, W in (("A", lp.A[nb]), ("Z", lp.Z[nb])):
            w = W.cpu().numpy()
            host[(key, nb)] = abi.MHandle(None, wX=w, nrows=w.shape[0], ncols=lp.ncols)
    yield lp, g, host
    g.close()


def test_large_an_ajdk_equals_oracle(large):
    lp, _, host = large
    for key, M in host.items():
        got = kc.call_an_ajdk("gpu", abi.TYPE_pm, abi.SPACING_b, M, lp.A_ajdk)
        want = kc.call_an_ajdk("oracle", abi.TYPE_pm, abi.SPACING_b, M, lp.A_ajdk)
        assert got.size == M.rpop_b * abi.AJDK_TOT
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64)), key


def _oracle_lf(lp, M):
    v = kc.call_an_ajdk("oracle", abi.TYPE_pm, abi.SPACING_b, M, lp.A_ajdk)
    return kc.lhandle_from(v, M.rpop_b, abi.AJDK_TOT, abi.SPACING_b)


def test_large_gram_pass_equals_oracle(large):
    import torch
    lp, g, host = large
    lf = {k: _oracle_lf(lp, M) for k, M in host.items()}
    assert len(lp.args) == 15
    for ((kind, nb1, nb2, sym), a, n), out in zip(lp.args, g.outputs()):
        zkey = ("Z", nb2) if kind == "AnZt" else ("A", nb2)
        want = kc.call_gram("oracle", sym, abi.TYPE_pm, abi.SPACING_b, abi.SPACING_b, host[("A", nb1)],
                            host[zkey], lp.A_ajdk, lf[("A", nb1)], lf[zkey])
        got = out[:n].view(torch.int64).cpu().numpy().view(np.uint64)
        assert want.size == n
        assert np.array_equal(got, want.view(np.uint64)), (kind, nb1, nb2)


def _xcalc(backend, lp, MA, MZ, L, B=32):
    """wrap_xcalc / lako_xcalc of the AnZt scores L (rows: MA's rows, columns:
    MZ's rows), as the solve's bcc_M_YnWt makes it (trm 0)."""
    MX = abi.MHandle(None, nrows=(B + 1) * MZ.nrows, ncols=MA.nrows,
                     wX=np.zeros(((B + 1) * MZ.nrows, abi.bsize(MA.nrows)), np.uint8))
    lib = kc.load_backend(backend)
    if backend == "oracle":
        lib.lako_set_d_mlt(C.c_longlong(1 << 32))
        lib.lako_xcalc(MA.mr_j.ctypes.data_as(C.c_void_p), MA.mr_b.ctypes.data_as(C.c_void_p),
                       MZ.mr_j.ctypes.data_as(C.c_void_p), MZ.mr_b.ctypes.data_as(C.c_void_p), L.ptr,
                       C.c_void_p(L.s.lf), MA.nrows, MZ.nrows, C.byref(MX.s), B, 0)
    else:
        from test_zz_no_alloc import _bind
        _bind(lib)
        px = C.pointer(MX.s)
        vpra = (C.c_void_p * 128)()
        lib.wrap_xcalc(C.byref(C.c_int(0)), C.cast(vpra, C.c_void_p), None, MA.mr_j.ctypes.data,
                       MA.mr_b.ctypes.data, MZ.mr_j.ctypes.data, MZ.mr_b.ctypes.data, L.ptr, L.s.lf,
                       C.byref(C.c_int(MA.nrows)), C.byref(C.c_int(MZ.nrows)), C.byref(px),
                       C.byref(C.c_int(B)), 0)
    return MX


def _subset_rows(W, snps, nrows):
    """Rows `snps` of the transpose of packed rows W (device tensor): a
    (len(snps), bsize(nrows)) packed array, MSB first."""
    import torch
    from lakcluster_c_gb300.large_pass import _pack_rows
    idx = torch.from_numpy(snps).to(W.device)
    byte = W[:, (idx // 8)].to(torch.int32)
    bits = ((byte >> (7 - (idx % 8)).to(torch.int32)) & 1).to(torch.bool)   # (nrows, k)
    return _pack_rows(bits.t().contiguous(), abi.bsize(nrows)).cpu().numpy()


def test_large_xcalc_and_bitplane_subset_equal_oracle(large):
    import torch
    lp, g, host = large
    MA, MZ = host[("A", 0)], host[("Z", 0)]
    (kind, nb1, nb2, sym), a, n = lp.args[0]
    assert (kind, nb1, nb2) == ("AnZt", 0, 0)
    scores = g.outputs()[0][:n].cpu().numpy()
    L = abi.LHandle(n)
    L.buf[:] = scores
    L.s.row_stride, L.s.col_stride = MA.rpop_b, MZ.rpop_b
    L.s.spacing_row = L.s.spacing_col = abi.SPACING_b
    MXg = _xcalc("gpu", lp, MA, MZ, L)
    MXo = _xcalc("oracle", lp, MA, MZ, L)
    for f in ("nrows", "ncols", "min_d", "max_d", "mlt_d", "ncols_per_z"):
        assert getattr(MXg.s, f) == getattr(MXo.s, f), f
    nbytes = MXo.s.nrows * MXo.s.mc_length
    assert np.array_equal(MXg.wX.reshape(-1)[:nbytes], MXo.wX.reshape(-1)[:nbytes])

    # the bit-plane product on a SNP subset (rows of At and Zt), bin 0 x bin 0
    rng = np.random.default_rng(5)
    snps = np.unique(np.concatenate([np.arange(256), rng.choice(np.arange(256, lp.ncols), 256, replace=False)]))
    assert snps.size == SUBSET_SNPS
    sel = np.zeros(lp.ncols, np.uint8)
    sel[snps] = 1
    nA, nZ = MA.nrows, MZ.nrows
    At = abi.MHandle(None, mr_b=sel, mr_j=sel, wX=_subset_rows(lp.A[0], snps, nA), nrows=lp.ncols, ncols=nA)
    Zt = abi.MHandle(None, mr_b=sel, mr_j=sel, wX=_subset_rows(lp.Z[0], snps, nZ), nrows=lp.ncols, ncols=nZ)
    Tt = abi.MHandle(np.ones((1, nA), np.uint8))
    St = abi.MHandle(np.ones((1, nZ), np.uint8))
    outs = {}
    for backend in ("oracle", "gpu"):
        lib = kc.load_backend(backend)
        out = C.POINTER(abi.L_handle)()
        aj = lp.A_ajdk.ctypes.data_as(C.POINTER(C.c_double))
        args = (abi.SPACING_a, abi.SPACING_a, At.ptr, Tt.ptr, MA.ptr, MZ.ptr, St.ptr, Zt.ptr, aj,
                C.pointer(MXg.s if backend == "gpu" else MXo.s), C.byref(out))
        if backend == "oracle":
            m = lib.lako_At_T_YnWt_S_Zn_ww(*args)
        else:
            m = lib.wrap_At_T_YnWt_S_Zn_ww__run(*kc._thread_args(), *args)
        outs[backend] = kc._take(out, m)
    assert outs["gpu"].size == lp.ncols
    got, want = outs["gpu"][snps], outs["oracle"][snps]
    assert np.count_nonzero(want) > SUBSET_SNPS // 2
    assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    torch.cuda.synchronize()
