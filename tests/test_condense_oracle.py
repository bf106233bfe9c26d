"""The condense row strategy's kernels without a GPU: the C oracle's
M_At_to_L2 / M_An_to_L2 / AnZt_mm (oracle/lak_oracle.c) against the
reference's own wrap_* compiled from its sources (oracle/_ref/liblakref.so,
where it exists) and against a numpy statement of the same arithmetic.  The
whole-solve goldens of the condense cases (tests/golden/bcc_traces.npz, from
the reference program) pin them again through the solve."""
import os

import numpy as np
import pytest

import kernel_cases as kc
from lakcluster_c_gb300 import abi

HAVE_REF = os.path.exists(kc.REF_LIB)


def to_l2_numpy(M, spec, A_ajdk, at):
    """Each retained entry (b - a) * sqrt(d) (or b) at its spacing's position."""
    s = M.s
    nr, nc = int(s.rpop_j), int(s.cpop_j)
    lr = {abi.SPACING_j: nr, abi.SPACING_b: int(s.rpop_b), abi.SPACING_a: int(s.nrows)}[spec["sr"]]
    lc = {abi.SPACING_j: nc, abi.SPACING_b: int(s.cpop_b), abi.SPACING_a: int(s.ncols)}[spec["sc"]]
    out = np.zeros(lr * lc)
    P = abi.psize(s.nrows if at else s.ncols)
    for r in range(nr):
        rb, ra = int(M.m_b_[r]), int(M.m_a_[r])
        bits = abi.unpack_bits(M.wX[rb], M.ncols)
        tr = {abi.SPACING_j: r, abi.SPACING_b: rb, abi.SPACING_a: ra}[spec["sr"]]
        for c in range(nc):
            cb, ca = int(M.n_b_[c]), int(M.n_a_[c])
            v = float(bits[ca]) if spec["type"] == abi.TYPE_00 else float(2 * int(bits[ca]) - 1)
            if A_ajdk is not None:
                snp = ra if at else ca
                v = (v - A_ajdk[snp // 1920 + 1 * P]) * np.sqrt(A_ajdk[snp // 1920 + 5 * P])
            tc = {abi.SPACING_j: c, abi.SPACING_b: cb, abi.SPACING_a: ca}[spec["sc"]]
            out[tr + tc * lr] = v
    return out


@pytest.mark.parametrize("at", [True, False])
@pytest.mark.parametrize("spec", kc.to_l2_specs(), ids=lambda s: s["name"])
def test_oracle_to_l2(spec, at):
    M, A_ajdk = kc.build_to_l2(spec, at)
    got, _ = kc.call_m_to_l2("oracle", at, spec["type"], spec["sr"], spec["sc"], M, A_ajdk)
    want = to_l2_numpy(M, spec, A_ajdk, at)
    assert got.tobytes() == want.tobytes()
    if HAVE_REF:
        ref, _ = kc.call_m_to_l2("ref", at, spec["type"], spec["sr"], spec["sc"], M, A_ajdk)
        assert got.tobytes() == ref.tobytes()


def test_oracle_to_l2_zeroes_the_whole_handle():
    spec = kc.to_l2_specs()[4]
    M, A_ajdk = kc.build_to_l2(spec)
    n = kc.call_m_to_l2("oracle", True, spec["type"], spec["sr"], spec["sc"], M, A_ajdk)[0].size
    buf, _ = kc.call_m_to_l2("oracle", True, spec["type"], spec["sr"], spec["sc"], M, A_ajdk, out_length=n + 50)
    assert not np.any(buf[n:])


@pytest.mark.parametrize("K,m,n,extra", kc.mm_specs())
def test_oracle_anzt_mm(K, m, n, extra):
    A, B, lfA, lfZ = kc.build_mm(K, m, n, extra, seed=K * 7 + m)
    got = kc.call_anzt_mm("oracle", lfA, lfZ)
    assert got.size == m * n
    # out[i + j*m] = sum_k A[k, i] * B[k, j]
    want = kc.mm_numpy(A, B[:K]).ravel(order="F") if K else np.zeros(m * n)
    assert got.tobytes() == want.tobytes()
    if HAVE_REF:
        assert got.tobytes() == kc.call_anzt_mm("ref", lfA, lfZ).tobytes()
