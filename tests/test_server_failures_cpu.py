"""Failure isolation of the serving loop without a GPU: requests whose
problem description is invalid fail alone, with their own message, before
any device work; unknown ids are reported; destroy returns.  (Cancellation
and deadlines of requests that reach the GPU are covered by the GPU tests.)"""
import ctypes as C

import numpy as np

from lakcluster_c_gb300 import serve
from lakcluster_c_gb300.solve import BccBin, BccProblem


def _lib():
    from lakcluster_c_gb300 import build
    return serve.bind(C.CDLL(build.build_lib()))


def _bad_problem(kind):
    p = BccProblem()
    keep = []
    if kind == "no_bins":
        p.ncols, p.row_bytes, p.nbins = 100, 16, 0
    elif kind == "short_rows":
        rows = np.zeros((4, 2), np.uint8)
        keep.append(rows)
        bins = (BccBin * 1)()
        bins[0].A_nrows, bins[0].A_rows = 4, rows.ctypes.data
        keep.append(bins)
        p.ncols, p.row_bytes, p.nbins, p.bins = 100, 2, 1, bins
    elif kind == "null_rows":
        bins = (BccBin * 1)()
        bins[0].A_nrows, bins[0].A_rows = 4, None
        keep.append(bins)
        p.ncols, p.row_bytes, p.nbins, p.bins = 100, 16, 1, bins
    p.B_MLT, p.gamma = 32, 0.05
    return p, keep


def test_invalid_requests_fail_alone_with_their_messages():
    lib = _lib()
    s = lib.lakgb_server_create(2, 0)
    try:
        want = {"no_bins": b"bad problem description", "short_rows": b"row_bytes smaller",
                "null_rows": b"bad bin description"}
        ids, keep = {}, []
        for kind in want:
            p, k = _bad_problem(kind)
            keep.append((p, k))
            ids[kind] = lib.lakgb_server_submit_deadline(s, C.byref(p), 0.0)
            assert ids[kind] > 0
        for kind, id_ in ids.items():
            msg = C.create_string_buffer(256)
            rc = lib.lakgb_server_wait_msg(s, id_, None, None, msg, 256)
            assert rc == 2 and want[kind] in msg.value, (kind, rc, msg.value)
        # collected ids are gone; unknown ids are reported, not waited for
        assert lib.lakgb_server_wait(s, ids["no_bins"], None, None) == -1
        assert lib.lakgb_server_cancel(s, 12345) == -1
        assert lib.lakgb_server_wait(s, 12345, None, None) == -1
    finally:
        lib.lakgb_server_destroy(s)


def test_python_server_raises_solve_failed():
    import pytest
    lib = _lib()
    with serve.Server(2, lib=lib) as srv:
        p, keep = _bad_problem("short_rows")

        class P:  # the minimal shape Server.submit reads
            prob = p
        rid = srv.submit(P)
        with pytest.raises(serve.SolveFailed) as e:
            srv.wait(rid)
        assert e.value.rc == 2 and "row_bytes" in e.value.msg
