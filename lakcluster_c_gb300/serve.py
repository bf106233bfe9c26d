"""Many solves on one GPU: batched null instances and a served request stream.

Both run on the library's native server (lakgb_server_*, csrc/bcc_server.cpp):
worker threads that each drive whole solves on their own CUDA stream, with
admission by estimated device footprint against an HBM budget (continuous
batching).  The "plain" path for comparison solves the same problems one at a
time through lakgb_bcc_solve.
"""
from __future__ import annotations

import ctypes as C
import statistics
import threading
import time

import numpy as np

from ._lib import load
from .solve import BccProblem, BccResult, Problem, bind as bind_solve, format_outputs


def bind(lib):
    bind_solve(lib)
    lib.lakgb_server_create.argtypes = [C.c_int, C.c_longlong]
    lib.lakgb_server_create.restype = C.c_void_p
    lib.lakgb_server_submit.argtypes = [C.c_void_p, C.POINTER(BccProblem)]
    lib.lakgb_server_submit.restype = C.c_longlong
    lib.lakgb_server_submit_deadline.argtypes = [C.c_void_p, C.POINTER(BccProblem), C.c_double]
    lib.lakgb_server_submit_deadline.restype = C.c_longlong
    lib.lakgb_server_wait.argtypes = [C.c_void_p, C.c_longlong, C.POINTER(BccResult), C.POINTER(C.c_double)]
    lib.lakgb_server_wait.restype = C.c_int
    lib.lakgb_server_wait_msg.argtypes = [C.c_void_p, C.c_longlong, C.POINTER(BccResult), C.POINTER(C.c_double),
                                          C.c_char_p, C.c_int]
    lib.lakgb_server_wait_msg.restype = C.c_int
    lib.lakgb_server_cancel.argtypes = [C.c_void_p, C.c_longlong]
    lib.lakgb_server_cancel.restype = C.c_int
    lib.lakgb_server_peak_concurrency.argtypes = [C.c_void_p]
    lib.lakgb_server_peak_concurrency.restype = C.c_int
    lib.lakgb_server_destroy.argtypes = [C.c_void_p]
    lib.lakgb_bcc_footprint.argtypes = [C.POINTER(BccProblem)]
    lib.lakgb_bcc_footprint.restype = C.c_longlong
    return lib


def _result_lines(lib, res):
    try:
        n6, n2 = 6 * res.iterations, 2 * res.n_xdrop
        tr = np.ctypeslib.as_array(res.trace, (n6,)).copy() if n6 else np.zeros(0)
        xa = np.ctypeslib.as_array(res.xdrop_a, (n2,)).copy() if n2 else np.zeros(0, int)
        xb = np.ctypeslib.as_array(res.xdrop_b, (n2,)).copy() if n2 else np.zeros(0, int)
    finally:
        lib.lakgb_bcc_result_free(C.byref(res))
    return format_outputs(tr, xa, xb)


E_CANCELLED, E_DEADLINE = 6, 7  # LAKGB_E_CANCELLED, LAKGB_E_DEADLINE


class SolveFailed(RuntimeError):
    """A request that failed on the server (the others are unaffected)."""

    def __init__(self, rid: int, rc: int, msg: str):
        super().__init__("solve %d failed (%d): %s" % (rid, rc, msg))
        self.rid, self.rc, self.msg = rid, rc, msg


class Server:
    """Python handle on a native lakgb_server."""

    def __init__(self, workers: int = 8, hbm_budget_bytes: int = 0, lib=None):
        self.lib = bind(lib or load())
        self.h = self.lib.lakgb_server_create(workers, hbm_budget_bytes)

    def submit(self, p: Problem, deadline_s: float = 0.0) -> int:
        """Queue a problem; with deadline_s > 0 it fails with E_DEADLINE if it
        has not finished that many seconds after submission."""
        return self.lib.lakgb_server_submit_deadline(self.h, C.byref(p.prob), float(deadline_s))

    def wait(self, rid: int):
        """(output lines, (queueing, solving, total) seconds); raises
        SolveFailed with the library's message if the request failed."""
        res = BccResult()
        t = (C.c_double * 3)()
        msg = C.create_string_buffer(512)
        rc = self.lib.lakgb_server_wait_msg(self.h, rid, C.byref(res), t, msg, len(msg))
        if rc != 0:
            raise SolveFailed(rid, rc, msg.value.decode(errors="replace"))
        return _result_lines(self.lib, res), tuple(t)

    def cancel(self, rid: int) -> bool:
        """Cancel a queued or running request; False if it is unknown or done."""
        return self.lib.lakgb_server_cancel(self.h, rid) == 0

    def peak_concurrency(self) -> int:
        return self.lib.lakgb_server_peak_concurrency(self.h)

    def close(self):
        if self.h:
            self.lib.lakgb_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def solve_plain(problems):
    """One solve at a time (the plain path).  Returns (results, seconds)."""
    out = []
    t0 = time.perf_counter()
    for p in problems:
        out.append(p.solve())
    return out, time.perf_counter() - t0


def solve_batched(problems, workers=8, hbm_budget_bytes=0):
    """All problems at once on a server.  Returns (results, seconds, peak concurrency)."""
    with Server(workers, hbm_budget_bytes) as srv:
        t0 = time.perf_counter()
        ids = [srv.submit(p) for p in problems]
        out = [srv.wait(i)[0] for i in ids]
        secs = time.perf_counter() - t0
        peak = srv.peak_concurrency()
    return out, secs, peak


def serve_stream(problems, rate_per_s, workers=8, hbm_budget_bytes=0, seed=0):
    """Submit problems with Poisson inter-arrival times (mean 1/rate) while a
    collector waits for results.  Returns (results, per-request latency
    seconds, wall seconds, peak concurrency)."""
    rng = np.random.default_rng(seed)
    gaps = rng.exponential(1.0 / rate_per_s, len(problems))
    results = [None] * len(problems)
    lat = [None] * len(problems)
    with Server(workers, hbm_budget_bytes) as srv:
        ids = [None] * len(problems)
        ready = threading.Semaphore(0)

        def collect():
            for k in range(len(problems)):
                ready.acquire()
                out, t = srv.wait(ids[k])
                results[k] = out
                lat[k] = t[2]

        th = threading.Thread(target=collect)
        th.start()
        t0 = time.perf_counter()
        for k, p in enumerate(problems):
            time.sleep(gaps[k])
            ids[k] = srv.submit(p)
            ready.release()
        th.join()
        wall = time.perf_counter() - t0
        peak = srv.peak_concurrency()
    return results, lat, wall, peak


def latency_stats(lat):
    lat = sorted(lat)
    return {"p50_s": statistics.median(lat), "p99_s": float(np.percentile(lat, 99)), "mean_s": statistics.mean(lat)}
