"""Many solves on one GPU: every result in a batch or a served mix must equal
the same problem solved alone (and, for the golden cases, the reference)."""
import pytest

import bcc_cases as bc

pytestmark = pytest.mark.gpu


def _problems():
    from lakcluster_c_gb300 import solve as sv, synth
    probs, names = [], []
    for name in ["case_only_200x300", "case_control_2bin_masked", "case_control_3bin_ragged"]:
        d = bc.build(name)
        probs.append(sv.Problem(d["A"], d.get("Z"), gamma=d["gamma"], A_masks=d.get("A_masks"),
                                Z_masks=d.get("Z_masks"), col_mask=d.get("col_mask")))
        names.append(name)
    for seed in range(3):
        inst = synth.served_request(100 + seed, rows=(256, 1024), cols=(1024, 4096))
        probs.append(sv.Problem(inst.A_bins, inst.Z_bins, gamma=0.05))
        names.append(None)
    for seed in range(2):
        inst = synth.null_instance(200 + seed, rows=(256, 1024), cols=(1024, 4096))
        probs.append(sv.Problem(inst.A_bins, inst.Z_bins, gamma=0.05))
        names.append(None)
    return probs, names


def test_batch_results_equal_solo(gpu_lib):
    from lakcluster_c_gb300 import serve
    probs, names = _problems()
    golden = bc.load_golden()
    solo = [p.solve() for p in probs]
    for out, name in zip(solo, names):
        if name:
            assert out == {k: golden[name][k] for k in ("trace", "xdrop_a", "xdrop_b")}, name
    batched, secs, peak = serve.solve_batched(probs, workers=4)
    assert peak >= 2
    for k, (a, b) in enumerate(zip(batched, solo)):
        assert a == b, "problem %d differs in the batch" % k


def test_served_stream_results_equal_solo(gpu_lib):
    from lakcluster_c_gb300 import serve
    probs, _ = _problems()
    solo = [p.solve() for p in probs]
    mixed, lat, wall, peak = serve.serve_stream(probs * 2, rate_per_s=200.0, workers=3, seed=1)
    for k, out in enumerate(mixed):
        assert out == solo[k % len(probs)], "request %d differs in the mix" % k
    assert all(x > 0 for x in lat)


def test_budget_admission_serialises_when_tight(gpu_lib):
    """With a budget smaller than two solves, the server runs one at a time."""
    from lakcluster_c_gb300 import serve
    probs, _ = _problems()
    lib = serve.bind(probs[0].lib)
    import ctypes as C
    fp = [lib.lakgb_bcc_footprint(C.byref(p.prob)) for p in probs[:4]]
    budget = min(fp) + 1
    out, secs, peak = serve.solve_batched(probs[:4], workers=4, hbm_budget_bytes=budget)
    assert peak == 1
    assert out == [p.solve() for p in probs[:4]]


def _long_problem():
    """A solve of about two seconds (the 4096 + 4096 x 16384 two-bin case)."""
    from lakcluster_c_gb300 import solve as sv
    d = bc.build("case_control_4096x4096x16384")
    return sv.Problem(d["A"], d["Z"], gamma=d["gamma"])


def test_cancel_running_and_queued_requests(gpu_lib):
    import time
    from lakcluster_c_gb300 import serve
    probs, names = _problems()
    small = probs[1]
    want = small.solve()
    with serve.Server(1) as srv:
        long_id = srv.submit(_long_problem())
        queued = srv.submit(small)
        time.sleep(0.5)                       # the long solve is running, the small one queued
        assert srv.cancel(queued)
        t0 = time.perf_counter()
        with pytest.raises(serve.SolveFailed) as e:
            srv.wait(queued)
        assert e.value.rc == serve.E_CANCELLED and time.perf_counter() - t0 < 0.5
        assert srv.cancel(long_id)
        with pytest.raises(serve.SolveFailed) as e:
            srv.wait(long_id)
        assert e.value.rc == serve.E_CANCELLED and "cancelled" in e.value.msg
        assert not srv.cancel(long_id)        # collected: unknown now
        # the worker and the device are fine afterwards
        out, _ = srv.wait(srv.submit(small))
        assert out == want


def test_deadline_of_a_queued_request(gpu_lib):
    import time
    from lakcluster_c_gb300 import serve
    probs, _ = _problems()
    with serve.Server(1) as srv:
        long_id = srv.submit(_long_problem())
        time.sleep(0.3)
        t0 = time.perf_counter()
        rid = srv.submit(probs[0], deadline_s=0.2)
        with pytest.raises(serve.SolveFailed) as e:
            srv.wait(rid)
        waited = time.perf_counter() - t0
        assert e.value.rc == serve.E_DEADLINE and 0.15 < waited < 1.0, waited
        srv.wait(long_id)                     # the running solve is unaffected


def test_destroy_releases_waiters_of_queued_requests(gpu_lib):
    import threading
    import time
    from lakcluster_c_gb300 import serve
    probs, _ = _problems()
    srv = serve.Server(1)
    srv.submit(_long_problem())
    rid = srv.submit(probs[0])
    got = {}

    def waiter():
        try:
            srv.wait(rid)
            got["rc"] = 0
        except serve.SolveFailed as e:
            got["rc"] = e.rc

    th = threading.Thread(target=waiter)
    th.start()
    time.sleep(0.3)
    t0 = time.perf_counter()
    srv.close()                               # cancels the running solve, fails the queued one
    th.join(timeout=10)
    assert not th.is_alive() and got["rc"] == serve.E_CANCELLED
    assert time.perf_counter() - t0 < 5.0


def test_footprint_estimate_covers_device_memory_held(gpu_lib):
    """The admission estimate is an upper bound of the device memory a solve
    holds at its peak (the library's pool high-water mark), and not far above."""
    import ctypes as C
    import torch
    from lakcluster_c_gb300 import serve, solve as sv, synth
    lib = serve.bind(gpu_lib)
    lib.lakgb_pool_high_water.argtypes = [C.c_int]
    lib.lakgb_pool_high_water.restype = C.c_longlong
    torch.cuda.synchronize()
    for seed, rows, cols in [(11, (512, 1024), (2048, 4096)), (12, (2048, 4096), (8192, 16384)),
                             (13, (4096, 8192), (16384, 32768))]:
        inst = synth.served_request(seed, rows=rows, cols=cols)
        p = sv.Problem(inst.A_bins, inst.Z_bins, gamma=0.05)
        est = lib.lakgb_bcc_footprint(C.byref(p.prob))
        base = lib.lakgb_pool_high_water(1)
        lib.lakgb_pool_high_water(1)
        p.solve()
        held = lib.lakgb_pool_high_water(0)
        assert held <= est, (seed, held, est)
        assert est <= 8 * max(held, 1 << 26), (seed, held, est)
        del base


def test_tensor_pipeline_wait_runs_out_and_recovers(gpu_lib):
    """A withheld arrival makes a wait of the tensor Gram's pipeline run out:
    the kernel returns, the status word is set and the next launch (its
    tensor memory freed) computes the right answer."""
    import ctypes as C
    import numpy as np
    import kernel_cases as kc
    from lakcluster_c_gb300 import abi
    lib = kc.load_backend("gpu")
    lib.lakgb_debug_tc_pipeline.argtypes = [C.c_ulonglong, C.c_int]
    rng = np.random.default_rng(3)
    A, ar_b, ar_j = kc.make_matrix_case(rng, 100, 3000)
    Z, zr_b, zr_j = kc.make_matrix_case(rng, 90, 3000)
    mc = np.ones(3000, np.uint8)
    MA, MZ = kc.mhandle(A, ar_b, ar_j, mc, mc), kc.mhandle(Z, zr_b, zr_j, mc, mc)
    A_ajdk = abi.calc_A_ajdk(0.1 + 0.8 * rng.random(abi.psize(3000)))
    want = kc.call_gram("oracle", False, abi.TYPE_pm, abi.SPACING_b, abi.SPACING_b, MA, MZ, A_ajdk, None, None)
    before = lib.lakgb_gram_impl()
    lib.lakgb_set_gram_impl(1)                # the tensor-core kernel
    try:
        assert lib.lakgb_device_status() == 0
        lib.lakgb_debug_tc_pipeline(1000000, 1)   # 1 ms limit, one arrival withheld
        try:
            kc.call_gram("gpu", False, abi.TYPE_pm, abi.SPACING_b, abi.SPACING_b, MA, MZ, A_ajdk, None, None)
            # 4: the MMA warp's wait for the withheld stage ran out (it waits
            # first; the other roles then stop on the CTA's abort flag)
            assert lib.lakgb_device_status() != 0
        finally:
            lib.lakgb_debug_tc_pipeline(0, 0)
        got = kc.call_gram("gpu", False, abi.TYPE_pm, abi.SPACING_b, abi.SPACING_b, MA, MZ, A_ajdk, None, None)
        assert lib.lakgb_device_status() == 0
        assert np.array_equal(got.view(np.uint64), want.view(np.uint64))
    finally:
        lib.lakgb_set_gram_impl(before)
