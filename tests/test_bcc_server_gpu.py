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
