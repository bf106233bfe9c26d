"""GPU parity of the grouped Gram (lakgb_gram_group_*): the Gram passes of
several independent problems of different sizes (bins, rows, blocks;
symmetric and non-symmetric products, row terms) run as one persistent
launch of the tensor-core kernel give the same outputs, bit for bit, as one
launch per product with the tensor-core and with the popcount kernel, also
when the grouped launch is captured in a CUDA graph and replayed."""
import ctypes as C

import pytest

pytestmark = pytest.mark.gpu

POPCOUNT, TENSOR = 0, 1


@pytest.fixture(scope="module")
def passes():
    torch = pytest.importorskip("torch")
    from lakcluster_c_gb300.large_pass import GroupedGramPasses, LargeGramPass
    shapes = [(700, 500, 5000, 2, 11), (1300, 900, 9000, 3, 12), (300, 1100, 2500, 1, 13), (129, 257, 1920, 2, 14)]
    ps = [LargeGramPass(n_cases=a, n_controls=z, ncols=m, nbins=nb, planted=(min(64, a), min(128, m)), seed=sd)
          for a, z, m, nb, sd in shapes]
    g = GroupedGramPasses(ps)
    yield torch, g
    g.close()


def _snapshot(torch, g):
    torch.cuda.synchronize()
    return [o.clone() for o in g.outputs()]


def _fill(torch, g, v):
    for o in g.outputs():
        o.fill_(v)


def _bits(xs):
    import torch
    return [x.view(torch.int64) for x in xs]


def test_grouped_matches_per_launch(passes):
    torch, g = passes
    lib = g.lib
    before = lib.lakgb_gram_impl()
    try:
        want = {}
        for impl in (TENSOR, POPCOUNT):
            lib.lakgb_set_gram_impl(impl)
            _fill(torch, g, float("nan"))
            g.run_plain()
            want[impl] = _bits(_snapshot(torch, g))
            assert lib.lakgb_device_status() == 0
        for x, y in zip(want[TENSOR], want[POPCOUNT]):
            assert torch.equal(x, y)
        _fill(torch, g, float("nan"))
        g.run_grouped()
        got = _bits(_snapshot(torch, g))
        assert lib.lakgb_device_status() == 0
        assert len(got) == g.n == sum(len(p.args) for p in g.passes)
        for i, (x, y) in enumerate(zip(got, want[TENSOR])):
            assert torch.equal(x, y), i
    finally:
        lib.lakgb_set_gram_impl(before)


def test_grouped_launch_in_cuda_graph(passes):
    torch, g = passes
    lib = g.lib
    before = lib.lakgb_gram_impl()
    lib.lakgb_set_gram_impl(TENSOR)
    try:
        _fill(torch, g, float("nan"))
        g.run_plain()
        want = _bits(_snapshot(torch, g))
        s = torch.cuda.Stream()
        graph = torch.cuda.CUDAGraph()
        g.run_grouped(s.cuda_stream)  # warm (module load, attributes) outside the capture
        torch.cuda.synchronize()
        with torch.cuda.stream(s):
            with torch.cuda.graph(graph, stream=s):
                g.run_grouped(s.cuda_stream)
        for _ in range(2):
            _fill(torch, g, float("nan"))
            torch.cuda.synchronize()
            graph.replay()
            got = _bits(_snapshot(torch, g))
            for i, (x, y) in enumerate(zip(got, want)):
                assert torch.equal(x, y), i
        assert lib.lakgb_device_status() == 0
    finally:
        lib.lakgb_set_gram_impl(before)


def test_group_rejects_mixed_types(passes):
    torch, g = passes
    from lakcluster_c_gb300 import abi
    from lakcluster_c_gb300.gram_pass import GramArgs
    a0 = g.items[0][2]
    a1 = GramArgs.from_buffer_copy(a0)
    a1.type_flag = abi.TYPE_00 if a0.type_flag == abi.TYPE_pm else abi.TYPE_pm
    arr = (GramArgs * 2)(a0, a1)
    assert not g.lib.lakgb_gram_group_create(C.cast(arr, C.c_void_p), 2)
    buf = C.create_string_buffer(256)
    assert g.lib.lakgb_last_error(buf, 256) != 0  # reading the error clears it
    assert b"type unlike instance 0" in buf.value
