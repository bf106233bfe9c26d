"""GPU parity of the .b16 transpose: the library's wrap_transpose (file to
file, dir_c/binary_read.c:174 signature) reproduces the reference's golden
output files byte for byte and the C oracle on larger ragged matrices; the
device entry (lakgb_bits_transpose_device) matches the oracle and is its own
inverse; a missing input file is reported, not fatal."""
import ctypes as C

import numpy as np
import pytest

import kernel_cases as kc
import transpose_cases as tc

pytestmark = pytest.mark.gpu


def test_wrap_transpose_matches_reference_golden(gpu_lib, tmp_path):
    d = np.load(tc.GOLDEN)
    for i in range(len(tc.SHAPES)):
        src, dst = str(tmp_path / ("g%d.b16" % i)), str(tmp_path / ("g%d_t.b16" % i))
        open(src, "wb").write(d["case%02d/in" % i].tobytes())
        assert tc.file_transpose("gpu", src, dst) == d["case%02d/out" % i].tobytes(), tc.SHAPES[i]


@pytest.mark.parametrize("n,m,p", [(3000, 5000, 0.5), (70001, 300, 0.2), (300, 70001, 0.7), (4097, 4111, 0.01),
                                   (4096, 8192, 0.5), (96, 1056, 0.4), (33, 4128, 0.6)])
def test_wrap_transpose_matches_oracle_large(gpu_lib, tmp_path, n, m, p):
    rng = np.random.default_rng(n * 7 + m)
    x = (rng.random((n, m)) < p).astype(np.uint8)
    src, dst = str(tmp_path / "x.b16"), str(tmp_path / "x_t.b16")
    raw = tc.write_file(src, x)
    assert tc.file_transpose("gpu", src, dst) == tc.oracle_transpose(raw)


@pytest.mark.parametrize("n,m", [(2345, 3071), (2048, 3072)])  # byte access; word access
def test_device_transpose_round_trip(gpu_lib, n, m):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5)
    in_rec, out_rec = 2 * ((m + 15) // 16), 2 * ((n + 15) // 16)
    x = (rng.random((n, m)) < 0.5).astype(np.uint8)
    packed = np.zeros((n, in_rec), np.uint8)
    packed[:, : (m + 7) // 8] = np.packbits(x, axis=1)
    want = np.zeros(out_rec * m, np.uint8)
    kc.load_backend("oracle").lako_bits_transpose(packed.ctypes.data_as(C.c_void_p), C.c_longlong(in_rec), n,
                                                  want.ctypes.data_as(C.c_void_p), C.c_longlong(out_rec), m)
    d_in = torch.from_numpy(packed.ravel()).cuda()
    d_out = torch.full((out_rec * m,), 0xAB, dtype=torch.uint8, device="cuda")
    d_back = torch.full((in_rec * n,), 0xCD, dtype=torch.uint8, device="cuda")
    assert gpu_lib.lakgb_bits_transpose_device(d_in.data_ptr(), n, m, d_out.data_ptr(), None) == 0
    assert gpu_lib.lakgb_bits_transpose_device(d_out.data_ptr(), m, n, d_back.data_ptr(), None) == 0
    torch.cuda.synchronize()
    assert np.array_equal(d_out.cpu().numpy(), want)
    assert np.array_equal(d_back.cpu().numpy(), packed.ravel())


def test_missing_file_is_reported(gpu_lib, tmp_path):
    gpu_lib.wrap_transpose(str(tmp_path / "none.b16").encode(), str(tmp_path / "o.b16").encode(), 8)
    buf = C.create_string_buffer(256)
    assert gpu_lib.lakgb_last_error(buf, 256) != 0
    assert b"cannot open" in buf.value
