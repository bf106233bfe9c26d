// Bit-matrix transpose of .b16 data: the reference's wrap_transpose
// (dir_c/binary_read.c:174-269), which converts a .b16 file of n_col records
// of n_row bits each into a .b16 file of n_row records of n_col bits, slowly,
// a few rows at a time through a small workspace.  Here the whole matrix goes
// through HBM once in each direction.
//
// Layout (both directions): a record is a row of bits, MSB first within each
// byte, padded with zero bits to a multiple of bitj (16 in every .b16 file of
// this project); record r starts at byte r * record_bytes.  Output record i
// holds bit i of every input record, in input-record order; its padding bits
// (input records past the last) are zero, as the reference clears them
// (binary_read.c:247-255).
//
// Kernels: a CTA stages a tile of 256 input records in shared memory (a
// contiguous run of each record's bytes, read by consecutive threads), each
// warp turns 32 x 32-bit sub-tiles around in registers (the recursive
// block-swap transpose: five exchanges of half-words, quarter-words, ...
// between lanes 16, 8, 4, 2, 1 apart), and the output leaves in contiguous
// runs of each output record.  When every record of both sides is a multiple
// of 16 bytes long (all large matrices), loads and stores are 16 bytes wide
// and each lane stores its output record's 32 bytes straight from registers
// (b16_transpose16_kernel: 128-byte input runs, 0.35 ms for 512 MB each way,
// 3.1 TB/s); otherwise 4-byte or 1-byte accesses through an output tile in
// shared memory.  Larger tiles (512 or 1024 records, 256-byte runs) measured
// slower: fewer CTAs fit on an SM.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "bit_transpose.cuh"
#include "lakgb_runtime.cuh"

namespace lakgb {

namespace {

constexpr int kTR = 256;        // input records (and output bit columns) per CTA
constexpr int kTB = 32;         // input bytes per record per CTA (256 bit columns)
constexpr int kR16 = 256;       // input records per CTA on the 16-byte path
constexpr int kTB16 = 128;      // input bytes of each record per CTA on the 16-byte path
constexpr int kPitch = 36;      // shared row pitch in bytes (9 words: conflict-free word reads)

// V: bytes per global access (1 or 4); TB: input bytes of each record
// per CTA (TB * 8 bit columns, i.e. output records, per CTA).
template <int V, int TB>
__global__ void __launch_bounds__(256) b16_transpose_kernel(const uint8_t *__restrict__ in, long long in_rec_bytes,
                                                           int n_in_rec, uint8_t *__restrict__ out,
                                                           long long out_rec_bytes, int n_out_rec) {
  constexpr int kInPitch = TB + 4;  // odd number of words: conflict-free word reads down a column
  extern __shared__ __align__(16) uint8_t tsm[];
  uint8_t *tin = tsm;                          // [kTR][kInPitch]
  uint8_t *tout = tsm + kTR * kInPitch;        // [TB * 8][kPitch]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long rec0 = (long long)blockIdx.y * kTR;  // first input record of the tile
  const long long byte0 = (long long)blockIdx.x * TB;  // first input byte (bit column / 8)
  // load, zeros outside the matrix (a record's length is a multiple of V, so
  // an access is wholly inside or wholly outside it)
  for (int idx = tid; idx < kTR * (TB / V); idx += 256) {
    const int r = idx / (TB / V), k = idx % (TB / V);
    const long long gr = rec0 + r, gb = byte0 + (long long)V * k;
    const bool inside = gr < n_in_rec && gb < in_rec_bytes;
    uint8_t *d = tin + r * kInPitch + V * k;
    if (V == 4) {
      *reinterpret_cast<uint32_t *>(d) = inside ? *reinterpret_cast<const uint32_t *>(in + gr * in_rec_bytes + gb) : 0u;
    } else {
      *d = inside ? in[gr * in_rec_bytes + gb] : (uint8_t)0;
    }
  }
  __syncthreads();
  // sub-tiles of 32 records x 32 bits.  Sub-tile (rb, w): records 32 rb +
  // lane, bits 32 w .. 32 w + 31 (bytes 4 w .. 4 w + 3).  Byte-swapping the
  // little-endian word puts bit column c at bit 31 - c (bytes hold their bits
  // MSB first); after the transpose, lane l holds output record 32 w + l with
  // input record 32 rb + c at bit 31 - c, and the byte swap back gives its 4
  // bytes in file order.
  for (int st = warp; st < (kTR / 32) * (TB / 4); st += 8) {
    const int rb = st / (TB / 4), w = st % (TB / 4);
    const uint32_t x = *reinterpret_cast<const uint32_t *>(tin + (32 * rb + lane) * kInPitch + 4 * w);
    const uint32_t y = transpose32(__byte_perm(x, 0, 0x0123), lane);
    *reinterpret_cast<uint32_t *>(tout + (32 * w + lane) * kPitch + 4 * rb) = __byte_perm(y, 0, 0x0123);
  }
  __syncthreads();
  // store: output record = bit column byte0 * 8 + row, its bytes rec0 / 8 ..
  // rec0 / 8 + 31
  const long long orec0 = byte0 * 8, obyte0 = rec0 / 8;
  for (int idx = tid; idx < TB * 8 * (kTB / V); idx += 256) {
    const int r = idx / (kTB / V), k = idx % (kTB / V);
    const long long gr = orec0 + r, gb = obyte0 + (long long)V * k;
    if (gr >= n_out_rec || gb >= out_rec_bytes) continue;
    const uint8_t *sp = tout + r * kPitch + V * k;
    if (V == 4) {
      *reinterpret_cast<uint32_t *>(out + gr * out_rec_bytes + gb) = *reinterpret_cast<const uint32_t *>(sp);
    } else {
      out[gr * out_rec_bytes + gb] = *sp;
    }
  }
}

// The 16-byte path: records of both sides a multiple of 16 bytes long.
// Input: one tile of R records x TB bytes (uint4 loads: TB contiguous bytes
// of each record); then for each of its word columns w a warp turns the
// R / 32 sub-tiles of that column around, so that lane l holds all R / 8
// bytes of output record 32 w + l that the tile covers, and stores them
// straight from registers as 16-byte writes.  No output tile, one barrier.
template <int R, int TB>
__global__ void __launch_bounds__(256) b16_transpose16_kernel(const uint8_t *__restrict__ in, long long in_rec_bytes,
                                                             int n_in_rec, uint8_t *__restrict__ out,
                                                             long long out_rec_bytes, int n_out_rec) {
  constexpr int kInPitch = TB + 4;  // an odd number of words: conflict-free reads down a column
  extern __shared__ __align__(16) uint8_t tin[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long rec0 = (long long)blockIdx.y * R;
  const long long byte0 = (long long)blockIdx.x * TB;
  for (int idx = tid; idx < R * (TB / 16); idx += 256) {
    const int r = idx / (TB / 16), k = idx % (TB / 16);
    const long long gr = rec0 + r, gb = byte0 + 16ll * k;
    const uint4 v = (gr < n_in_rec && gb < in_rec_bytes) ? *reinterpret_cast<const uint4 *>(in + gr * in_rec_bytes + gb)
                                                          : make_uint4(0, 0, 0, 0);
    uint32_t *dw = reinterpret_cast<uint32_t *>(tin + r * kInPitch + 16 * k);
    dw[0] = v.x; dw[1] = v.y; dw[2] = v.z; dw[3] = v.w;
  }
  __syncthreads();
  for (int w = warp; w < TB / 4; w += 8) {  // word column: output records 32 w .. 32 w + 31 of the tile
    uint32_t o[R / 32];
#pragma unroll
    for (int rb = 0; rb < R / 32; ++rb) {
      const uint32_t x = *reinterpret_cast<const uint32_t *>(tin + (32 * rb + lane) * kInPitch + 4 * w);
      o[rb] = __byte_perm(transpose32(__byte_perm(x, 0, 0x0123), lane), 0, 0x0123);
    }
    const long long gr = byte0 * 8 + 32 * w + lane, gb = rec0 / 8;
    if (gr < n_out_rec) {
      uint8_t *dst = out + gr * out_rec_bytes + gb;
#pragma unroll
      for (int q = 0; q < R / 128; ++q)
        if (gb + 16 * q < out_rec_bytes)
          *reinterpret_cast<uint4 *>(dst + 16 * q) = make_uint4(o[4 * q], o[4 * q + 1], o[4 * q + 2], o[4 * q + 3]);
    }
  }
}

template <int V, int TB>
void launch_v(const uint8_t *in, long long in_rec_bytes, int n_in_rec, uint8_t *out, long long out_rec_bytes,
              int n_out_rec, cudaStream_t s) {
  const size_t smem = (size_t)kTR * (TB + 4) + (size_t)TB * 8 * kPitch;
  static bool configured = false;
  if (!configured) {
    LAKGB_CUDA(cudaFuncSetAttribute(b16_transpose_kernel<V, TB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem));
    configured = true;
  }
  dim3 grid((unsigned)((in_rec_bytes + TB - 1) / TB), (unsigned)((n_in_rec + kTR - 1) / kTR));
  b16_transpose_kernel<V, TB><<<grid, 256, smem, s>>>(in, in_rec_bytes, n_in_rec, out, out_rec_bytes, n_out_rec);
}

}  // namespace

void launch_b16_transpose(const uint8_t *in, long long in_rec_bytes, int n_in_rec, uint8_t *out,
                          long long out_rec_bytes, int n_out_rec, cudaStream_t s) {
  if (n_in_rec <= 0 || in_rec_bytes <= 0) return;
  // widest access that every record of both sides allows: a record length
  // that is a multiple of the width and a buffer aligned to it put every
  // record's start on that boundary
  auto fits = [&](int v) {
    return in_rec_bytes % v == 0 && out_rec_bytes % v == 0 && ((uintptr_t)in % v) == 0 && ((uintptr_t)out % v) == 0;
  };
  if (fits(16)) {
    constexpr int R = kR16, TB = kTB16;
    constexpr size_t smem = (size_t)R * (TB + 4);
    static bool configured = false;
    if (!configured) {
      LAKGB_CUDA(cudaFuncSetAttribute(b16_transpose16_kernel<R, TB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
      configured = true;
    }
    dim3 grid((unsigned)((in_rec_bytes + TB - 1) / TB), (unsigned)((n_in_rec + R - 1) / R));
    b16_transpose16_kernel<R, TB><<<grid, 256, smem, s>>>(in, in_rec_bytes, n_in_rec, out, out_rec_bytes, n_out_rec);
  } else if (fits(4))
    launch_v<4, kTB>(in, in_rec_bytes, n_in_rec, out, out_rec_bytes, n_out_rec, s);
  else
    launch_v<1, kTB>(in, in_rec_bytes, n_in_rec, out, out_rec_bytes, n_out_rec, s);
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
}

}  // namespace lakgb

using namespace lakgb;

// Device entry: n_records input records of n_bits bits each (records padded to
// 16 bits) -> n_bits records of n_records bits (padded to 16 bits).
extern "C" int lakgb_bits_transpose_device(const unsigned char *in, int n_records, int n_bits, unsigned char *out,
                                           void *stream) {
  if (!in || !out || n_records < 0 || n_bits < 0) {
    set_error(3, "lakgb_bits_transpose_device: bad arguments");
    return -1;
  }
  const long long in_rec = 2ll * ((n_bits + 15) / 16), out_rec = 2ll * ((n_records + 15) / 16);
  launch_b16_transpose(in, in_rec, n_records, out, out_rec, n_bits, stream ? (cudaStream_t)stream : lakgb::stream());
  return 0;
}

// The reference's wrap_transpose (dir_c/binary_read.c:174): reads the .b16
// file fname_0in (header bitj, n_row, n_col as ints; then n_col records of
// n_row bits padded to bitj), writes fname_out (header bitj, n_col, n_row;
// n_row records of n_col bits padded to bitj).  n_bytes_per_read only sized
// the reference's workspace and is not needed here.  Problems are reported
// as the reference reports them (a printed warning) and recorded in
// lakgb_last_error.
extern "C" void wrap_transpose(char *fname_0in, char *fname_out, int n_bytes_per_read) {
  LAKGB_PROFILE_CALL("wrap_transpose");
  (void)n_bytes_per_read;
  FILE *fi = fopen(fname_0in, "rb");
  if (!fi) {
    printf(" Warning! cannot open %s in wrap_transpose\n", fname_0in);
    set_error(4, "wrap_transpose: cannot open %s", fname_0in);
    return;
  }
  int hdr[3] = {0, 0, 0};
  if (fread(hdr, sizeof(int), 3, fi) != 3 || hdr[0] <= 0 || hdr[0] % 8 || hdr[1] < 0 || hdr[2] < 0) {
    fclose(fi);
    printf(" Warning! bad header in %s in wrap_transpose\n", fname_0in);
    set_error(4, "wrap_transpose: bad header in %s", fname_0in);
    return;
  }
  const int bitj = hdr[0], n_row = hdr[1], n_col = hdr[2];
  const long long in_rec = (long long)(n_row + (bitj - n_row % bitj) % bitj) / 8;
  const long long out_rec = (long long)(n_col + (bitj - n_col % bitj) % bitj) / 8;
  const size_t in_bytes = (size_t)in_rec * (size_t)n_col, out_bytes = (size_t)out_rec * (size_t)n_row;
  std::vector<unsigned char> h_in(in_bytes ? in_bytes : 1), h_out(out_bytes ? out_bytes : 1);
  const size_t got = in_bytes ? fread(h_in.data(), 1, in_bytes, fi) : 0;
  fclose(fi);
  if (got != in_bytes) {
    printf(" Warning! %s is shorter than its header says in wrap_transpose\n", fname_0in);
    set_error(4, "wrap_transpose: %s is truncated", fname_0in);
    return;
  }
  if (in_bytes && out_bytes) {
    cudaStream_t s = lakgb::stream();
    DBuf d_in(in_bytes), d_out(out_bytes);
    d_in.upload(h_in.data(), in_bytes);
    launch_b16_transpose(d_in.as<uint8_t>(), in_rec, n_col, d_out.as<uint8_t>(), out_rec, n_row, s);
    LAKGB_CUDA(cudaMemcpyAsync(h_out.data(), d_out.p, out_bytes, cudaMemcpyDeviceToHost, s));
    LAKGB_CUDA(cudaStreamSynchronize(s));
  }
  FILE *fo = fopen(fname_out, "wb");
  if (!fo) {
    printf(" Warning! cannot open %s in wrap_transpose\n", fname_out);
    set_error(4, "wrap_transpose: cannot open %s", fname_out);
    return;
  }
  const int ohdr[3] = {bitj, n_col, n_row};
  bool ok = fwrite(ohdr, sizeof(int), 3, fo) == 3;
  if (out_bytes) ok = ok && fwrite(h_out.data(), 1, out_bytes, fo) == out_bytes;
  if (fclose(fo) != 0 || !ok) set_error(4, "wrap_transpose: short write to %s", fname_out);
}
