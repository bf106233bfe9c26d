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
// Kernel: one CTA per 256 input records x 256 bit columns.  The CTA stages the
// 256 x 32-byte input tile in shared memory (each record's 32 bytes read by 32
// consecutive threads), each warp turns 32 x 32-bit sub-tiles around with
// __ballot_sync (one ballot per bit column gives the 32 input records' bits of
// one output record), and the 256 x 32-byte output tile leaves the same way.
// Every load and store of global memory is a byte in a contiguous 32-byte run
// per record, so the kernel streams at HBM rate.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "lakgb_runtime.cuh"

namespace lakgb {

namespace {

constexpr int kTR = 256;        // input records (and output bit columns) per CTA
constexpr int kTB = 32;         // input bytes per record per CTA (256 bit columns)
constexpr int kPitch = 36;      // shared row pitch in bytes (9 words: conflict-free word reads)

__global__ void __launch_bounds__(256) b16_transpose_kernel(const uint8_t *__restrict__ in, long long in_rec_bytes,
                                                           int n_in_rec, uint8_t *__restrict__ out,
                                                           long long out_rec_bytes, int n_out_rec) {
  __shared__ __align__(16) uint8_t tin[kTR * kPitch];
  __shared__ __align__(16) uint8_t tout[kTR * kPitch];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const long long rec0 = (long long)blockIdx.y * kTR;  // first input record of the tile
  const long long byte0 = (long long)blockIdx.x * kTB;  // first input byte (bit column / 8)
  // load: idx = record * 32 + byte; zeros outside the matrix
  for (int idx = tid; idx < kTR * kTB; idx += 256) {
    const int r = idx >> 5, b = idx & 31;
    const long long gr = rec0 + r, gb = byte0 + b;
    uint8_t v = 0;
    if (gr < n_in_rec && gb < in_rec_bytes) v = in[gr * in_rec_bytes + gb];
    tin[r * kPitch + b] = v;
  }
  __syncthreads();
  // 64 sub-tiles of 32 records x 32 bits, 8 per warp.  Sub-tile (rb, w):
  // records 32 rb + lane, bits 32 w .. 32 w + 31 (bytes 4 w .. 4 w + 3).
  for (int st = warp; st < (kTR / 32) * (kTB / 4); st += 8) {
    const int rb = st >> 3, w = st & 7;
    const uint32_t x = *reinterpret_cast<const uint32_t *>(tin + (32 * rb + lane) * kPitch + 4 * w);
    uint32_t mine = 0;
#pragma unroll
    for (int b = 0; b < 32; ++b) {
      // bit b of the sub-tile is bit 7 - b % 8 of byte b / 8, i.e. bit
      // 8 (b / 8) + 7 - b % 8 of the little-endian word
      const uint32_t m = __ballot_sync(0xffffffffu, (x >> (8 * (b >> 3) + 7 - (b & 7))) & 1u);
      if (lane == b) mine = m;
    }
    // ballot bit l = record 32 rb + l; output byte l / 8, bit 7 - l % 8:
    // reverse the bits, then the byte order
    const uint32_t o = __byte_perm(__brev(mine), 0, 0x0123);
    *reinterpret_cast<uint32_t *>(tout + (32 * w + lane) * kPitch + 4 * rb) = o;
  }
  __syncthreads();
  // store: output record = bit column byte0 * 8 + row, bytes rec0 / 8 + b
  const long long orec0 = byte0 * 8, obyte0 = rec0 / 8;
  for (int idx = tid; idx < kTR * kTB; idx += 256) {
    const int r = idx >> 5, b = idx & 31;
    const long long gr = orec0 + r, gb = obyte0 + b;
    if (gr < n_out_rec && gb < out_rec_bytes) out[gr * out_rec_bytes + gb] = tout[r * kPitch + b];
  }
}

}  // namespace

void launch_b16_transpose(const uint8_t *in, long long in_rec_bytes, int n_in_rec, uint8_t *out,
                          long long out_rec_bytes, int n_out_rec, cudaStream_t s) {
  if (n_in_rec <= 0 || in_rec_bytes <= 0) return;
  dim3 grid((unsigned)((in_rec_bytes + kTB - 1) / kTB), (unsigned)((n_in_rec + kTR - 1) / kTR));
  b16_transpose_kernel<<<grid, 256, 0, s>>>(in, in_rec_bytes, n_in_rec, out, out_rec_bytes, n_out_rec);
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
