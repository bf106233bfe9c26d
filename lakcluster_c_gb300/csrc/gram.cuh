// Device entry for the +/-1 Gram (AnZt_vv / AnAt_vv) on device-resident data.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace lakgb {

struct GramParams {
  const uint8_t *wA;       // packed rows of A (row r at wA + a_rowb[i]*a_row_bytes)
  const uint32_t *a_rowb;  // wX row of the i-th retained A row (M_An->m_b_)
  int nA;
  long long a_row_bytes;   // M_An->mc_length
  const uint8_t *wZ;
  const uint32_t *z_rowb;
  int nZ;
  long long z_row_bytes;
  const uint8_t *mask;     // M_An->mc_j, P*240 bytes
  int P;                   // number of 1920-bit blocks
  const double *D;         // A_ajdk + AJDK_0_1*P, or null (unweighted counts)
  int type;                // 1: XOR (TYPE_pm), 2: AND (TYPE_00)
  double a0d1, a2d1;       // sum_blocks D*popcnt(mask) and sum_blocks alpha^2 D*popcnt(mask)
  const double *lfA;       // AJDK_1_1 row term per retained A row, or null
  const double *lfZ;       // AJDK_1_1 row term per retained Z row, or null
  const uint32_t *out_r;   // output row index of the i-th A row
  const uint32_t *out_c;   // output column index of the k-th Z row
  const uint32_t *out_r2;  // symmetric only: output row index of the k-th Z row
  const uint32_t *out_c2;  // symmetric only: output column index of the i-th A row
  long long out_stride;    // row_stride of the output
  double *out;
  int symmetric;           // AnAt: compute pairs i<=k only and mirror them
  cudaStream_t stream;     // launch stream (null: the library stream)
};

// Several independent Grams launched as one (the tensor-core kernel's grouped
// form): their parameters, the prefix sums of their tile counts (n + 1) and
// of their block counts (n + 1, rows of the table array), all in device
// memory.  Every instance has the same type; a symmetric instance has a
// square tile grid.
struct GramGroupDev {
  const GramParams *ps;
  const int *tile0;
  const long long *blk0;
  int n;
};

// Tiles of one Gram on the tensor-core kernel's 128 x 128 grid (symmetric
// with a square grid: the upper triangle).
int gram_tc_tiles(const GramParams &p);

// Enqueue the grouped tensor-core Gram on stream s: the table kernel for all
// instances' blocks into T (total_blocks x 1922 doubles), then one
// persistent launch over all instances' tiles.
void launch_gram_tc_group(const GramGroupDev &g, int type, int total_tiles, long long total_blocks, double *T,
                          cudaStream_t s);
// Bytes of one table row (per instance block) of the grouped launch.
size_t gram_tc_table_row_bytes();

// Enqueue the Gram kernel on the library stream: the tensor-core kernel
// (gram_tc.cu) or the popcount kernel (gram.cu), as lakgb_set_gram_impl selects.
void launch_gram(const GramParams &p);

// The tensor-core Gram (gram_tc.cu) on stream s.
void launch_gram_tc(const GramParams &p, cudaStream_t s);

// Read and clear the device status word of the tensor-core kernels
// (0 = no pipeline error).
int tc_status_take();
int tc_status_take_stream();
// Device address of that status word, for tensor-core kernels of other
// translation units.
int *tc_status_device_ptr();
// Test hooks of the tensor-core pipelines: wall-time limit of a wait (ns) and
// the withheld arrival (lakgb_debug_tc_pipeline).
void tc_debug_set(unsigned long long wait_ns, int withhold);

// Algorithmic bit-ops of one Gram launch: rows_A * rows_Z * retained columns
// (the full square for the symmetric variant, as the reference counts it).
double gram_bitops(const GramParams &p, long long retained_cols);

}  // namespace lakgb
