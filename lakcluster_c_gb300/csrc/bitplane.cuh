// Parameters of the bit-plane loop product At_T_YnWt_S_Zn_ww shared by its
// CUDA-core kernel (bitplane.cu) and its tensor-core kernel (bitplane_tc.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace lakgb {

struct BitplaneParams {
  // At / Tt / planes share the row length `kbytes` (patients, a-space bits).
  const uint8_t *At; const uint32_t *at_rowb;   // per pair: At row (b index)
  long long at_row_bytes;
  const uint8_t *Tt; long long tt_row_bytes; const uint32_t *tt_rowb;  // per t
  const uint8_t *planes; long long plane_bytes;
  const uint8_t *mask;                          // M_At->mc_j
  int P;                                        // 1920-bit blocks per row
  int npairs;
  const uint8_t *Zt; const uint32_t *zt_rowb; long long zt_row_bytes;
  const uint32_t *mw_a;                         // a-index of each Wn row (j order)
  int nW; int B; int ncols_per;
  const int8_t *vS;                             // [t][mw] +/-1
  const double *aA; const double *aZ;           // per pair
  const int *ycnt;                              // per plane row: popcount(y & mask)
  const double *T_base; const double *T_tmp;    // [t], [t][mw]
  double min_d, mlt_d;
  const unsigned long long *out_off;            // per pair: row index in the output
  const unsigned long long *t_off;              // per t: column offset (index * row_stride)
  double *out;
};

// The tensor-core main kernel (bitplane_tc.cu), in place of
// bitplane_main_kernel; requires B in {8, 16, 32}.
void launch_bitplane_tc(const BitplaneParams &p, int nT, cudaStream_t s);
// CTAs of one call (pair tiles x covariate columns), and many calls of the
// same B in one launch: ps / tile0 in device memory, tile0 the prefix sums
// of the calls' CTA counts, `tiles` their total.
int bitplane_tc_tiles(const BitplaneParams &p, int nT);
void launch_bitplane_tc_group(int B, const BitplaneParams *ps, const int *tile0, int n, int tiles, cudaStream_t s);

}  // namespace lakgb
