// Row-vector products over packed bit rows (HBM-bound scans).
//
//  An_v    (dir_c/An_v.c:5-57):       out_r = -cpop_j + 2*popcount(row & mc_j)   (TYPE_pm)
//                                      out_r =          popcount(row & mc_j)    (TYPE_00)
//  An_ajdk (dir_c/An_ajdk_v.c:272-363): for each of the 15 weight vectors w_k,
//          out_rk = -sum_b w_kb*popcount(mc_j block b) + 2*sum_b w_kb*c_rb  (TYPE_pm)
//          with the block sums accumulated in ascending block order, one multiply
//          and one add per block and no FMA, as popcount_lf (popcount.c:252-308).
//
// An_v: one warp per row; lanes 0..29 read the 240-byte block as 8-byte
// words and the warp reduces the block count with shuffles.  An_ajdk: the
// same counts for two rows per warp, whose 2 x 15 FP64 accumulators sit on
// lanes 0..14 and 16..30.
#include "lakgb_runtime.cuh"
#include "rowvec.cuh"

namespace lakgb {

namespace {

// Rows from which An_ajdk runs two rows per warp.
constexpr int kAjdkTwoRows = 16384;

__device__ __forceinline__ int block_count(const uint8_t *row, const uint8_t *mask, int lane) {
  int c = 0;
  if (lane < 30) {
    const uint2 x = __ldg(reinterpret_cast<const uint2 *>(row) + lane);
    const uint2 m = __ldg(reinterpret_cast<const uint2 *>(mask) + lane);
    c = __popc(x.x & m.x) + __popc(x.y & m.y);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  return c;
}

__global__ void an_v_kernel(RowvecParams p) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= p.n) return;
  const uint8_t *row = p.w + (long long)p.rowb[warp] * p.row_bytes;
  long long tot = 0;
  for (int b = 0; b < p.P; ++b)
    tot += block_count(row + (long long)b * kBlockBytes, p.mask + (long long)b * kBlockBytes, lane);
  if (lane == 0) {
    double o = (p.type == 1) ? __dadd_rn(-(double)p.cpop_j, __dmul_rn(2.0, (double)tot)) : (double)tot;
    p.out[p.out_r[warp]] = o;
  }
}

// RPW rows per warp.  With two, lanes 0..14 carry the 15 accumulators of row
// 2w and lanes 16..30 those of row 2w+1, so each FP64 multiply and add
// instruction (which holds the sub-partition's FP64 unit whatever its active
// lanes) serves both rows: 1.7x faster on 32768 rows; small launches keep one
// row per warp, which gives them twice the warps.
template <int RPW>
__global__ void an_ajdk_kernel(RowvecParams p) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int r0 = RPW * warp;
  if (r0 >= p.n) return;
  const bool two = RPW == 2 && r0 + 1 < p.n;
  const uint8_t *rowA = p.w + (long long)p.rowb[r0] * p.row_bytes;
  const uint8_t *rowB = two ? p.w + (long long)p.rowb[r0 + 1] * p.row_bytes : rowA;
  const int k = lane & 15;
  const bool mine = k < 15 && (lane < 16 || two);
  double s = 0.0;
  for (int b = 0; b < p.P; ++b) {
    const long long bo = (long long)b * kBlockBytes;
    const int cA = block_count(rowA + bo, p.mask + bo, lane);
    int c = cA;
    if (RPW == 2) {
      const int cB = block_count(rowB + bo, p.mask + bo, lane);
      c = lane < 16 ? cA : cB;
    }
    if (mine) s = __dadd_rn(s, __dmul_rn(p.ajdk[b + (long long)k * p.P], (double)c));
  }
  if (mine) {
    double o = (p.type == 1) ? __dadd_rn(-p.base[k], __dmul_rn(2.0, s)) : s;
    p.out[(long long)p.out_r[r0 + (lane >> 4)] + (long long)k * p.out_stride] = o;
  }
}

}  // namespace

void launch_an_v(const RowvecParams &p) {
  if (p.n <= 0) return;
  const int threads = 256;
  const int blocks = (int)(((long long)p.n * 32 + threads - 1) / threads);
  an_v_kernel<<<blocks, threads, 0, stream()>>>(p);
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
}

void launch_an_ajdk(const RowvecParams &p) {
  if (p.n <= 0) return;
  const int threads = 256;
  if (p.n >= kAjdkTwoRows) {
    const long long warps = ((long long)p.n + 1) / 2;
    an_ajdk_kernel<2><<<(int)((warps * 32 + threads - 1) / threads), threads, 0, stream()>>>(p);
  } else {
    an_ajdk_kernel<1><<<(int)(((long long)p.n * 32 + threads - 1) / threads), threads, 0, stream()>>>(p);
  }
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
}

}  // namespace lakgb
