// +/-1 Gram of packed bit rows, popcount path.
//
// out[i,k] = a0d1 - 2*S_ik - ((lfA_i + lfZ_k) - a2d1),   S_ik = sum_blocks D_b * c_ikb
// where c_ikb = popcount((A_i xor Z_k) & mask) over 1920-bit block b (TYPE_pm)
// or popcount(A_i & Z_k & mask) (TYPE_00, out = S_ik).
// This is the arithmetic of get_AnZt_vv__run (dir_c/AnZt_vv.c:62-95) with the
// block-weighted popcount of popcount_xor_lf / popcount_and_lf
// (dir_c/popcount.c:310-423).  The integer counts are exact; the FP64 combine
// keeps the reference's order -- one multiply and one add per block, blocks in
// ascending order, no fused multiply-add -- so every output is bit-identical.
//
// Layout: each CTA owns a BM x BN tile of (A rows) x (Z rows).  Per 1920-bit
// block it stages the tile's BM + BN masked row segments (240 B each) in
// shared memory (row pitch 61 words: conflict-free column reads), every
// thread accumulates a TM x TN micro-tile of integer counts over the block's
// 60 words, then folds them into FP64 accumulators with the block weight.
#include <atomic>

#include "gram.cuh"
#include "lakgb_runtime.cuh"

namespace lakgb {

namespace {

constexpr int kLd = kBlockWords + 1;  // smem row pitch in words

template <int BM, int BN, int TM, int TN, int TYPE>
__global__ void __launch_bounds__((BM / TM) * (BN / TN), 2)
gram_popc_kernel(GramParams p) {
  constexpr int TX = BN / TN;
  constexpr int TY = BM / TM;
  constexpr int NT = TX * TY;
  extern __shared__ uint32_t smem[];
  uint32_t *As = smem;
  uint32_t *Zs = smem + BM * kLd;
  __shared__ long long a_off[BM];
  __shared__ long long z_off[BN];

  const int tile_n = blockIdx.x * BN;
  const int tile_m = blockIdx.y * BM;
  // Symmetric Gram: only pairs i <= k are computed (and mirrored).  A tile
  // whose smallest row index exceeds its largest column index has none.
  if (p.symmetric && tile_m > tile_n + BN - 1) return;

  const int tid = threadIdx.x;
  const int tx = tid % TX;
  const int ty = tid / TX;

  for (int i = tid; i < BM; i += NT)
    a_off[i] = (tile_m + i < p.nA) ? (long long)p.a_rowb[tile_m + i] * p.a_row_bytes : -1;
  for (int i = tid; i < BN; i += NT)
    z_off[i] = (tile_n + i < p.nZ) ? (long long)p.z_rowb[tile_n + i] * p.z_row_bytes : -1;

  double acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = 0.0;

  for (int blk = 0; blk < p.P; ++blk) {
    __syncthreads();
    const long long boff = (long long)blk * kBlockBytes;
    const uint4 *mk = reinterpret_cast<const uint4 *>(p.mask + boff);
    for (int idx = tid; idx < BM * 15; idx += NT) {
      const int r = idx / 15, v = idx - r * 15;
      uint4 x = make_uint4(0u, 0u, 0u, 0u);
      const long long o = a_off[r];
      if (o >= 0) {
        const uint4 m = __ldg(mk + v);
        x = __ldg(reinterpret_cast<const uint4 *>(p.wA + o + boff) + v);
        x.x &= m.x; x.y &= m.y; x.z &= m.z; x.w &= m.w;
      }
      uint32_t *d = As + r * kLd + 4 * v;
      d[0] = x.x; d[1] = x.y; d[2] = x.z; d[3] = x.w;
    }
    for (int idx = tid; idx < BN * 15; idx += NT) {
      const int r = idx / 15, v = idx - r * 15;
      uint4 x = make_uint4(0u, 0u, 0u, 0u);
      const long long o = z_off[r];
      if (o >= 0) {
        const uint4 m = __ldg(mk + v);
        x = __ldg(reinterpret_cast<const uint4 *>(p.wZ + o + boff) + v);
        x.x &= m.x; x.y &= m.y; x.z &= m.z; x.w &= m.w;
      }
      uint32_t *d = Zs + r * kLd + 4 * v;
      d[0] = x.x; d[1] = x.y; d[2] = x.z; d[3] = x.w;
    }
    __syncthreads();

    int cnt[TM][TN];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) cnt[i][j] = 0;

#pragma unroll 4
    for (int w = 0; w < kBlockWords; ++w) {
      uint32_t a[TM], z[TN];
#pragma unroll
      for (int i = 0; i < TM; ++i) a[i] = As[(ty + i * TY) * kLd + w];
#pragma unroll
      for (int j = 0; j < TN; ++j) z[j] = Zs[(tx + j * TX) * kLd + w];
#pragma unroll
      for (int i = 0; i < TM; ++i)
#pragma unroll
        for (int j = 0; j < TN; ++j)
          cnt[i][j] += __popc(TYPE == 1 ? (a[i] ^ z[j]) : (a[i] & z[j]));
    }
    const double d = p.D ? p.D[blk] : 1.0;
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j)
        acc[i][j] = __dadd_rn(acc[i][j], __dmul_rn(d, (double)cnt[i][j]));
  }

#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int ga = tile_m + ty + i * TY;
    if (ga >= p.nA) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int gz = tile_n + tx + j * TX;
      if (gz >= p.nZ) continue;
      if (p.symmetric && ga > gz) continue;
      double o = (TYPE == 1) ? __dsub_rn(p.a0d1, __dmul_rn(2.0, acc[i][j])) : acc[i][j];
      if (p.lfA && p.lfZ) o = __dsub_rn(o, __dsub_rn(__dadd_rn(p.lfA[ga], p.lfZ[gz]), p.a2d1));
      p.out[(long long)p.out_r[ga] + (long long)p.out_c[gz] * p.out_stride] = o;
      if (p.symmetric)
        p.out[(long long)p.out_r2[gz] + (long long)p.out_c2[ga] * p.out_stride] = o;
    }
  }
}

template <int BM, int BN, int TM, int TN, int TYPE>
void launch_tile(const GramParams &p) {
  constexpr int NT = (BM / TM) * (BN / TN);
  const size_t smem = (size_t)(BM + BN) * kLd * sizeof(uint32_t);
  static bool configured = false;
  if (!configured) {
    LAKGB_CUDA(cudaFuncSetAttribute(gram_popc_kernel<BM, BN, TM, TN, TYPE>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured = true;
  }
  dim3 grid((p.nZ + BN - 1) / BN, (p.nA + BM - 1) / BM);
  gram_popc_kernel<BM, BN, TM, TN, TYPE><<<grid, NT, smem, p.stream ? p.stream : stream()>>>(p);
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
}

}  // namespace

std::atomic<int> g_gram_impl{LAKGB_GRAM_TENSOR};

void launch_gram(const GramParams &p) {
  if (p.nA <= 0 || p.nZ <= 0 || p.P <= 0) return;
  cudaStream_t s = p.stream ? p.stream : stream();
  gram_timer_begin(s);
  if (g_gram_impl.load(std::memory_order_relaxed) == LAKGB_GRAM_TENSOR)
    launch_gram_tc(p, s);
  else if (p.type == 1)
    launch_tile<128, 64, 8, 4, 1>(p);
  else
    launch_tile<128, 64, 8, 4, 2>(p);
  gram_timer_end(s);
}

}  // namespace lakgb

extern "C" void lakgb_set_gram_impl(int impl) {
  lakgb::g_gram_impl.store(impl == LAKGB_GRAM_POPCOUNT ? LAKGB_GRAM_POPCOUNT : LAKGB_GRAM_TENSOR);
}

extern "C" int lakgb_gram_impl(void) { return lakgb::g_gram_impl.load(); }

extern "C" int lakgb_device_status(void) { return lakgb::tc_status_take(); }

extern "C" int lakgb_gram_device(const lakgb_gram_args *a) {
  using namespace lakgb;
  if (!a || (a->type_flag != LAKGB_TYPE_pm && a->type_flag != LAKGB_TYPE_00)) {
    set_error(3, "lakgb_gram_device: bad arguments");
    return -1;
  }
  GramParams p{};
  p.wA = a->wA; p.a_rowb = a->a_rowb; p.nA = a->nA; p.a_row_bytes = a->a_row_bytes;
  p.wZ = a->wZ; p.z_rowb = a->z_rowb; p.nZ = a->nZ; p.z_row_bytes = a->z_row_bytes;
  p.mask = a->mask; p.P = a->P; p.D = a->D;
  p.type = (a->type_flag == LAKGB_TYPE_pm) ? 1 : 2;
  p.a0d1 = a->a0d1; p.a2d1 = a->a2d1; p.lfA = a->lfA; p.lfZ = a->lfZ;
  p.out_r = a->out_r; p.out_c = a->out_c; p.out_r2 = a->out_r2; p.out_c2 = a->out_c2;
  p.out_stride = a->out_stride; p.out = a->out; p.symmetric = a->symmetric;
  p.stream = (cudaStream_t)a->stream;
  launch_gram(p);
  return 0;
}

namespace lakgb {

double gram_bitops(const GramParams &p, long long retained_cols) {
  return (double)p.nA * (double)p.nZ * (double)retained_cols;
}

}  // namespace lakgb
