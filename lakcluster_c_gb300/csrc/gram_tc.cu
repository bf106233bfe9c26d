// +/-1 Gram of packed bit rows on the tensor cores (tcgen05, e4m3 operands).
//
// Computes exactly what the popcount kernel (gram.cu) computes, bit for bit:
//   out[i,k] = a0d1 - 2*S_ik - ((lfA_i + lfZ_k) - a2d1),  S_ik = sum_b D_b * c_ikb
// with c_ikb = popcount((A_i xor Z_k) & mask) over 1920-bit block b (TYPE_pm),
// or out = S_ik with c_ikb = popcount(A_i & Z_k & mask) (TYPE_00) -- the
// arithmetic of get_AnZt_vv__run (dir_c/AnZt_vv.c:62-95) with the block-
// weighted popcounts of popcount_xor_lf / popcount_and_lf
// (dir_c/popcount.c:310-423).
//
// Integer part on the tensor cores.  Every packed bit becomes one e4m3 byte:
// 0x08 (= 2^-6) for a set bit, 0 otherwise, the mask applied to the A side.
// One product is 2^-12, so the fp32 accumulator of a block holds
// n_ikb * 2^-12 with n_ikb = popcount(A_i & mask & Z_k) <= 1920: an exact
// value (11 significant bits).  The XOR count is c = pa_ib + pz_kb - 2 n_ikb
// with the row counts pa = popcount(A_i & mask), pz = popcount(Z_k & mask)
// that the producer threads take while they expand the bits.  Which bit goes
// to which K position does not matter (a dot product is order-free) as long
// as A and Z use the same map; the map used makes the expansion two integer
// operations per output word: bit 8i+j of a 32-bit word goes to byte i of
// output word j.
//
// FP64 part on the CUDA cores, in the reference's order: acc = acc + D_b * c,
// one rounding each, blocks ascending.  The product D_b * c is read from a
// table T_b[c] (c = 0..1920), built once per launch with the same rounded
// multiply, so the FP64 pipe -- slow on this part -- does only the add.
//
// CTA: a 128 (A rows) x 128 (Z rows) tile, 9 warps.
//   warps 0-3  producers: per 128-column chunk, load each tile row's 16
//              bytes, mask, expand to 128 e4m3 bytes in shared memory
//              (K-major core matrices, no swizzle), count pa / pz.
//   warp 4     owns TMEM; lane 0 issues the MMAs (M=128, N=128, K=32; 4 per
//              chunk, 15 chunks per block) into one of two count buffers.
//   warps 5-8  fold: per block, read the counts from TMEM (warp w reads
//              lanes 32*(w%4)..+31), look up T_b[c], add into the FP64
//              accumulators, which live in TMEM as well (columns 256..511,
//              two 32-bit halves per value).
// Shared memory: 4 stages x (16 KB A + 16 KB B) + 2 x T_b (15 KB) + counts.
// TMEM: 512 columns (2 x 128 count columns + 256 accumulator columns).
#include "gram.cuh"
#include "lakgb_runtime.cuh"
#include "tc_ptx.cuh"

namespace lakgb {

__device__ int g_tc_status;  // first pipeline error code of any tensor-core kernel (0 = none)

namespace {

constexpr int kBM = 128, kBN = 128;
constexpr int kStages = 4;
constexpr int kChunks = 15;               // 128-bit chunks per 1920-bit block
constexpr int kPrefetch = 5;              // producer loads in flight (divides kChunks)
constexpr int kStageA = kBM * 128;        // bytes: 128 rows x 128 e4m3
constexpr int kStageB = kBN * 128;
constexpr int kStageBytes = kStageA + kStageB;
constexpr int kTabStride = 1922;          // doubles per block table (1921 used, 16-byte multiple)
constexpr int kTabBytes = kTabStride * 8;
constexpr int kSBO = 8 * 128;             // bytes between 8-row core-matrix groups (8 k-groups of 16 B)
constexpr int kThreads = 288;
constexpr uint32_t kTmemCols = 512;
constexpr size_t kSmemBytes = (size_t)kStages * kStageBytes + 2 * kTabBytes + 2 * (kBM + kBN) * 4 + 128;

struct Smem {
  uint64_t full[kStages], empty[kStages];
  uint64_t acc_full[2], acc_empty[2], aux_full[2], aux_empty[2], done;
  uint32_t tmem_base;
  int abort;
  long long a_off[kBM], z_off[kBN];
};

// Expand the 128 bits of x into 128 e4m3 bytes of one tile row: words q of x
// fill k-groups 2q and 2q+1 (16 bytes each) at row_base + g*128.
__device__ __forceinline__ void expand_row(uint32_t row_base, uint4 x) {
  const uint32_t w[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uint32_t v = w[q];
    tc::st_shared_v4(row_base + (2 * q) * 128, (v << 3) & 0x08080808u, (v << 2) & 0x08080808u,
                     (v << 1) & 0x08080808u, v & 0x08080808u);
    tc::st_shared_v4(row_base + (2 * q + 1) * 128, (v >> 1) & 0x08080808u, (v >> 2) & 0x08080808u,
                     (v >> 3) & 0x08080808u, (v >> 4) & 0x08080808u);
  }
}

__device__ __forceinline__ int popc4(uint4 x) { return __popc(x.x) + __popc(x.y) + __popc(x.z) + __popc(x.w); }
__device__ __forceinline__ uint4 and4(uint4 a, uint4 b) {
  return make_uint4(a.x & b.x, a.y & b.y, a.z & b.z, a.w & b.w);
}

// Counts decoded from the accumulator: n * 2^-12 -> n (exact for n < 2^22).
__device__ __forceinline__ int decode_count(uint32_t bits) {
  return __float_as_int(__fmaf_rn(__uint_as_float(bits), 4096.0f, 12582912.0f)) - 0x4B400000;
}

// 2.0 * x, exactly as __dmul_rn(2.0, x) rounds it: for a normal x whose
// double does not overflow, one more in the exponent field; otherwise (zero,
// subnormal, near-overflow, inf, nan) the multiply itself.  Keeps the FP64
// pipe for the adds.
__device__ __forceinline__ double twice(double x) {
  const long long bits = __double_as_longlong(x);
  const int e = (int)((bits >> 52) & 0x7FF);
  return (e >= 1 && e <= 2045) ? __longlong_as_double(bits + (1ll << 52)) : __dmul_rn(2.0, x);
}

template <int TYPE>
__global__ void __launch_bounds__(kThreads, 1) gram_tc_kernel(GramParams p, const double *__restrict__ T) {
  extern __shared__ __align__(128) uint8_t dsm[];
  __shared__ Smem sm;
  uint8_t *stages = dsm;
  double *sT = reinterpret_cast<double *>(dsm + (size_t)kStages * kStageBytes);  // [2][kTabStride]
  int *s_pa = reinterpret_cast<int *>(dsm + (size_t)kStages * kStageBytes + 2 * kTabBytes);  // [2][kBM]
  int *s_pz = s_pa + 2 * kBM;                                                                   // [2][kBN]

  const int tile_n = blockIdx.x * kBN;
  const int tile_m = blockIdx.y * kBM;
  if (p.symmetric && tile_m > tile_n + kBN - 1) return;

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  volatile int *abort = &sm.abort;
  const int P = p.P;

  for (int i = tid; i < kBM; i += kThreads)
    sm.a_off[i] = (tile_m + i < p.nA) ? (long long)p.a_rowb[tile_m + i] * p.a_row_bytes : -1;
  for (int i = tid; i < kBN; i += kThreads)
    sm.z_off[i] = (tile_n + i < p.nZ) ? (long long)p.z_rowb[tile_n + i] * p.z_row_bytes : -1;
  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      tc::mbar_init(&sm.full[s], 128);
      tc::mbar_init(&sm.empty[s], 1);
    }
    for (int t = 0; t < 2; ++t) {
      tc::mbar_init(&sm.acc_full[t], 1);
      tc::mbar_init(&sm.acc_empty[t], 128);
      tc::mbar_init(&sm.aux_full[t], 128);
      tc::mbar_init(&sm.aux_empty[t], 128);
    }
    tc::mbar_init(&sm.done, 1);
    sm.abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 4) tc::tmem_alloc(&sm.tmem_base, kTmemCols);
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = sm.tmem_base;

  if (warp < 4) {
    // ---------------- producers ----------------
    const int r = tid;  // A row r and Z row r of the tile
    const long long ao = sm.a_off[r], zo = sm.z_off[r];
    const uint32_t row_in_stage = (uint32_t)((r >> 3) * kSBO + (r & 7) * 16);
    const uint32_t st0 = tc::smem_u32(stages);
    const int G = P * kChunks;
    // Loads run kPrefetch chunks ahead of the expansion (register ring).
    uint4 rm[kPrefetch], ra[kPrefetch], rz[kPrefetch];
    auto load = [&](int g, uint4 &m, uint4 &xa, uint4 &xz) {
      m = xa = xz = make_uint4(0, 0, 0, 0);
      if (g < G) {
        const long long off = (long long)(g / kChunks) * kBlockBytes + (g % kChunks) * 16;
        m = __ldg(reinterpret_cast<const uint4 *>(p.mask + off));
        if (ao >= 0) xa = __ldg(reinterpret_cast<const uint4 *>(p.wA + ao + off));
        if (zo >= 0) xz = __ldg(reinterpret_cast<const uint4 *>(p.wZ + zo + off));
      }
    };
#pragma unroll
    for (int u = 0; u < kPrefetch; ++u) load(u, rm[u], ra[u], rz[u]);
    bool ok = true;
    int pa = 0, pz = 0;
    for (int g0 = 0; g0 < G; g0 += kPrefetch) {
#pragma unroll
      for (int u = 0; u < kPrefetch; ++u) {
        const int g = g0 + u, s = g % kStages, it = g / kStages;
        const uint4 m = rm[u], xz = rz[u];
        const uint4 xa = and4(ra[u], m);
        load(g + kPrefetch, rm[u], ra[u], rz[u]);
        if (TYPE == 1) {
          pa += popc4(xa);
          pz += popc4(and4(xz, m));
        }
        if (it > 0 && ok) ok = tc::mbar_wait(&sm.empty[s], (it - 1) & 1, abort, &g_tc_status, 1);
        if (ok) {
          const uint32_t sa = st0 + s * kStageBytes + row_in_stage;
          expand_row(sa, xa);
          expand_row(sa + kStageA, xz);
          tc::fence_proxy_async();
        }
        tc::mbar_arrive(&sm.full[s]);
        if ((g + 1) % kChunks == 0) {
          // end of block b: publish its row counts
          const int b = g / kChunks, t = b & 1;
          if (b >= 2 && ok) ok = tc::mbar_wait(&sm.aux_empty[t], ((b >> 1) - 1) & 1, abort, &g_tc_status, 2);
          s_pa[t * kBM + r] = pa;
          s_pz[t * kBN + r] = pz;
          tc::mbar_arrive(&sm.aux_full[t]);
          pa = pz = 0;
        }
      }
    }
  } else if (warp == 4) {
    // ---------------- MMA issue ----------------
    if (lane == 0) {
      constexpr uint32_t idesc = tc::idesc_e4m3_f32(kBM, kBN);
      const uint32_t st0 = tc::smem_u32(stages);
      bool ok = true;
      for (int b = 0; b < P && ok; ++b) {
        const int t = b & 1;
        if (b >= 2) ok = tc::mbar_wait(&sm.acc_empty[t], ((b >> 1) - 1) & 1, abort, &g_tc_status, 3);
        tc::fence_after_sync();
        for (int ch = 0; ch < kChunks && ok; ++ch) {
          const int g = b * kChunks + ch, s = g % kStages, it = g / kStages;
          ok = tc::mbar_wait(&sm.full[s], it & 1, abort, &g_tc_status, 4);
          if (!ok) break;
          tc::fence_after_sync();
          const uint32_t sa = st0 + s * kStageBytes, sb = sa + kStageA;
#pragma unroll
          for (int kk = 0; kk < 4; ++kk) {
            const uint64_t ad = tc::smem_desc(sa + kk * 256, 128, kSBO);
            const uint64_t bd = tc::smem_desc(sb + kk * 256, 128, kSBO);
            tc::mma_e4m3(tmem + t * kBN, ad, bd, idesc, (ch | kk) != 0);
          }
          tc::mma_commit(&sm.empty[s]);
        }
        if (ok) tc::mma_commit(&sm.acc_full[t]);
      }
      // every issued MMA has completed before TMEM is released (waited for
      // even after an abort, within the same time limit)
      tc::mma_commit(&sm.done);
      const unsigned long long t0 = tc::globaltimer();
      while (!tc::mbar_try(&sm.done, 0)) {
        if (tc::globaltimer() - t0 > tc::kWaitNs) {
          atomicCAS(&g_tc_status, 0, 5);
          break;
        }
      }
    }
  } else {
    // ---------------- FP64 fold ----------------
    const int q = warp & 3;
    const int et = tid - 160;  // 0..127
    const int row = 32 * q + lane;
    const int ga = tile_m + row;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    for (int i = et; i < kTabBytes / 16; i += 128)
      tc::cp_async16(reinterpret_cast<uint8_t *>(sT) + 16 * i, reinterpret_cast<const uint8_t *>(T) + 16 * i);
    tc::cp_async_commit();
    const double lfa = (p.lfA && ga < p.nA) ? p.lfA[ga] : 0.0;
    const long long orow = ga < p.nA ? (long long)p.out_r[ga] : 0;
    const long long ocol2 = (p.symmetric && ga < p.nA) ? (long long)p.out_c2[ga] * p.out_stride : 0;
    bool ok = true;
    for (int b = 0; b < P; ++b) {
      const int t = b & 1;
      if (b + 1 < P) {
        tc::named_bar_sync(1, 128);  // block b-1 no longer reads its table buffer
        const uint8_t *src = reinterpret_cast<const uint8_t *>(T + (size_t)(b + 1) * kTabStride);
        uint8_t *dst = reinterpret_cast<uint8_t *>(sT + (t ^ 1) * kTabStride);
        for (int i = et; i < kTabBytes / 16; i += 128) tc::cp_async16(dst + 16 * i, src + 16 * i);
        tc::cp_async_commit();
        tc::cp_async_wait<1>();
      } else {
        tc::cp_async_wait<0>();
      }
      tc::named_bar_sync(1, 128);  // T_b is in shared memory
      bool w = ok && tc::mbar_wait(&sm.aux_full[t], (b >> 1) & 1, abort, &g_tc_status, 6);
      w = w && tc::mbar_wait(&sm.acc_full[t], (b >> 1) & 1, abort, &g_tc_status, 7);
      ok = __all_sync(0xffffffffu, w);
      tc::fence_after_sync();
      const double *Tb = sT + t * kTabStride;
      const int pa = s_pa[t * kBM + row];
      const int *pzb = s_pz + t * kBN;
#pragma unroll 1
      for (int c0 = 0; c0 < kBN; c0 += 32) {
        // counts of columns c0..c0+31 and their accumulators (TMEM columns
        // 256 + 2*c0 + 2j low word, + 2j + 1 high word), one wait for all
        uint32_t cnt[32], aw[2][32];
        const uint32_t acol = lane_base + 256 + 2 * c0;
        if (ok) {
          tc::tmem_ld32(lane_base + t * kBN + c0, cnt);
          if (b > 0) {
            tc::tmem_ld32(acol, aw[0]);
            tc::tmem_ld32(acol + 32, aw[1]);
          }
          tc::tmem_wait_ld();
        } else {
#pragma unroll
          for (int j = 0; j < 32; ++j) cnt[j] = 0;
        }
        if (c0 == kBN - 32) {
          // all count columns of buffer t read: the MMA may refill it
          tc::fence_before_sync();
          tc::mbar_arrive(&sm.acc_empty[t]);
        }
#pragma unroll
        for (int h = 0; h < 2; ++h) {
          double acc[16];
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int n = decode_count(cnt[16 * h + j]);
            int c = (TYPE == 1) ? pa + pzb[c0 + 16 * h + j] - 2 * n : n;
            c = min(max(c, 0), kTabStride - 1);
            const double x = Tb[c];
            acc[j] = (b > 0) ? __dadd_rn(__hiloint2double((int)aw[h][2 * j + 1], (int)aw[h][2 * j]), x) : x;
          }
          if (b + 1 < P) {
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              aw[h][2 * j] = (uint32_t)__double2loint(acc[j]);
              aw[h][2 * j + 1] = (uint32_t)__double2hiint(acc[j]);
            }
          } else if (ok && ga < p.nA) {
#pragma unroll
            for (int j = 0; j < 16; ++j) {
              const int gz = tile_n + c0 + 16 * h + j;
              if (gz >= p.nZ || (p.symmetric && ga > gz)) continue;
              double o = (TYPE == 1) ? __dsub_rn(p.a0d1, twice(acc[j])) : acc[j];
              if (p.lfA && p.lfZ) o = __dsub_rn(o, __dsub_rn(__dadd_rn(lfa, p.lfZ[gz]), p.a2d1));
              p.out[orow + (long long)p.out_c[gz] * p.out_stride] = o;
              if (p.symmetric) p.out[(long long)p.out_r2[gz] + ocol2] = o;
            }
          }
        }
        if (ok && b + 1 < P) {
          tc::tmem_st32(acol, aw[0]);
          tc::tmem_st32(acol + 32, aw[1]);
        }
      }
      if (ok) tc::tmem_wait_st();
      tc::mbar_arrive(&sm.aux_empty[t]);
    }
  }

  tc::fence_before_sync();
  __syncthreads();
  if (warp == 4) {
    __syncwarp();
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kTmemCols);
  }
}

__global__ void gram_table_kernel(const double *__restrict__ D, int P, double *__restrict__ T) {
  const int b = blockIdx.x;
  const double d = D ? D[b] : 1.0;
  for (int c = threadIdx.x; c < kTabStride; c += blockDim.x)
    T[(size_t)b * kTabStride + c] = c < kTabStride - 1 ? __dmul_rn(d, (double)c) : __longlong_as_double(0x7ff8dead00000000ll);
}

template <int TYPE>
void launch_tc_type(const GramParams &p, const double *T, cudaStream_t s) {
  static bool configured = false;
  if (!configured) {
    LAKGB_CUDA(cudaFuncSetAttribute(gram_tc_kernel<TYPE>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kSmemBytes));
    configured = true;
  }
  dim3 grid((p.nZ + kBN - 1) / kBN, (p.nA + kBM - 1) / kBM);
  gram_tc_kernel<TYPE><<<grid, kThreads, kSmemBytes, s>>>(p, T);
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
}

}  // namespace

void launch_gram_tc(const GramParams &p, cudaStream_t s) {
  double *T = nullptr;
  LAKGB_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&T), (size_t)p.P * kTabBytes, s));
  gram_table_kernel<<<p.P, 256, 0, s>>>(p.D, p.P, T);
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
  if (p.type == 1)
    launch_tc_type<1>(p, T, s);
  else
    launch_tc_type<2>(p, T, s);
  LAKGB_CUDA(cudaFreeAsync(T, s));
}

int tc_status_take() {
  int v = 0;
  LAKGB_CUDA(cudaDeviceSynchronize());
  LAKGB_CUDA(cudaMemcpyFromSymbol(&v, g_tc_status, sizeof v));
  if (v) {
    const int zero = 0;
    LAKGB_CUDA(cudaMemcpyToSymbol(g_tc_status, &zero, sizeof zero));
  }
  return v;
}

}  // namespace lakgb
