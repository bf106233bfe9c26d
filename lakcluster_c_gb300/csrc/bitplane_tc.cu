// Bit-plane loop product At_T_YnWt_S_Zn_ww (dir_c/At_T_YnWt_S_Zn_ww.c:5-190)
// with its integer part on the tensor cores.
//
// Same outputs as bitplane_main_kernel (bitplane.cu), bit for bit.  The
// integer part is the count
//   cnt[na][q] = popcount(a'_na & plane_q)  over all patient bits,
//   a' = ~(At_na ^ Tt_t) & mask,
// for every value plane q = (Wn row mw, bit k): a GEMM over bits, M = SNP
// pairs, N = planes, K = patients.  Bits become e4m3 bytes (0x08 = 2^-6 for a
// set bit, 0 otherwise), so the fp32 accumulator in TMEM holds cnt * 2^-12
// exactly (cnt <= patients < 2^22).  The fold then forms, exactly as the
// CUDA-core kernel does,
//   At_tmp = sum_k 2^k (2 cnt[k] - popcount(plane_k & mask))   (int64)
// and runs the FP64 recurrence over the Wn rows in their order, one thread per
// SNP pair, with the reference's operations in the reference's order.
//
// CTA: 128 SNP pairs x one covariate column t; it walks N tiles of CW = 256/B
// Wn rows (256 planes) in order.  17 warps:
//   warps 0-11  producers: per 128-patient chunk, 128 rows a' and 256 plane
//               rows, expanded to e4m3 in a 4-stage ring of 128-byte-swizzled
//               K-major tiles (16 KB + 32 KB a stage).
//   warp 12     owns TMEM (2 x 256 count columns); lane 0 issues the MMAs
//               (M=128, N=256, K=32), a whole N tile into one count buffer.
//   warps 13-16 fold: thread = SNP pair = TMEM lane.
// Every wait is bounded (tc_ptx.cuh); a pipeline error is recorded in the
// tensor-core status word read by lakgb_device_status.
#include <mutex>

#include "bitplane.cuh"
#include "gram.cuh"
#include "lakgb_runtime.cuh"
#include "tc_ptx.cuh"

namespace lakgb {

namespace {

constexpr int kM = 128, kN = 256;
constexpr int kStages = 4;
constexpr int kChunks = 15;                // 128-bit chunks per 1920-bit block
constexpr int kPrefetch = 3;               // producer loads in flight (divides kChunks)
constexpr int kStageA = kM * 128, kStageB = kN * 128, kStageBytes = kStageA + kStageB;
constexpr int kSBO = 1024;                 // bytes between 8-row swizzle atoms
constexpr int kProducers = kM + kN;        // warps 0-11
constexpr int kMmaWarp = kProducers / 32;  // 12
constexpr int kFold = 128;                 // warps 13-16
constexpr int kThreads = kProducers + 32 + kFold;
constexpr uint32_t kTmemCols = 512;
constexpr size_t kSmemBytes = (size_t)kStages * kStageBytes + 1024;

struct Smem {
  uint64_t full[kStages], empty[kStages];
  uint64_t acc_full[2], acc_empty[2], done;
  uint32_t tmem_base;
  int abort;
};

__device__ __forceinline__ void expand_row(uint32_t row_base, uint32_t sw, uint4 x) {
  const uint32_t w[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
  for (int q = 0; q < 4; ++q) {
    const uint32_t v = w[q];
    tc::st_shared_v4(row_base + (((2 * q) ^ sw) << 4), (v << 3) & 0x08080808u, (v << 2) & 0x08080808u,
                     (v << 1) & 0x08080808u, v & 0x08080808u);
    tc::st_shared_v4(row_base + (((2 * q + 1) ^ sw) << 4), (v >> 1) & 0x08080808u, (v >> 2) & 0x08080808u,
                     (v >> 3) & 0x08080808u, (v >> 4) & 0x08080808u);
  }
}

__device__ __forceinline__ int decode_count(uint32_t bits) {
  return __float_as_int(__fmaf_rn(__uint_as_float(bits), 4096.0f, 12582912.0f)) - 0x4B400000;
}

__device__ __forceinline__ int plane_row(int mw, int k, int ncols_per) {
  return mw * ncols_per + ncols_per - 1 - k;
}

// One CTA's work: SNP pairs pair0 .. pair0 + 127 of covariate column t.
template <int B>
__device__ __forceinline__ void bitplane_tc_cta(const BitplaneParams &p, int t, int pair0, int *status) {
  constexpr int CW = kN / B;  // Wn rows per N tile
  extern __shared__ __align__(128) uint8_t dsm[];
  __shared__ Smem sm;
  uint8_t *stages = dsm + ((1024 - (tc::smem_u32(dsm) & 1023)) & 1023);

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  volatile int *abort = &sm.abort;
  const int NT = (p.nW + CW - 1) / CW;   // N tiles
  const int G = p.P * kChunks;            // chunks per N tile
  const uint8_t *trow = p.Tt + (long long)p.tt_rowb[t] * p.tt_row_bytes;

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      tc::mbar_init(&sm.full[s], kProducers);
      tc::mbar_init(&sm.empty[s], 1);
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(&sm.acc_full[b], 1);
      tc::mbar_init(&sm.acc_empty[b], kFold);
    }
    tc::mbar_init(&sm.done, 1);
    sm.abort = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == kMmaWarp) tc::tmem_alloc(&sm.tmem_base, kTmemCols);
  tc::fence_proxy_async();
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = sm.tmem_base;

  if (tid < kProducers) {
    // ---------------- producers ----------------
    const bool is_a = tid < kM;
    const int rr = is_a ? tid : tid - kM;
    long long a_off = -1;
    if (is_a && pair0 + rr < p.npairs) a_off = (long long)p.at_rowb[pair0 + rr] * p.at_row_bytes;
    const uint32_t region = tc::smem_u32(stages) + (is_a ? 0 : kStageA);
    const uint32_t my_row = region + (uint32_t)((rr >> 3) * kSBO + (rr & 7) * 128);
    const uint32_t my_sw = (uint32_t)(rr & 7);
    const uint4 *mk = reinterpret_cast<const uint4 *>(p.mask);
    const uint4 *tk = reinterpret_cast<const uint4 *>(trow);
    bool ok = true;
    int s = 0, wrap = 0;
    for (int nt = 0; nt < NT; ++nt) {
      // this thread's row: an a' row, or value plane (mw, k) of the tile
      const uint4 *src = nullptr;
      if (is_a) {
        if (a_off >= 0) src = reinterpret_cast<const uint4 *>(p.At + a_off);
      } else {
        const int mw = nt * CW + rr / B;
        if (mw < p.nW) src = reinterpret_cast<const uint4 *>(p.planes + (long long)plane_row(mw, rr % B, p.ncols_per) * p.plane_bytes);
      }
      uint4 rx[kPrefetch], rm[kPrefetch], rt[kPrefetch];
      auto load = [&](int g, uint4 &x, uint4 &m, uint4 &tt) {
        x = m = tt = make_uint4(0, 0, 0, 0);
        if (g < G && src) {
          x = __ldg(src + g);
          if (is_a) {
            m = __ldg(mk + g);
            tt = __ldg(tk + g);
          }
        }
      };
#pragma unroll
      for (int u = 0; u < kPrefetch; ++u) load(u, rx[u], rm[u], rt[u]);
      for (int g0 = 0; g0 < G; g0 += kPrefetch) {
#pragma unroll
        for (int u = 0; u < kPrefetch; ++u) {
          uint4 x = rx[u];
          if (is_a) {  // a' = ~(At ^ Tt) & mask (zero for a missing row)
            const uint4 m = rm[u], tt = rt[u];
            x = src ? make_uint4(~(x.x ^ tt.x) & m.x, ~(x.y ^ tt.y) & m.y, ~(x.z ^ tt.z) & m.z,
                                 ~(x.w ^ tt.w) & m.w)
                    : make_uint4(0, 0, 0, 0);
          }
          load(g0 + u + kPrefetch, rx[u], rm[u], rt[u]);
          if (wrap > 0 && ok) ok = tc::mbar_wait(&sm.empty[s], (uint32_t)((wrap - 1) & 1), abort, status, 11);
          if (ok) {
            expand_row(my_row + s * kStageBytes, my_sw, x);
            tc::fence_proxy_async();
          }
          tc::mbar_arrive(&sm.full[s]);
          if (++s == kStages) {
            s = 0;
            ++wrap;
          }
        }
      }
    }
  } else if (warp == kMmaWarp) {
    // ---------------- MMA issue ----------------
    if (lane == 0) {
      constexpr uint32_t idesc = tc::idesc_e4m3_f32(kM, kN);
      const uint32_t st0 = tc::smem_u32(stages);
      bool ok = true;
      int s = 0, wrap = 0;
      for (int nt = 0; nt < NT && ok; ++nt) {
        const int b = nt & 1;
        if (nt >= 2) ok = tc::mbar_wait(&sm.acc_empty[b], (uint32_t)(((nt >> 1) - 1) & 1), abort, status, 13);
        tc::fence_after_sync();
        for (int g = 0; g < G && ok; ++g) {
          const int cs = s;
          ok = tc::mbar_wait(&sm.full[cs], (uint32_t)(wrap & 1), abort, status, 14);
          if (++s == kStages) {
            s = 0;
            ++wrap;
          }
          if (!ok) break;
          tc::fence_after_sync();
          const uint32_t sa = st0 + cs * kStageBytes, sb = sa + kStageA;
#pragma unroll
          for (int kk = 0; kk < 4; ++kk)
            tc::mma_e4m3(tmem + b * kN, tc::smem_desc_sw128(sa + kk * 32, kSBO), tc::smem_desc_sw128(sb + kk * 32, kSBO),
                         idesc, (g | kk) != 0);
          tc::mma_commit(&sm.empty[cs]);
        }
        if (ok) tc::mma_commit(&sm.acc_full[b]);
      }
      tc::mma_commit(&sm.done);
      const unsigned long long t0 = tc::globaltimer();
      while (!tc::mbar_try(&sm.done, 0)) {
        if (tc::globaltimer() - t0 > tc::g_wait_ns) {
          atomicCAS(status, 0, 15);
          break;
        }
      }
    }
  } else {
    // ---------------- fold: thread = SNP pair ----------------
    const int q = warp & 3;
    const int row = 32 * q + lane;
    const int pr = pair0 + row;
    const bool live = pr < p.npairs;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    // At_base: pmpm0(At, Tt, plane 0) * min * mlt, from popcount(a' & p0)
    double At_base = 0.0, aA = 0.0, aZ = 0.0, acc = 0.0;
    long long z_off = 0;
    if (live) {
      const uint32_t *aw = reinterpret_cast<const uint32_t *>(p.At + (long long)p.at_rowb[pr] * p.at_row_bytes);
      const uint32_t *tw = reinterpret_cast<const uint32_t *>(trow);
      const uint32_t *m = reinterpret_cast<const uint32_t *>(p.mask);
      const uint32_t *p0 = reinterpret_cast<const uint32_t *>(p.planes);
      int c = 0;
      for (int i = 0; i < p.P * kBlockWords; ++i) c += __popc(~(__ldg(aw + i) ^ __ldg(tw + i)) & __ldg(m + i) & __ldg(p0 + i));
      const long long pm = 2ll * c - p.ycnt[0];
      At_base = __dmul_rn(__dmul_rn((double)pm, p.min_d), p.mlt_d);
      aA = p.aA[pr];
      aZ = p.aZ[pr];
      z_off = (long long)p.zt_rowb[pr] * p.zt_row_bytes;
    }
    const double at_base = __dmul_rn(p.T_base[t], aA);
    bool ok = true;
    for (int nt = 0; nt < NT; ++nt) {
      const int b = nt & 1;
      const bool w = ok && tc::mbar_wait(&sm.acc_full[b], (uint32_t)((nt >> 1) & 1), abort, status, 16);
      ok = __all_sync(0xffffffffu, w);
      tc::fence_after_sync();
      const int mwend = min(CW, p.nW - nt * CW);
      for (int mwl = 0; mwl < CW; ++mwl) {
        uint32_t cnt[B];
        if (ok && mwl < mwend) {
          const uint32_t col = lane_base + b * kN + mwl * B;
          if constexpr (B == 32) {
            tc::tmem_ld32(col, cnt);
          } else if constexpr (B == 16) {
            tc::tmem_ld16(col, cnt);
          } else {
            tc::tmem_ld8(col, cnt);
          }
          tc::tmem_wait_ld();
        } else {
#pragma unroll
          for (int k = 0; k < B; ++k) cnt[k] = 0;
        }
        if (mwl == CW - 1) {
          tc::fence_before_sync();
          tc::mbar_arrive(&sm.acc_empty[b]);
        }
        if (!(ok && live && mwl < mwend)) continue;
        const int mw = nt * CW + mwl;
        long long v = 0;
        const int *yc = p.ycnt + 1 + (long long)mw * B;
#pragma unroll
        for (int k = 0; k < B; ++k) v += (2ll * decode_count(cnt[k]) - __ldg(yc + k)) * (1ll << k);
        // the FP64 step, as bitplane_main_kernel does it
        const double At_tmp = (double)v;
        const double at_tmp = __dmul_rn(p.T_tmp[(long long)t * p.nW + mw], aA);
        const double X = __dsub_rn(__ddiv_rn(__dadd_rn(At_base, At_tmp), p.mlt_d),
                                   __ddiv_rn(__dadd_rn(at_base, at_tmp), p.mlt_d));
        const int mwa = (int)p.mw_a[mw];
        const int vZ = ((p.Zt[z_off + (mwa >> 3)] >> (7 - (mwa & 7))) & 1) ? 1 : -1;
        const double vS = (double)p.vS[(long long)t * p.nW + mw];
        acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(X, vS), __dsub_rn((double)vZ, aZ)));
      }
    }
    if (live && ok) p.out[p.out_off[pr] + p.t_off[t]] = acc;
  }

  tc::fence_before_sync();
  __syncthreads();
  if (warp == kMmaWarp) {
    __syncwarp();
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kTmemCols);
  }
}

template <int B>
__global__ void __launch_bounds__(kThreads, 1) bitplane_tc_kernel(BitplaneParams p, int *status) {
  bitplane_tc_cta<B>(p, blockIdx.y, blockIdx.x * kM, status);
}

// Several calls in one launch (a deferral scope's group): CTA k belongs to
// the last call whose tile0 <= k; within it, pair tile (k - tile0) % pair
// tiles, covariate column (k - tile0) / pair tiles.
template <int B>
__global__ void __launch_bounds__(kThreads, 1) bitplane_tc_group_kernel(const BitplaneParams *ps, const int *tile0,
                                                                       int n, int *status) {
  const int k = blockIdx.x;
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tile0[mid] <= k) lo = mid; else hi = mid - 1;
  }
  const BitplaneParams &p = ps[lo];
  const int ptiles = (p.npairs + kM - 1) / kM;
  const int j = k - tile0[lo];
  bitplane_tc_cta<B>(p, j / ptiles, (j % ptiles) * kM, status);
}

template <int B>
void launch_b(const BitplaneParams &p, int nT, cudaStream_t s) {
  static std::once_flag configured;
  std::call_once(configured, [] {
    LAKGB_CUDA(cudaFuncSetAttribute(bitplane_tc_kernel<B>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kSmemBytes));
  });
  dim3 grid((p.npairs + kM - 1) / kM, nT);
  bitplane_tc_kernel<B><<<grid, kThreads, kSmemBytes, s>>>(p, tc_status_device_ptr());
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
}

template <int B>
void launch_group_b(const BitplaneParams *ps, const int *tile0, int n, int tiles, cudaStream_t s) {
  static std::once_flag configured;
  std::call_once(configured, [] {
    LAKGB_CUDA(cudaFuncSetAttribute(bitplane_tc_group_kernel<B>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kSmemBytes));
  });
  bitplane_tc_group_kernel<B><<<tiles, kThreads, kSmemBytes, s>>>(ps, tile0, n, tc_status_device_ptr());
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
}

}  // namespace

void launch_bitplane_tc(const BitplaneParams &p, int nT, cudaStream_t s) {
  if (p.B == 32)
    launch_b<32>(p, nT, s);
  else if (p.B == 16)
    launch_b<16>(p, nT, s);
  else
    launch_b<8>(p, nT, s);
}

int bitplane_tc_tiles(const BitplaneParams &p, int nT) { return ((p.npairs + kM - 1) / kM) * nT; }

void launch_bitplane_tc_group(int B, const BitplaneParams *ps, const int *tile0, int n, int tiles, cudaStream_t s) {
  if (B == 32)
    launch_group_b<32>(ps, tile0, n, tiles, s);
  else if (B == 16)
    launch_group_b<16>(ps, tile0, n, tiles, s);
  else
    launch_group_b<8>(ps, tile0, n, tiles, s);
}

}  // namespace lakgb
