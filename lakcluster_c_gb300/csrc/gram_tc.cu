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
// Persistent CTAs, one per SM, each looping over 128 (A rows) x 128 (Z rows)
// output tiles; the pipeline runs on across tile boundaries.  25 warps:
//   warps 0-7   producers, one tile row each (A rows 0-127, then Z rows
//               0-127): per 128-column chunk, load the row's 16 bytes, mask,
//               expand to 128 e4m3 bytes in shared memory (K-major, 128-byte
//               swizzle), count pa / pz.
//   warp 8      owns TMEM; lane 0 issues the MMAs (M=128, N=128, K=32; 4 per
//               chunk, 15 chunks per block) into one of two count buffers.
//   warps 9-24  fold, four warps per lane quadrant (warp w reads TMEM lanes
//               32*(w%4)..+31), each for 32 of the 128 columns: per block,
//               read the counts from TMEM, look up T_b[c], add into the FP64
//               accumulators, which live in TMEM as well (columns 256..511,
//               two 32-bit halves per value).
// Shared memory: 6 stages x (16 KB A + 16 KB B) + 2 x T_b (15 KB) + counts.
// The T_b buffers are filled by bulk copies on mbarriers, issued by whichever
// fold warp finishes a block last, so fold warps drift apart by up to a block
// instead of meeting at every block boundary.
// TMEM: 512 columns (2 x 128 count columns + 256 accumulator columns).
#include <algorithm>

#include "gram.cuh"
#include "lakgb_runtime.cuh"
#include "tc_ptx.cuh"

namespace lakgb {

// Test hook: when set, producer warp 0 of CTA 0 withholds its arrival for
// the first operand stage, so the MMA warp's wait for that stage runs out
// (lakgb_debug_tc_withhold).
static __device__ int g_withhold;

namespace {

constexpr int kBM = 128, kBN = 128;
constexpr int kStages = 6;
constexpr int kChunks = 15;               // 128-bit chunks per 1920-bit block
constexpr int kPrefetch = 3;              // producer loads in flight (divides kChunks)
constexpr int kStageA = kBM * 128;        // bytes: 128 rows x 128 e4m3
constexpr int kStageB = kBN * 128;
constexpr int kStageBytes = kStageA + kStageB;
constexpr int kTabStride = 1922;          // doubles per block table (1921 used, 16-byte multiple)
constexpr int kTabBytes = kTabStride * 8;
constexpr int kSBO = 8 * 128;             // bytes between 8-row swizzle atoms (8 rows of 128 B)
constexpr int kProducers = 256;           // warps 0-7
constexpr int kMmaWarp = 8;
constexpr int kFold = 512;                // warps 9-24
constexpr int kFoldWarps = kFold / 32;
constexpr int kRound = 4;                 // columns per TMEM round of a fold warp
constexpr int kFoldCols = kBN / (kFold / 128);  // tile columns per fold warp
constexpr int kRounds = kFoldCols / kRound;
constexpr int kThreads = kProducers + 32 + kFold;
constexpr uint32_t kTmemCols = 512;
constexpr size_t kSmemBytes = (size_t)kStages * kStageBytes + 2 * kTabBytes + 2 * (kBM + kBN) * 4 + 1024;

struct Smem {
  uint64_t full[kStages], empty[kStages];
  uint64_t acc_full[2], acc_empty[2], aux_full[2], aux_empty[2], done;
  uint64_t tab_full[2];            // T_b buffer t loaded (bulk copy)
  unsigned tab_read[2];            // fold warps done with buffer t (monotonic)
  unsigned tab_issued[2];          // bulk copies issued into buffer t
  uint32_t tmem_base;
  int abort;
};

// Expand the 128 bits of x into the 128 e4m3 bytes of one tile row (a
// 128-byte row of a 128-byte-swizzled atom): word q of x fills the 16-byte
// chunks 2q and 2q+1, stored at chunk index c ^ sw (sw = row % 8).
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

template <int R>
__device__ __forceinline__ void tmem_ld_n(uint32_t taddr, uint32_t (&v)[R]) {
  if constexpr (R == 4) tc::tmem_ld4(taddr, v);
  else if constexpr (R == 8) tc::tmem_ld8(taddr, v);
  else if constexpr (R == 16) tc::tmem_ld16(taddr, v);
  else tc::tmem_ld32(taddr, v);
}
template <int R>
__device__ __forceinline__ void tmem_st_n(uint32_t taddr, const uint32_t (&v)[R]) {
  if constexpr (R == 8) tc::tmem_st8(taddr, v);
  else if constexpr (R == 16) tc::tmem_st16(taddr, v);
  else tc::tmem_st32(taddr, v);
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

// (tile_m, tile_n) of tile r of one Gram's list.  A full grid is walked in
// bands of kBand tile rows, each band column by column: the CTAs of a wave
// (consecutive r) then share a few A row panels and a few Z row panels, a
// working set that stays in L2 even when a whole side of the product does
// not (32768-row bins: 2 MB per 128-row panel).  A symmetric Gram with a
// square tile grid lists only the pairs on or above the diagonal, row by row.
constexpr int kBand = 8;
__device__ __forceinline__ void tile_coords(int ntm, int ntn, bool tri, int r, int &tile_m, int &tile_n) {
  if (!tri) {
    const int band = r / (kBand * ntn), in = r - band * (kBand * ntn);
    const int rows = min(kBand, ntm - band * kBand);
    tile_m = (band * kBand + in % rows) * kBM;
    tile_n = (in / rows) * kBN;
    return;
  }
  int i = 0;
  while (r >= ntn - i) {  // row i of the upper triangle holds ntn - i tiles
    r -= ntn - i;
    ++i;
  }
  tile_m = i * kBM;
  tile_n = (i + r) * kBN;
}

// The instance of a grouped launch that holds global tile (or table row) k:
// the last i with start[i] <= k.
template <typename I>
__device__ __forceinline__ int find_instance(const I *start, int n, long long k) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if ((long long)start[mid] <= k) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Tile order shared by every role: tile k of the launch's list goes to CTA
// k % gridDim.x, so the active tiles, not all tiles, are spread evenly over
// the CTAs.  A single Gram lists its own tiles (tile_coords; a symmetric call
// with unequal row counts skips the tiles below the diagonal as it walks); a
// grouped launch lists the tiles of its instances one instance after another.
template <bool GRP>
struct TileWalk {
  int ntm, ntn, ntiles, k;
  bool tri;
  __device__ TileWalk(const GramParams &p, const GramGroupDev &g) : k((int)blockIdx.x - (int)gridDim.x) {
    if (GRP) {
      ntiles = g.tile0[g.n];
      ntm = ntn = 0;
      tri = false;
    } else {
      ntn = (p.nZ + kBN - 1) / kBN;
      ntm = (p.nA + kBM - 1) / kBM;
      tri = p.symmetric && ntm == ntn;
      ntiles = tri ? ntn * (ntn + 1) / 2 : ntm * ntn;
    }
  }
  __device__ bool next(const GramParams &p, const GramGroupDev &g, int &inst, int &tile_m, int &tile_n) {
    if (GRP) {
      k += gridDim.x;
      if (k >= ntiles) return false;
      inst = find_instance(g.tile0, g.n, k);
      const GramParams &q = g.ps[inst];
      const int n_z = (q.nZ + kBN - 1) / kBN, n_m = (q.nA + kBM - 1) / kBM;
      tile_coords(n_m, n_z, q.symmetric && n_m == n_z, k - g.tile0[inst], tile_m, tile_n);
      return true;
    }
    inst = 0;
    for (;;) {
      k += gridDim.x;
      if (k >= ntiles) return false;
      tile_coords(ntm, ntn, tri, k, tile_m, tile_n);
      if (tri || !(p.symmetric && tile_m > tile_n + kBN - 1)) return true;
    }
  }
};

// The parameters of instance `inst` (a grouped launch) or the launch's own.
template <bool GRP>
__device__ __forceinline__ const GramParams &params_of(const GramParams &p, const GramGroupDev &g, int inst) {
  if constexpr (GRP) return g.ps[inst];
  else return p;
}

template <int TYPE, bool GRP>
__global__ void __launch_bounds__(kThreads, 1)
    gram_tc_kernel(GramParams p, GramGroupDev grp, const double *__restrict__ T, int *status) {
  extern __shared__ __align__(128) uint8_t dsm[];
  __shared__ Smem sm;
  // stages first, on a 1024-byte boundary (swizzle atoms)
  uint8_t *stages = dsm + ((1024 - (tc::smem_u32(dsm) & 1023)) & 1023);
  double *sT = reinterpret_cast<double *>(stages + (size_t)kStages * kStageBytes);  // [2][kTabStride]
  int *s_cnt = reinterpret_cast<int *>(stages + (size_t)kStages * kStageBytes + 2 * kTabBytes);  // [2][256]

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  volatile int *abort = &sm.abort;

  if (tid == 0) {
    for (int s = 0; s < kStages; ++s) {
      tc::mbar_init(&sm.full[s], kProducers / 32);  // one arrival per warp
      tc::mbar_init(&sm.empty[s], 1);
    }
    for (int t = 0; t < 2; ++t) {
      tc::mbar_init(&sm.acc_full[t], 1);
      tc::mbar_init(&sm.acc_empty[t], kFoldWarps);
      tc::mbar_init(&sm.aux_full[t], kProducers / 32);
      tc::mbar_init(&sm.aux_empty[t], kFoldWarps);
      tc::mbar_init(&sm.tab_full[t], 1);
      sm.tab_read[t] = sm.tab_issued[t] = 0;
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
  TileWalk<GRP> walk(p, grp);
  int inst, tile_m, tile_n;

  if (tid < kProducers) {
    // ---------------- producers ----------------
    const int side = tid >> 7, rr = tid & 127;  // side 0: A row rr, side 1: Z row rr
    const uint32_t st0 = tc::smem_u32(stages);
    const uint32_t my_row = st0 + side * kStageA + (uint32_t)((rr >> 3) * kSBO + (rr & 7) * 128);
    const uint32_t my_sw = (uint32_t)(rr & 7);
    // the test hook, read once: this thread withholds its first arrival
    bool withhold = g_withhold && blockIdx.x == 0 && tid == 0;
    bool ok = true;
    // ring position of the next chunk: stage s, in pass `wrap` over the ring
    int s = 0, wrap = 0;
    int gbb = 0;  // blocks this CTA has produced
    while (walk.next(p, grp, inst, tile_m, tile_n)) {
      const GramParams &q = params_of<GRP>(p, grp, inst);
      const uint8_t *base = side ? q.wZ : q.wA;
      const uint32_t *rowb = side ? q.z_rowb : q.a_rowb;
      const long long row_bytes = side ? q.z_row_bytes : q.a_row_bytes;
      const int nrows = side ? q.nZ : q.nA;
      const uint8_t *mask = q.mask;
      const int G = q.P * kChunks;
      const int grow = (side ? tile_n : tile_m) + rr;
      const long long ro = grow < nrows ? (long long)rowb[grow] * row_bytes : -1;
      uint4 rm[kPrefetch], rx[kPrefetch];
      // chunk g of the tile covers bytes 16g..16g+15 of each row (blocks of
      // 240 bytes are contiguous)
      auto load = [&](int g, uint4 &m, uint4 &x) {
        m = x = make_uint4(0, 0, 0, 0);
        if (g < G) {
          m = __ldg(reinterpret_cast<const uint4 *>(mask) + g);
          if (ro >= 0) x = __ldg(reinterpret_cast<const uint4 *>(base + ro) + g);
        }
      };
#pragma unroll
      for (int u = 0; u < kPrefetch; ++u) load(u, rm[u], rx[u]);
      int cnt = 0, ch = 0;
      for (int g0 = 0; g0 < G; g0 += kPrefetch) {
#pragma unroll
        for (int u = 0; u < kPrefetch; ++u) {
          const int g = g0 + u;
          const uint4 m = rm[u];
          const uint4 xm = and4(rx[u], m);
          // A rows enter masked; Z rows unmasked (the mask on A already
          // restricts every product), their count masked
          const uint4 x = side ? rx[u] : xm;
          load(g + kPrefetch, rm[u], rx[u]);
          if (TYPE == 1) cnt += popc4(xm);
          if (wrap > 0 && ok) ok = tc::mbar_wait(&sm.empty[s], (uint32_t)((wrap - 1) & 1), abort, status, 1);
          if (ok) {
            expand_row(my_row + s * kStageBytes, my_sw, x);
            tc::fence_proxy_async();
          }
          __syncwarp();
          if (lane == 0 && !withhold) tc::mbar_arrive(&sm.full[s]);
          withhold = false;
          if (++s == kStages) {
            s = 0;
            ++wrap;
          }
          if (++ch == kChunks) {
            // end of a block: publish the row counts
            const int t = gbb & 1;
            if (gbb >= 2 && ok)
              ok = tc::mbar_wait(&sm.aux_empty[t], (uint32_t)(((gbb >> 1) - 1) & 1), abort, status, 2);
            s_cnt[t * 256 + tid] = cnt;
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&sm.aux_full[t]);
            cnt = 0;
            ch = 0;
            ++gbb;
          }
        }
      }
    }
  } else if (warp == kMmaWarp) {
    // ---------------- MMA issue ----------------
    if (lane == 0) {
      constexpr uint32_t idesc = tc::idesc_e4m3_f32(kBM, kBN);
      const uint32_t st0 = tc::smem_u32(stages);
      bool ok = true;
      int s = 0, wrap = 0, gbb = 0;
      while (ok && walk.next(p, grp, inst, tile_m, tile_n)) {
        const int P = params_of<GRP>(p, grp, inst).P;
        for (int b = 0; b < P && ok; ++b, ++gbb) {
          const int t = gbb & 1;
          if (gbb >= 2)
            ok = tc::mbar_wait(&sm.acc_empty[t], (uint32_t)(((gbb >> 1) - 1) & 1), abort, status, 3);
          tc::fence_after_sync();
          for (int ch = 0; ch < kChunks && ok; ++ch) {
            const int cs = s;
            ok = tc::mbar_wait(&sm.full[cs], (uint32_t)(wrap & 1), abort, status, 4);
            if (++s == kStages) {
              s = 0;
              ++wrap;
            }
            if (!ok) break;
            tc::fence_after_sync();
            const uint32_t sa = st0 + cs * kStageBytes, sb = sa + kStageA;
#pragma unroll
            for (int kk = 0; kk < 4; ++kk) {
              const uint64_t ad = tc::smem_desc_sw128(sa + kk * 32, kSBO);
              const uint64_t bd = tc::smem_desc_sw128(sb + kk * 32, kSBO);
              tc::mma_e4m3(tmem + t * kBN, ad, bd, idesc, (ch | kk) != 0);
            }
            tc::mma_commit(&sm.empty[cs]);
          }
          if (ok) tc::mma_commit(&sm.acc_full[t]);
        }
      }
      // every issued MMA has completed before TMEM is released (waited for
      // even after an abort, within the same time limit)
      tc::mma_commit(&sm.done);
      const unsigned long long t0 = tc::globaltimer();
      while (!tc::mbar_try(&sm.done, 0)) {
        if (tc::globaltimer() - t0 > tc::g_wait_ns) {
          atomicCAS(status, 0, 5);
          break;
        }
      }
    }
  } else {
    // ---------------- FP64 fold ----------------
    const int et = tid - (kProducers + 32);  // 0..kFold-1
    const int q = warp & 3;
    const int col0 = (et >> 7) * kFoldCols;   // this warp's columns of the tile
    const int row = 32 * q + lane;
    const uint32_t lane_base = tmem + ((uint32_t)(32 * q) << 16);
    // The table T_b of the CTA's g-th block goes into buffer g & 1 by one
    // bulk copy.  Copies g = 0, 1 start here; the last fold warp to finish
    // block g issues g + 2 into the buffer g read, so the fold warps are never
    // held together at block boundaries.  issue_table(t, jt, boff) loads the
    // block `boff` blocks after the start of this CTA's tile jt: block
    // boff % P of a single Gram (every tile has P blocks); in a grouped launch
    // it is found by walking on through this CTA's tiles, and nothing is
    // loaded past its last block.  (Copies issued past the CTA's last block
    // of a single Gram are waited for at the end.)
    const int ntiles_grp = GRP ? grp.tile0[grp.n] : 0;
    auto issue_table = [&](int t, int jt, int boff) {
      int in = 0, blk = 0;
      if constexpr (GRP) {
        for (;;) {
          const int k = (int)blockIdx.x + jt * (int)gridDim.x;
          if (k >= ntiles_grp) return;
          in = find_instance(grp.tile0, grp.n, k);
          const int pj = grp.ps[in].P;
          if (boff < pj) break;
          boff -= pj;
          ++jt;
        }
        blk = boff;
      } else {
        blk = boff % p.P;
      }
      const double *src = T + ((GRP ? grp.blk0[in] : 0ll) + blk) * (long long)kTabStride;
      tc::fence_proxy_async();
      tc::mbar_arrive_expect_tx(&sm.tab_full[t], kTabBytes);
      tc::bulk_g2s(sT + t * kTabStride, src, kTabBytes, &sm.tab_full[t]);
      atomicAdd(&sm.tab_issued[t], 1u);
    };
    if (et == 0) {
      issue_table(0, 0, 0);
      issue_table(1, 0, 1);
    }
    bool ok = true;
    long long gb0 = 0;
    int jt = 0;  // this CTA's tiles so far
    while (walk.next(p, grp, inst, tile_m, tile_n)) {
      const GramParams &pp = params_of<GRP>(p, grp, inst);
      const int P = pp.P;
      const int ga = tile_m + row;
      const bool row_in = ga < pp.nA;
      const double lfa = (pp.lfA && row_in) ? pp.lfA[ga] : 0.0;
      const long long orow = row_in ? (long long)pp.out_r[ga] : 0;
      const long long ocol2 = (pp.symmetric && row_in) ? (long long)pp.out_c2[ga] * pp.out_stride : 0;
      for (int b = 0; b < P; ++b) {
        const long long gbb = gb0 + b;
        const int t = (int)(gbb & 1);
        bool w = ok && tc::mbar_wait(&sm.tab_full[t], (uint32_t)((gbb >> 1) & 1), abort, status, 8);
        w = w && tc::mbar_wait(&sm.aux_full[t], (uint32_t)((gbb >> 1) & 1), abort, status, 6);
        w = w && tc::mbar_wait(&sm.acc_full[t], (uint32_t)((gbb >> 1) & 1), abort, status, 7);
        ok = __all_sync(0xffffffffu, w);
        tc::fence_after_sync();
        const double *Tb = sT + t * kTabStride;
        const int pa = s_cnt[t * 256 + row];
        const int *pzb = s_cnt + t * 256 + 128;
        // Rounds of kRound columns, software-pipelined: the TMEM loads of
        // round r + 1 (counts, and accumulators after block 0) are in flight
        // while round r is added, so their latency hides behind the adds.
        uint32_t cn[2][kRound], a[2][2 * kRound];
        auto load_round = [&](int r, int buf) {
          const int c0 = col0 + r * kRound;
          tmem_ld_n<kRound>(lane_base + t * kBN + c0, cn[buf]);
          if (b > 0) tmem_ld_n<2 * kRound>(lane_base + 256 + 2 * c0, a[buf]);
        };
        if (ok) {
          load_round(0, 0);
          tc::tmem_wait_ld();
          tc::reg_fence(cn[0]);
          tc::reg_fence(a[0]);
        }
#pragma unroll
        for (int r = 0; r < kRounds; ++r) {
          const int cur = r & 1, nxt = cur ^ 1;
          const int c0 = col0 + r * kRound;
          if (!ok) {
#pragma unroll
            for (int j = 0; j < kRound; ++j) cn[cur][j] = 0;
          }
          if (ok && r + 1 < kRounds) load_round(r + 1, nxt);
          if (r == kRounds - 1) {
            // all this warp's count columns of buffer t have been read
            tc::fence_before_sync();
            __syncwarp();
            if (lane == 0) tc::mbar_arrive(&sm.acc_empty[t]);
          }
          // the four columns' Z row counts in one 16-byte load (c0 is a
          // multiple of kRound = 4)
          static_assert(kRound == 4, "one int4 of Z row counts per round");
          const int4 pz4 = *reinterpret_cast<const int4 *>(pzb + c0);
          const int pzr[4] = {pz4.x, pz4.y, pz4.z, pz4.w};
#pragma unroll
          for (int j = 0; j < kRound; ++j) {
            const int n = decode_count(cn[cur][j]);
            const int c = (TYPE == 1) ? pa + pzr[j] - 2 * n : n;
            // 0 <= c <= 1920 for counts of a completed block; anything else
            // (counts of an aborted pipeline) reads the NaN entry 1921
            const double x = Tb[min((unsigned)c, (unsigned)(kTabStride - 1))];
            const double v =
                (b > 0) ? __dadd_rn(__hiloint2double((int)a[cur][2 * j + 1], (int)a[cur][2 * j]), x) : x;
            a[cur][2 * j] = (uint32_t)__double2loint(v);
            a[cur][2 * j + 1] = (uint32_t)__double2hiint(v);
          }
          if (b + 1 < P) {
            // accumulators of columns c0 + j: TMEM columns 256 + 2 (c0 + j)
            // (low word) and + 1 (high word)
            if (ok) tmem_st_n<2 * kRound>(lane_base + 256 + 2 * c0, a[cur]);
          } else if (ok && row_in) {
#pragma unroll
            for (int j = 0; j < kRound; ++j) {
              const int gz = tile_n + c0 + j;
              if (gz >= pp.nZ || (pp.symmetric && ga > gz)) continue;
              const double v = __hiloint2double((int)a[cur][2 * j + 1], (int)a[cur][2 * j]);
              double o = (TYPE == 1) ? __dsub_rn(pp.a0d1, twice(v)) : v;
              if (pp.lfA && pp.lfZ) o = __dsub_rn(o, __dsub_rn(__dadd_rn(lfa, pp.lfZ[gz]), pp.a2d1));
              pp.out[orow + (long long)pp.out_c[gz] * pp.out_stride] = o;
              if (pp.symmetric) pp.out[(long long)pp.out_r2[gz] + ocol2] = o;
            }
          }
          if (ok && r + 1 < kRounds) {
            tc::tmem_wait_ld();
            tc::reg_fence(cn[nxt]);
            tc::reg_fence(a[nxt]);
          }
        }
        // this warp no longer reads T buffer t; the last of the fold warps
        // to get here loads block gbb + 2 into it (after the copy it read
        // has landed; no new copies once the CTA has aborted)
        __syncwarp();
        if (lane == 0) {
          __threadfence_block();
          const unsigned prev = atomicAdd(&sm.tab_read[t], 1u);
          if ((prev + 1) % kFoldWarps == 0) {
            __threadfence_block();
            if (!*abort) {
              if (tc::mbar_wait_landed(&sm.tab_full[t], (uint32_t)((gbb >> 1) & 1)))
                issue_table(t, jt, b + 2);
              else
                atomicCAS(status, 0, 9);
            }
          }
        }
        __syncwarp();
        if (ok) tc::tmem_wait_st();
        __syncwarp();
        if (lane == 0) tc::mbar_arrive(&sm.aux_empty[t]);
      }
      gb0 += P;
      ++jt;
    }
    // every bulk copy into the tables has landed before the CTA exits (each
    // copy was issued after the previous one into its buffer landed)
    tc::named_bar_sync(1, kFold);
    if (et == 0) {
      for (int t = 0; t < 2; ++t) {
        const unsigned n = *(volatile unsigned *)&sm.tab_issued[t];
        if (n && !tc::mbar_wait_landed(&sm.tab_full[t], (n - 1) & 1)) atomicCAS(status, 0, 10);
      }
    }
  }

  tc::fence_before_sync();
  __syncthreads();
  if (warp == kMmaWarp) {
    __syncwarp();
    tc::fence_after_sync();
    tc::tmem_dealloc(tmem, kTmemCols);
  }
}

__device__ __forceinline__ void write_table_row(double d, double *__restrict__ row) {
  for (int c = threadIdx.x; c < kTabStride; c += blockDim.x)
    row[c] = c < kTabStride - 1 ? __dmul_rn(d, (double)c) : __longlong_as_double(0x7ff8dead00000000ll);
}

__global__ void gram_table_kernel(const double *__restrict__ D, int P, double *__restrict__ T) {
  const int b = blockIdx.x;
  write_table_row(D ? D[b] : 1.0, T + (size_t)b * kTabStride);
}

// Table rows of a grouped launch: row r is block r - blk0[i] of instance i.
__global__ void gram_table_group_kernel(GramGroupDev g, double *__restrict__ T) {
  const long long r = blockIdx.x;
  const int in = find_instance(g.blk0, g.n, r);
  const double *D = g.ps[in].D;
  write_table_row(D ? D[r - g.blk0[in]] : 1.0, T + (size_t)r * kTabStride);
}

int sm_count() {
  static int n = 0;
  if (!n) {
    int dev = 0;
    LAKGB_CUDA(cudaGetDevice(&dev));
    LAKGB_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
  }
  return n;
}

// Tiles a launch computes (symmetric Grams: the tiles on or above the
// diagonal of the square tile grid).
int active_tiles(const GramParams &p) {
  const int ntm = (p.nA + kBM - 1) / kBM, ntn = (p.nZ + kBN - 1) / kBN;
  return (p.symmetric && ntm == ntn) ? ntn * (ntn + 1) / 2 : ntm * ntn;
}

template <int TYPE, bool GRP>
void configure_tc() {
  static bool configured = false;
  if (!configured) {
    LAKGB_CUDA(cudaFuncSetAttribute(gram_tc_kernel<TYPE, GRP>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)kSmemBytes));
    configured = true;
  }
}

template <int TYPE>
void launch_tc_type(const GramParams &p, const double *T, cudaStream_t s) {
  configure_tc<TYPE, false>();
  const int grid = std::max(1, std::min(active_tiles(p), sm_count()));
  gram_tc_kernel<TYPE, false><<<grid, kThreads, kSmemBytes, s>>>(p, GramGroupDev{}, T, tc_status_device_ptr());
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
}

template <int TYPE>
void launch_tc_group_type(const GramGroupDev &g, int total_tiles, const double *T, cudaStream_t s) {
  configure_tc<TYPE, true>();
  const int grid = std::max(1, std::min(total_tiles, sm_count()));
  gram_tc_kernel<TYPE, true><<<grid, kThreads, kSmemBytes, s>>>(GramParams{}, g, T, tc_status_device_ptr());
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

int gram_tc_tiles(const GramParams &p) { return active_tiles(p); }

size_t gram_tc_table_row_bytes() { return (size_t)kTabBytes; }

void launch_gram_tc_group(const GramGroupDev &g, int type, int total_tiles, long long total_blocks, double *T,
                          cudaStream_t s) {
  if (total_tiles <= 0 || total_blocks <= 0) return;
  gram_table_group_kernel<<<(unsigned)total_blocks, 256, 0, s>>>(g, T);
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
  if (type == 1)
    launch_tc_group_type<1>(g, total_tiles, T, s);
  else
    launch_tc_group_type<2>(g, total_tiles, T, s);
}

// The status word of the calling host thread's launches: every thread (a
// solve, a server worker) has its own, so a pipeline timeout in one solve is
// reported to that solve alone.  Zeroed on the thread's own stream (which
// does not wait for the legacy default stream).
namespace {
thread_local int *t_status = nullptr;
}

int *tc_status_device_ptr() {
  if (!t_status) {
    LAKGB_CUDA(cudaMalloc(reinterpret_cast<void **>(&t_status), sizeof(int)));
    LAKGB_CUDA(cudaMemsetAsync(t_status, 0, sizeof(int), stream()));
  }
  return t_status;
}

// Read and clear the calling thread's status word (after every launch made
// so far has finished: the launches may be on a caller's stream).
int tc_status_take() {
  if (!t_status) return 0;
  int v = 0;
  LAKGB_CUDA(cudaDeviceSynchronize());
  LAKGB_CUDA(cudaMemcpy(&v, t_status, sizeof v, cudaMemcpyDeviceToHost));
  if (v) {
    LAKGB_CUDA(cudaMemsetAsync(t_status, 0, sizeof(int), stream()));
    LAKGB_CUDA(cudaStreamSynchronize(stream()));
  }
  return v;
}

// As tc_status_take, for launches on the calling thread's own stream only
// (a whole solve): waits for that stream, not for the device.
int tc_status_take_stream() {
  if (!t_status) return 0;
  int v = 0;
  LAKGB_CUDA(cudaMemcpyAsync(&v, t_status, sizeof v, cudaMemcpyDeviceToHost, stream()));
  LAKGB_CUDA(cudaStreamSynchronize(stream()));
  if (v) {
    LAKGB_CUDA(cudaMemsetAsync(t_status, 0, sizeof(int), stream()));
    LAKGB_CUDA(cudaStreamSynchronize(stream()));
  }
  return v;
}

void tc_debug_set(unsigned long long wait_ns, int withhold) {
  LAKGB_CUDA(cudaDeviceSynchronize());
  LAKGB_CUDA(cudaMemcpyToSymbol(tc::g_wait_ns, &wait_ns, sizeof wait_ns));
  LAKGB_CUDA(cudaMemcpyToSymbol(g_withhold, &withhold, sizeof withhold));
  LAKGB_CUDA(cudaDeviceSynchronize());
}

}  // namespace lakgb

// ---------------------------------------------------------------------------
// Throughput of the FP64 add on this device: the pipe that bounds the fold of
// the tensor-core Gram (one add per element per block).  Independent add
// chains on every SM, timed with CUDA events.

namespace lakgb {
namespace {

__global__ void fp64_add_rate_kernel(double *out, double y, int iters) {
  double a[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) a[j] = threadIdx.x * 1e-3 + j;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 8; ++j) a[j] = __dadd_rn(a[j], y);
  }
  double s = 0.0;
#pragma unroll
  for (int j = 0; j < 8; ++j) s = __dadd_rn(s, a[j]);
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace
}  // namespace lakgb

extern "C" double lakgb_measure_fp64_add_rate(void) {
  using namespace lakgb;
  const int blocks = sm_count() * 4, threads = 256, iters = 4096;
  double *d = nullptr;
  cudaEvent_t e0, e1;
  LAKGB_CUDA(cudaMalloc(&d, sizeof(double) * blocks * threads));
  LAKGB_CUDA(cudaEventCreate(&e0));
  LAKGB_CUDA(cudaEventCreate(&e1));
  float best = 0.f;
  for (int rep = 0; rep < 4; ++rep) {
    LAKGB_CUDA(cudaEventRecord(e0, stream()));
    fp64_add_rate_kernel<<<blocks, threads, 0, stream()>>>(d, 1.5e-9, iters);
    LAKGB_CUDA(cudaGetLastError());
    count_launch();
    LAKGB_CUDA(cudaEventRecord(e1, stream()));
    LAKGB_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    LAKGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    if (rep > 0 && (best == 0.f || ms < best)) best = ms;
  }
  LAKGB_CUDA(cudaEventDestroy(e0));
  LAKGB_CUDA(cudaEventDestroy(e1));
  LAKGB_CUDA(cudaFree(d));
  return (double)blocks * threads * iters * 8 / (best * 1e-3);
}
