// Products that read the bit planes made by wrap_xcalc.
//
// At_T_YnWt_S_Zn_ww (dir_c/At_T_YnWt_S_Zn_ww.c:5-190, wrapper :435-466): for
// each paired covariate column t (Tt row nt_j with St row ns_j) and each
// paired SNP (At row na_j with Zt row nz_j),
//   out[na, t] = sum over Wn rows mw, in order, of
//       X(na, mw) * vS(t, mw) * (vZ(nz, mw) - a[nz])
//   X = (At_base + At_tmp[mw]) / mlt - (a[na]*T_base + a[na]*T_tmp[mw]) / mlt
// where, with pmpm0(a, t, y) = #(+1 products) - #(-1 products) of (a.t) over
// the bits set in y (popcount_pmpm0, dir_c/popcount.c:492-540), masked by
// M_At->mc_j,
//   At_tmp[mw] = sum_nb 2^nb pmpm0(At_na, Tt_t, plane(mw, nb))   (exact int)
//   At_base    = pmpm0(At_na, Tt_t, plane 0) * min * mlt
//   T_tmp[mw]  = sum_nb 2^nb pmpm0(plane 0, Tt_t, plane(mw, nb))
//   T_base     = pmpm0(plane 0, Tt_t, plane 0) * min * mlt.
// Integer parts are exact; the FP64 part repeats the reference's operations
// in its order (left-to-right, no FMA, sequential over mw).
//
// An_ZtSn_ww (dir_c/An_ZtSn_ww.c:5-136): out[ma, s] =
//   (pm0(An_ma, plane 0)*min*mlt + sum_nb 2^nb pm0(An_ma, plane(s, nb))) / mlt
// with pm0(a, y) = #(a=+1, y=1) - #(a=-1, y=1) over M_An->mc_j
// (popcount_pm0, popcount.c:425-490).
//
// Kernel layout for At_T_YnWt_S_Zn_ww: one CTA per (32 SNP pairs, t).  It
// walks the Wn rows in chunks of 256/B (B value planes each); per 1920-bit
// block it stages the 32 rows a' = ~(At ^ Tt) & mask and the chunk's 256
// plane rows in shared memory, and each thread accumulates a 4 x 8 tile of
// popcount(a' & plane).  With pmpm0 = 2*popcount(a' & y) - popcount(y & mask),
// the chunk's counts fold into exact At_tmp values, and 32 threads (one per
// SNP) then run the FP64 recurrence over the chunk's Wn rows in order.
#include <atomic>
#include <mutex>
#include <optional>

#include "abi_common.cuh"
#include "bcc_model.h"
#include "bitplane.cuh"
#include "gram.cuh"

namespace lakgb {

namespace {

constexpr int kLd = kBlockWords + 1;   // smem row pitch (words)
constexpr int kBP_M = 32;              // SNP pairs per CTA
constexpr int kBP_N = 256;             // plane rows per chunk
constexpr int kBP_T = 256;             // threads

__device__ __forceinline__ int plane_row(int mw, int k, int ncols_per) {
  return mw * ncols_per + ncols_per - 1 - k;
}

// pmpm0 pieces for plane 0 / value planes against plane 0 combined with Tt:
// warp per plane row.  pm[t][q] = 2*popcount(~(p0 ^ t) & y & m) - popcount(y & m)
// for q = 0 (plane 0 itself) and q = 1 + mw*B + k (value plane of bit k).
__global__ void bitplane_prep_kernel(BitplaneParams p, int nT, int *pm, int *ycnt) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int nq = 1 + p.nW * p.B;
  if (warp >= nq * nT) return;
  const int q = warp % nq, t = warp / nq;
  const int prow = q == 0 ? 0 : plane_row((q - 1) / p.B, (q - 1) % p.B, p.ncols_per);
  const uint32_t *y = reinterpret_cast<const uint32_t *>(p.planes + (long long)prow * p.plane_bytes);
  const uint32_t *p0 = reinterpret_cast<const uint32_t *>(p.planes);
  const uint32_t *tt = reinterpret_cast<const uint32_t *>(p.Tt + (long long)p.tt_rowb[t] * p.tt_row_bytes);
  const uint32_t *m = reinterpret_cast<const uint32_t *>(p.mask);
  const int nw = p.P * kBlockWords;
  int c = 0, yc = 0;
  for (int i = lane; i < nw; i += 32) {
    const uint32_t ym = __ldg(y + i) & __ldg(m + i);
    yc += __popc(ym);
    c += __popc(~(__ldg(p0 + i) ^ __ldg(tt + i)) & ym);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    c += __shfl_xor_sync(0xffffffffu, c, o);
    yc += __shfl_xor_sync(0xffffffffu, yc, o);
  }
  if (lane == 0) {
    pm[(long long)t * nq + q] = 2 * c - yc;
    if (t == 0) ycnt[q] = yc;
  }
}

// T_base[t] = pm[t][0] * min * mlt;  T_tmp[t][mw] = sum_k 2^k pm[t][1 + mw*B + k]
// (sums of exact integers, accumulated in the reference's order).
__global__ void bitplane_tsum_kernel(BitplaneParams p, int nT, const int *pm, double *T_base,
                                     double *T_tmp) {
  const int idx = blockIdx.x * blockDim.x + threadIdx.x;
  const int nq = 1 + p.nW * p.B;
  if (idx >= nT * (p.nW + 1)) return;
  const int t = idx / (p.nW + 1), mw = idx % (p.nW + 1) - 1;
  const int *row = pm + (long long)t * nq;
  if (mw < 0) {
    T_base[t] = __dmul_rn(__dmul_rn((double)row[0], p.min_d), p.mlt_d);
    return;
  }
  double s = 0.0, n2 = 1.0;
  for (int k = 0; k < p.B; ++k) {
    s = __dadd_rn(s, __dmul_rn(n2, (double)row[1 + mw * p.B + k]));
    n2 *= 2.0;
  }
  T_tmp[(long long)t * p.nW + mw] = s;
}

__global__ void __launch_bounds__(kBP_T, 1)
bitplane_main_kernel(BitplaneParams p) {
  // Dynamic shared memory, two phases: the block loop stages As (kBP_M x kLd
  // words) and Ys (kBP_N x kLd words); after it, cnt (kBP_M x (kBP_N+1) ints)
  // and tmpd (kBP_M x CW doubles) reuse the same bytes.
  extern __shared__ __align__(16) uint32_t smem[];
  uint32_t *As = smem;
  uint32_t *Ys = smem + kBP_M * kLd;
  int *cnt = reinterpret_cast<int *>(smem);
  double *tmpd = reinterpret_cast<double *>(smem + kBP_M * (kBP_N + 1));
  __shared__ long long a_off[kBP_M];
  __shared__ int yrow[kBP_N];
  __shared__ int base_cnt[kBP_M];

  const int t = blockIdx.y;
  const int pair0 = blockIdx.x * kBP_M;
  const int tid = threadIdx.x;
  const int tx = tid & 31;        // planes tx, tx+32, ..., tx+224
  const int ty = tid >> 5;        // SNP rows 4*ty .. 4*ty+3
  const uint8_t *trow = p.Tt + (long long)p.tt_rowb[t] * p.tt_row_bytes;
  const int CW = kBP_N / p.B;     // Wn rows per chunk

  for (int i = tid; i < kBP_M; i += kBP_T)
    a_off[i] = (pair0 + i < p.npairs) ? (long long)p.at_rowb[pair0 + i] * p.at_row_bytes : -1;
  __syncthreads();

  // At_base counts: popcount(a' & p0), warp w handles rows 4w..4w+3.
  {
    const int warp = tid >> 5, lane = tid & 31;
    const uint32_t *p0 = reinterpret_cast<const uint32_t *>(p.planes);
    const uint32_t *m = reinterpret_cast<const uint32_t *>(p.mask);
    const uint32_t *tw = reinterpret_cast<const uint32_t *>(trow);
    const int nw = p.P * kBlockWords;
    for (int r = warp * 4; r < warp * 4 + 4; ++r) {
      int c = 0;
      if (a_off[r] >= 0) {
        const uint32_t *aw = reinterpret_cast<const uint32_t *>(p.At + a_off[r]);
        for (int i = lane; i < nw; i += 32)
          c += __popc(~(__ldg(aw + i) ^ __ldg(tw + i)) & __ldg(m + i) & __ldg(p0 + i));
      }
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
      if (lane == 0) base_cnt[r] = c;
    }
  }
  __syncthreads();

  // Per-SNP state, held by threads tid < kBP_M.
  double acc = 0.0, At_base = 0.0, aA = 0.0, aZ = 0.0;
  long long z_off = 0;
  const double T_base = p.T_base[t];
  if (tid < kBP_M && pair0 + tid < p.npairs) {
    const long long pm = 2ll * base_cnt[tid] - p.ycnt[0];
    At_base = __dmul_rn(__dmul_rn((double)pm, p.min_d), p.mlt_d);
    aA = p.aA[pair0 + tid];
    aZ = p.aZ[pair0 + tid];
    z_off = (long long)p.zt_rowb[pair0 + tid] * p.zt_row_bytes;
  }
  const double at_base = __dmul_rn(T_base, aA);

  for (int mw0 = 0; mw0 < p.nW; mw0 += CW) {
    for (int q = tid; q < kBP_N; q += kBP_T) {
      const int mwl = q / p.B, k = q % p.B;
      yrow[q] = (q < CW * p.B && mw0 + mwl < p.nW) ? plane_row(mw0 + mwl, k, p.ncols_per) : -1;
    }
    int c[4][8];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) c[i][j] = 0;

    for (int blk = 0; blk < p.P; ++blk) {
      __syncthreads();
      const long long boff = (long long)blk * kBlockBytes;
      const uint4 *mk = reinterpret_cast<const uint4 *>(p.mask + boff);
      const uint4 *tk = reinterpret_cast<const uint4 *>(trow + boff);
      for (int idx = tid; idx < kBP_M * 15; idx += kBP_T) {
        const int r = idx / 15, v = idx - r * 15;
        uint4 x = make_uint4(0u, 0u, 0u, 0u);
        if (a_off[r] >= 0) {
          const uint4 a = __ldg(reinterpret_cast<const uint4 *>(p.At + a_off[r] + boff) + v);
          const uint4 tt = __ldg(tk + v), m = __ldg(mk + v);
          x.x = ~(a.x ^ tt.x) & m.x; x.y = ~(a.y ^ tt.y) & m.y;
          x.z = ~(a.z ^ tt.z) & m.z; x.w = ~(a.w ^ tt.w) & m.w;
        }
        uint32_t *d = As + r * kLd + 4 * v;
        d[0] = x.x; d[1] = x.y; d[2] = x.z; d[3] = x.w;
      }
      for (int idx = tid; idx < kBP_N * 15; idx += kBP_T) {
        const int r = idx / 15, v = idx - r * 15;
        uint4 x = make_uint4(0u, 0u, 0u, 0u);
        const int pr = yrow[r];
        if (pr >= 0) x = __ldg(reinterpret_cast<const uint4 *>(p.planes + (long long)pr * p.plane_bytes + boff) + v);
        uint32_t *d = Ys + r * kLd + 4 * v;
        d[0] = x.x; d[1] = x.y; d[2] = x.z; d[3] = x.w;
      }
      __syncthreads();
#pragma unroll 4
      for (int w = 0; w < kBlockWords; ++w) {
        uint32_t a[4], y[8];
#pragma unroll
        for (int i = 0; i < 4; ++i) a[i] = As[(ty * 4 + i) * kLd + w];
#pragma unroll
        for (int j = 0; j < 8; ++j) y[j] = Ys[(tx + 32 * j) * kLd + w];
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int j = 0; j < 8; ++j) c[i][j] += __popc(a[i] & y[j]);
      }
    }
    __syncthreads();
    // Counts to shared memory: cnt[row][q], pitch kBP_N + 1.
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) cnt[(ty * 4 + i) * (kBP_N + 1) + tx + 32 * j] = c[i][j];
    __syncthreads();
    // Exact At_tmp per (SNP, Wn row of the chunk): 256 threads over 32 x CW.
    for (int e = tid; e < kBP_M * CW; e += kBP_T) {
      const int r = e / CW, mwl = e % CW;
      double s = 0.0;
      if (mw0 + mwl < p.nW) {
        long long v = 0;
        for (int k = 0; k < p.B; ++k) {
          const int q = mwl * p.B + k;
          const long long pm = 2ll * cnt[r * (kBP_N + 1) + q] - p.ycnt[1 + (mw0 + mwl) * p.B + k];
          v += pm * (1ll << k);
        }
        s = (double)v;
      }
      tmpd[r * CW + mwl] = s;
    }
    __syncthreads();
    if (tid < kBP_M && pair0 + tid < p.npairs) {
      const int mwend = min(CW, p.nW - mw0);
      for (int mwl = 0; mwl < mwend; ++mwl) {
        const int mw = mw0 + mwl;
        const double At_tmp = tmpd[tid * CW + mwl];
        const double at_tmp = __dmul_rn(p.T_tmp[(long long)t * p.nW + mw], aA);
        const double X = __dsub_rn(__ddiv_rn(__dadd_rn(At_base, At_tmp), p.mlt_d),
                                   __ddiv_rn(__dadd_rn(at_base, at_tmp), p.mlt_d));
        const int mwa = (int)p.mw_a[mw];
        const int vZ = ((p.Zt[z_off + (mwa >> 3)] >> (7 - (mwa & 7))) & 1) ? 1 : -1;
        const double vS = (double)p.vS[(long long)t * p.nW + mw];
        acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(X, vS), __dsub_rn((double)vZ, aZ)));
      }
    }
    __syncthreads();
  }
  if (tid < kBP_M && pair0 + tid < p.npairs) p.out[p.out_off[pair0 + tid] + p.t_off[t]] = acc;
}

// An_ZtSn_ww (dir_c/An_ZtSn_ww.c:5-108).  With pm0(a, y) = 2 pos - all,
// pos = popcount(a & y & mask) and all = popcount(y & mask) over the whole
// row, each output is
//   (pm0(a, plane 0) * min * mlt + sum_{mx = B..1} 2^(B-mx) pm0(a, plane(s, mx))) / mlt
// in that order.  The pos counts of every (row, plane) pair are one
// masked-AND Gram of the An rows against the plane rows (launch_gram with
// unit block weights: its FP64 sums of integer block counts are exact), the
// all counts one warp per plane, and the FP64 combination a thread per
// (row, s).
struct AnZtSnFinish {
  const double *pos;              // n x nplanes, pos[i + k*n]
  const long long *all;           // per plane
  int n, nS, ncols_per;
  double min_d, mlt_d;
  const unsigned long long *out_r; const unsigned long long *s_off;
  double *out;
};

__global__ void plane_counts_kernel(const uint8_t *planes, long long plane_bytes, const uint8_t *mask, int nwords,
                                    int nplanes, long long *all) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= nplanes) return;
  const uint32_t *y = reinterpret_cast<const uint32_t *>(planes + (long long)warp * plane_bytes);
  const uint32_t *m = reinterpret_cast<const uint32_t *>(mask);
  int c = 0;
  for (int i = lane; i < nwords; i += 32) c += __popc(__ldg(y + i) & __ldg(m + i));
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if (lane == 0) all[warp] = c;
}

__global__ void an_ztsn_finish_kernel(AnZtSnFinish p) {
  const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (t >= (long long)p.n * p.nS) return;
  const int i = (int)(t % p.n), s = (int)(t / p.n);
  auto pm0 = [&](int k) { return 2ll * (long long)p.pos[i + (long long)k * p.n] - p.all[k]; };
  const double base = __dmul_rn(__dmul_rn((double)pm0(0), p.min_d), p.mlt_d);
  double tmp = 0.0, n2 = 1.0;
  for (int mx = p.ncols_per - 1; mx > 0; --mx) {
    tmp = __dadd_rn(tmp, __dmul_rn(n2, (double)pm0(p.ncols_per * s + mx)));
    n2 *= 2.0;
  }
  p.out[p.out_r[i] + p.s_off[s]] = __ddiv_rn(__dadd_rn(base, tmp), p.mlt_d);
}

inline unsigned long long pick_u(int s, unsigned long long j, unsigned long long b, unsigned long long a) {
  return s == LAKGB_SPACING_j ? j : (s == LAKGB_SPACING_b ? b : a);
}

// An_ZtSWn_Yt_ww (dir_c/An_ZtSWn_Yt_ww.c:5-111).  For St row s the planes of
// one xcalc'd ZtSWn slice (B value planes per Wt row after the mask plane);
// with pm0_lf(x, y; D) = sum over 1920-bit blocks, in order, of
// D[block] * pm0_block(x, y) (popcount_pm0_lf, dir_c/popcount.c:556-621):
//   X(a, w) = (pm0_lf(An_a, p0; D01)*min*mlt + sum_k 2^k pm0_lf(An_a, plane(w, k); D01)) / mlt
//           - (pm0_lf(p0, p0; D11)*min*mlt + sum_k 2^k pm0_lf(p0, plane(w, k); D11)) / mlt
//   out[a, s] = sum over w in order of X(a, w) * D_Y[w] * (vY(a, w) - a_Y[w]).
// Kernels: the pm0_lf terms of p0 and of each An row against p0 (warp per
// value); then one CTA per (32 paired rows, 256/B Wt rows, s) stages per block
// the 32 An rows and its 256 masked plane rows in shared memory, each thread
// folds its 4 x 8 tile of block counts into FP64 sums with the block's D (no
// FMA), as the reference does per plane row, and the CTA writes X for its
// rows and Wt rows to a scratch array; a last kernel adds the X terms of each
// (row, s) in Wt order onto the output.  Wt rows are taken in ranges sized so
// the scratch stays bounded, the output carrying the running sums between ranges.
struct AnZtSWnParams {
  const uint8_t *An; const uint32_t *a_rowb; long long a_row_bytes; int n;
  const uint8_t *Yn; const uint32_t *y_rowb; long long y_row_bytes;
  const uint8_t *mask; int P;
  const uint8_t *const *planes; long long plane_bytes; const double *min_d, *mlt_d;
  int nS, ncols_per, B, nW;
  const double *D01, *D11;
  const uint32_t *w_a; const double *wD, *wa;
  const double *base_, *t_, *baseA;
  double *X; int w_lo, w_hi;  // scratch X[(s*(w_hi-w_lo) + w - w_lo)*n + row] for Wt rows [w_lo, w_hi)
  const unsigned long long *out_r, *s_off;
  double *out;
};

__device__ __forceinline__ double pm0_lf_warp(const uint32_t *x, const uint32_t *y, const uint32_t *m,
                                              const double *D, int P, int lane) {
  double acc = 0.0;
  for (int blk = 0; blk < P; ++blk) {
    int pos = 0, all = 0;
    for (int i = lane; i < kBlockWords; i += 32) {
      const int w = blk * kBlockWords + i;
      const uint32_t ym = __ldg(y + w) & __ldg(m + w);
      pos += __popc(__ldg(x + w) & ym);
      all += __popc(ym);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      pos += __shfl_xor_sync(0xffffffffu, pos, o);
      all += __shfl_xor_sync(0xffffffffu, all, o);
    }
    acc = __dadd_rn(acc, __dmul_rn(__ldg(D + blk), (double)(2 * pos - all)));
  }
  return acc;
}

// Warps [0, nS*nq): dq[s][q] = pm0_lf(p0, y_q; D11), y_0 = p0 and
// y_{1 + w*B + k} = plane(w, k).  Warps [nS*nq, nS*(nq + n)):
// baseA[s][r] = pm0_lf(An_r, p0; D01) * min * mlt.
__global__ void an_ztswn_prep_kernel(AnZtSWnParams p, double *dq, double *baseA) {
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const long long nq = 1 + (long long)p.nW * p.B;
  const uint32_t *m = reinterpret_cast<const uint32_t *>(p.mask);
  if (warp < nq * p.nS) {
    const int s = (int)(warp / nq), q = (int)(warp % nq);
    const uint8_t *pl = p.planes[s];
    const int prow = q == 0 ? 0 : plane_row((q - 1) / p.B, (q - 1) % p.B, p.ncols_per);
    const double v = pm0_lf_warp(reinterpret_cast<const uint32_t *>(pl),
                                 reinterpret_cast<const uint32_t *>(pl + (long long)prow * p.plane_bytes), m,
                                 p.D11, p.P, lane);
    if (lane == 0) dq[warp] = v;
    return;
  }
  const long long e = warp - nq * p.nS;
  if (e >= (long long)p.nS * p.n) return;
  const int s = (int)(e / p.n), r = (int)(e % p.n);
  const double v = pm0_lf_warp(reinterpret_cast<const uint32_t *>(p.An + (long long)p.a_rowb[r] * p.a_row_bytes),
                               reinterpret_cast<const uint32_t *>(p.planes[s]), m, p.D01, p.P, lane);
  if (lane == 0) baseA[e] = __dmul_rn(__dmul_rn(v, p.min_d[s]), p.mlt_d[s]);
}

// base_[s] = dq[s][0]*min*mlt;  t_[s][w] = sum_k 2^k dq[s][1 + w*B + k], k upward.
__global__ void an_ztswn_tsum_kernel(AnZtSWnParams p, const double *dq, double *base_, double *t_) {
  const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (idx >= (long long)p.nS * (p.nW + 1)) return;
  const int s = (int)(idx / (p.nW + 1)), w = (int)(idx % (p.nW + 1)) - 1;
  const double *row = dq + (long long)s * (1 + (long long)p.nW * p.B);
  if (w < 0) {
    base_[s] = __dmul_rn(__dmul_rn(row[0], p.min_d[s]), p.mlt_d[s]);
    return;
  }
  double t = 0.0, n2 = 1.0;
  for (int k = 0; k < p.B; ++k) {
    t = __dadd_rn(t, __dmul_rn(n2, row[1 + (long long)w * p.B + k]));
    n2 *= 2.0;
  }
  t_[(long long)s * p.nW + w] = t;
}

// Two CTAs per SM (128 registers, a 32-byte spill): 1.5x the throughput of
// one CTA per SM with 243 registers on 2048 x 16384 x (1024 x 33 planes).
__global__ void __launch_bounds__(kBP_T, 2)
an_ztswn_ww_kernel(AnZtSWnParams p) {
  // Dynamic shared memory, two phases: As (kBP_M x kLd words) and Ys (kBP_N x
  // kLd words) during the block loop; then dv (kBP_M x (kBP_N+1) doubles, the
  // per-plane sums) over the same bytes.
  extern __shared__ __align__(16) uint32_t smem[];
  uint32_t *As = smem;
  uint32_t *Ys = smem + kBP_M * kLd;
  double *dv = reinterpret_cast<double *>(smem);
  __shared__ long long a_off[kBP_M];
  __shared__ int yrow[kBP_N];
  __shared__ int ycs[kBP_N];

  const int CW = kBP_N / p.B;  // Wt rows per CTA
  const int s = blockIdx.z;
  const int r0 = blockIdx.x * kBP_M;
  const int w0 = p.w_lo + blockIdx.y * CW;
  const int tid = threadIdx.x;
  const int tx = tid & 31, ty = tid >> 5;
  const uint8_t *pl = p.planes[s];
  const double mlt = p.mlt_d[s];

  for (int i = tid; i < kBP_M; i += kBP_T)
    a_off[i] = (r0 + i < p.n) ? (long long)p.a_rowb[r0 + i] * p.a_row_bytes : -1;
  for (int q = tid; q < kBP_N; q += kBP_T) {
    const int wl = q / p.B, k = q % p.B;
    yrow[q] = (q < CW * p.B && w0 + wl < p.w_hi) ? plane_row(w0 + wl, k, p.ncols_per) : -1;
  }
  double acc[4][8];
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) acc[i][j] = 0.0;

  for (int blk = 0; blk < p.P; ++blk) {
    __syncthreads();
    const long long boff = (long long)blk * kBlockBytes;
    const uint4 *mk = reinterpret_cast<const uint4 *>(p.mask + boff);
    for (int idx = tid; idx < kBP_M * 15; idx += kBP_T) {
      const int r = idx / 15, v = idx - r * 15;
      uint4 x = make_uint4(0u, 0u, 0u, 0u);
      if (a_off[r] >= 0) x = __ldg(reinterpret_cast<const uint4 *>(p.An + a_off[r] + boff) + v);
      uint32_t *d = As + r * kLd + 4 * v;
      d[0] = x.x; d[1] = x.y; d[2] = x.z; d[3] = x.w;
    }
    for (int idx = tid; idx < kBP_N * 15; idx += kBP_T) {
      const int r = idx / 15, v = idx - r * 15;
      uint4 x = make_uint4(0u, 0u, 0u, 0u);
      const int pr = yrow[r];
      if (pr >= 0) {
        const uint4 y = __ldg(reinterpret_cast<const uint4 *>(pl + (long long)pr * p.plane_bytes + boff) + v);
        const uint4 m = __ldg(mk + v);
        x.x = y.x & m.x; x.y = y.y & m.y; x.z = y.z & m.z; x.w = y.w & m.w;
      }
      uint32_t *d = Ys + r * kLd + 4 * v;
      d[0] = x.x; d[1] = x.y; d[2] = x.z; d[3] = x.w;
    }
    __syncthreads();
    {
      int c = 0;
      for (int w = 0; w < kBlockWords; ++w) c += __popc(Ys[tid * kLd + w]);
      ycs[tid] = c;
    }
    int c[4][8];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j) c[i][j] = 0;
#pragma unroll 4
    for (int w = 0; w < kBlockWords; ++w) {
      uint32_t a[4], y[8];
#pragma unroll
      for (int i = 0; i < 4; ++i) a[i] = As[(ty * 4 + i) * kLd + w];
#pragma unroll
      for (int j = 0; j < 8; ++j) y[j] = Ys[(tx + 32 * j) * kLd + w];
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) c[i][j] += __popc(a[i] & y[j]);
    }
    __syncthreads();
    const double D = __ldg(p.D01 + blk);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int j = 0; j < 8; ++j)
        acc[i][j] = __dadd_rn(acc[i][j], __dmul_rn(D, (double)(2 * c[i][j] - ycs[tx + 32 * j])));
  }
  __syncthreads();
#pragma unroll
  for (int i = 0; i < 4; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j) dv[(ty * 4 + i) * (kBP_N + 1) + tx + 32 * j] = acc[i][j];
  __syncthreads();
  // X for (row, Wt row): consecutive threads take consecutive rows, so the
  // scratch writes (rows contiguous per Wt row) coalesce.
  const double base_ = p.base_[s];
  const long long wspan = p.w_hi - p.w_lo;
  for (int e = tid; e < kBP_M * CW; e += kBP_T) {
    const int r = e % kBP_M, wl = e / kBP_M;
    const int w = w0 + wl;
    if (w >= p.w_hi || r0 + r >= p.n) continue;
    double t = 0.0, n2 = 1.0;
    for (int k = 0; k < p.B; ++k) {
      t = __dadd_rn(t, __dmul_rn(n2, dv[r * (kBP_N + 1) + wl * p.B + k]));
      n2 *= 2.0;
    }
    const double X = __dsub_rn(__ddiv_rn(__dadd_rn(p.baseA[(long long)s * p.n + r0 + r], t), mlt),
                               __ddiv_rn(__dadd_rn(base_, p.t_[(long long)s * p.nW + w]), mlt));
    p.X[((long long)s * wspan + (w - p.w_lo)) * p.n + r0 + r] = X;
  }
}

// out[row, s] += X(row, w) * D_Y[w] * (vY(row, w) - a_Y[w]) for w in [w_lo, w_hi), in order.
__global__ void an_ztswn_sum_kernel(AnZtSWnParams p) {
  const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= (long long)p.nS * p.n) return;
  const int s = (int)(e / p.n), r = (int)(e % p.n);
  const long long y_off = (long long)p.y_rowb[r] * p.y_row_bytes;
  double *o = p.out + p.out_r[r] + p.s_off[s];
  double acc = *o;
  const long long wspan = p.w_hi - p.w_lo;
  const double *x = p.X + (long long)s * wspan * p.n + r;
  for (int w = p.w_lo; w < p.w_hi; ++w) {
    const uint32_t wa = p.w_a[w];
    const int vY = ((p.Yn[y_off + (wa >> 3)] >> (7 - (wa & 7))) & 1) ? 1 : -1;
    acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(x[(long long)(w - p.w_lo) * p.n], p.wD[w]), __dsub_rn((double)vY, p.wa[w])));
  }
  *o = acc;
}

constexpr size_t kAnZtSWnSmem = std::max((size_t)(kBP_M + kBP_N) * kLd * sizeof(uint32_t),
                                          (size_t)kBP_M * (kBP_N + 1) * sizeof(double));
constexpr size_t kAnZtSWnScratch = 256ull << 20;  // bytes of X scratch per range of Wt rows

}  // namespace

}  // namespace lakgb

using namespace lakgb;

namespace lakgb {
std::atomic<int> g_bitplane_impl{LAKGB_IMPL_TENSOR};
}

extern "C" void lakgb_set_bitplane_impl(int impl) {
  g_bitplane_impl.store(impl == LAKGB_IMPL_POPCOUNT ? LAKGB_IMPL_POPCOUNT : LAKGB_IMPL_TENSOR);
}

extern "C" int lakgb_bitplane_impl(void) { return g_bitplane_impl.load(); }

namespace lakgb {
namespace {

// Bit-plane products held back by a deferral scope (tensor-core path): the
// prep kernels of each call run when it is made; the main kernels of all
// calls with the same B run as one grouped launch when the scope ends.
struct BitplaneDeferred {
  BitplaneParams p{};
  int nT = 0;
  std::vector<DBuf> keep;
  double *host_out = nullptr;
  unsigned long long length = 0;
};
thread_local std::vector<BitplaneDeferred> t_bp;
thread_local std::vector<DBuf> t_bp_groups;

void bitplane_deferred_enqueue() {
  for (int B : {8, 16, 32}) {
    std::vector<BitplaneParams> ps;
    std::vector<int> tile0;
    int tiles = 0;
    for (const auto &d : t_bp)
      if (d.p.B == B) {
        ps.push_back(d.p);
        tile0.push_back(tiles);
        tiles += bitplane_tc_tiles(d.p, d.nT);
      }
    if (ps.empty()) continue;
    t_bp_groups.push_back(defer_upload(ps));
    t_bp_groups.push_back(defer_upload(tile0));
    defer_flush();
    launch_bitplane_tc_group(B, t_bp_groups[t_bp_groups.size() - 2].as<BitplaneParams>(),
                             t_bp_groups.back().as<int>(), (int)ps.size(), tiles, stream());
  }
  for (const auto &d : t_bp)
    if (d.length)
      LAKGB_CUDA(cudaMemcpyAsync(d.host_out, d.p.out, d.length * sizeof(double), cudaMemcpyDeviceToHost, stream()));
}

void bitplane_deferred_clear() {
  t_bp.clear();
  t_bp_groups.clear();
}

}  // namespace
}  // namespace lakgb

extern "C" int wrap_At_T_YnWt_S_Zn_ww__run(int *tidx, void **vpra, pthread_t *thread_in, int spacing_a,
                                           int spacing_t, M_handle *M_At, M_handle *M_Tt, M_handle *M_Yn,
                                           M_handle *M_Wn, M_handle *M_St, M_handle *M_Zt, double *A_ajdk,
                                           M_handle *M_YnWt, L_handle **output_p) {
  LAKGB_PROFILE_CALL("wrap_At_T_YnWt_S_Zn_ww__run");
  (void)tidx; (void)vpra; (void)thread_in; (void)M_Yn;
  const unsigned long long length_a = spacing_length(spacing_a, M_At);
  const unsigned long long length_t = spacing_length(spacing_t, M_Tt);
  const unsigned long long length = length_a * length_t;
  L_handle *out = ensure_output(output_p, length, "wrap_At_T_YnWt_S_Zn_ww__run");
  if (!out) return (int)length;
  out->spacing_row = spacing_a; out->row_stride = length_a;
  out->spacing_col = spacing_t; out->col_stride = length_t;
  const int nT = (int)std::min(M_Tt->rpop_j, M_St->rpop_j);
  const int npairs = (int)std::min(M_At->rpop_j, M_Zt->rpop_j);
  const int nW = (int)M_Wn->rpop_j;
  const int ncols_per = M_YnWt->ncols_per_z, B = ncols_per - 1;
  if (nT == 0 || npairs == 0) return (int)length;
  if (B < 1 || B > 62 || M_YnWt->mc_length != M_At->mc_length || M_Tt->mc_length != M_At->mc_length) {
    set_error(4, "wrap_At_T_YnWt_S_Zn_ww__run: planes / rows of unequal length or B_MLT out of range");
    return (int)length;
  }
  if (nW == 0) return (int)length;  // every output is an empty sum
  if ((long long)nW * ncols_per > M_YnWt->nrows || (long long)M_Zt->mc_length * 8 < M_Wn->nrows ||
      (long long)M_St->mc_length * 8 < M_Wn->nrows) {
    set_error(4, "wrap_At_T_YnWt_S_Zn_ww__run: planes / masks do not cover the Wn rows");
    return (int)length;
  }
  const int P = (int)(M_At->mc_length / kBlockBytes);
  const int A_pcols = (int)lakbcc::psize(M_At->nrows);
  const double *a_An = A_ajdk + (size_t)lakbcc::AJDK_1_0 * A_pcols;

  std::vector<uint32_t> at_rowb(npairs), zt_rowb(npairs), tt_rowb(nT), mw_a(nW);
  std::vector<double> aA(npairs), aZ(npairs);
  std::vector<unsigned long long> out_off(npairs), t_off(nT);
  for (int i = 0; i < npairs; ++i) {
    at_rowb[i] = M_At->m_b_[i]; zt_rowb[i] = M_Zt->m_b_[i];
    aA[i] = a_An[M_At->m_a_[i] / lakbcc::POPLENGTH];
    aZ[i] = a_An[M_Zt->m_a_[i] / lakbcc::POPLENGTH];
    out_off[i] = pick_u(spacing_a, i, M_At->m_b_[i], M_At->m_a_[i]);
  }
  std::vector<int8_t> vS((size_t)nT * nW);
  for (int t = 0; t < nT; ++t) {
    tt_rowb[t] = M_Tt->m_b_[t];
    t_off[t] = pick_u(spacing_t, t, M_Tt->m_b_[t], M_Tt->m_a_[t]) * length_a;
    const unsigned char *st = M_St->wX + (size_t)M_St->m_b_[t] * M_St->mc_length;
    for (int mw = 0; mw < nW; ++mw) vS[(size_t)t * nW + mw] = (int8_t)lakbcc::bget_pm(st, M_Wn->m_a_[mw]);
  }
  for (int mw = 0; mw < nW; ++mw) mw_a[mw] = M_Wn->m_a_[mw];

  // Inside a deferral scope the tensor-core main kernel waits for the scope's
  // end (its uploads are then owned buffers, not staging views).  Only with
  // residency on: the matrices' device copies must stay where they are until
  // the scope ends, which an upload of the same host buffer without residency
  // would not guarantee.
  const bool defer = defer_active() && residency_enabled() &&
                     g_bitplane_impl.load(std::memory_order_relaxed) == LAKGB_IMPL_TENSOR &&
                     (B == 8 || B == 16 || B == 32);
  BitplaneParams p{};
  std::optional<Stager> st;
  if (!defer) st.emplace();
  p.At = (const uint8_t *)resident(M_At->wX, (size_t)M_At->rpop_b * M_At->mc_length);
  p.at_row_bytes = (long long)M_At->mc_length;
  p.Tt = (const uint8_t *)resident(M_Tt->wX, (size_t)M_Tt->rpop_b * M_Tt->mc_length);
  p.tt_row_bytes = (long long)M_Tt->mc_length;
  p.planes = (const uint8_t *)resident(M_YnWt->wX, (size_t)M_YnWt->nrows * M_YnWt->mc_length);
  p.plane_bytes = (long long)M_YnWt->mc_length;
  p.Zt = (const uint8_t *)resident(M_Zt->wX, (size_t)M_Zt->rpop_b * M_Zt->mc_length);
  p.zt_row_bytes = (long long)M_Zt->mc_length;
  // a held-back call's small inputs go through the scope's page-locked chunks
  auto up = [&](const auto &v) { return defer ? defer_upload(v) : upload_vec(v); };
  DBuf mask = defer ? DBuf::view(defer_put(M_At->mc_j, M_At->mc_length), M_At->mc_length)
                    : upload_bytes(M_At->mc_j, M_At->mc_length);
  p.mask = mask.as<uint8_t>(); p.P = P; p.npairs = npairs;
  DBuf d_at = up(at_rowb), d_zt = up(zt_rowb), d_tt = up(tt_rowb), d_mw = up(mw_a);
  DBuf d_vS = up(vS), d_aA = up(aA), d_aZ = up(aZ);
  DBuf d_oo = up(out_off), d_to = up(t_off);
  if (defer) defer_flush();
  p.at_rowb = d_at.as<uint32_t>(); p.zt_rowb = d_zt.as<uint32_t>(); p.tt_rowb = d_tt.as<uint32_t>();
  p.mw_a = d_mw.as<uint32_t>(); p.nW = nW; p.B = B; p.ncols_per = ncols_per;
  p.vS = d_vS.as<int8_t>(); p.aA = d_aA.as<double>(); p.aZ = d_aZ.as<double>();
  p.min_d = M_YnWt->min_d; p.mlt_d = M_YnWt->mlt_d;
  p.out_off = d_oo.as<unsigned long long>(); p.t_off = d_to.as<unsigned long long>();

  const int nq = 1 + nW * B;
  DBuf d_pm((size_t)nT * nq * sizeof(int)), d_ycnt((size_t)nq * sizeof(int));
  DBuf d_Tb((size_t)nT * sizeof(double)), d_Tt((size_t)nT * nW * sizeof(double));
  {
    const long long warps = (long long)nq * nT;
    if (st) st->flush();
    bitplane_prep_kernel<<<(int)((warps * 32 + 255) / 256), 256, 0, stream()>>>(p, nT, d_pm.as<int>(), d_ycnt.as<int>());
    LAKGB_CUDA(cudaGetLastError());
    const int n = nT * (nW + 1);
    bitplane_tsum_kernel<<<(n + 255) / 256, 256, 0, stream()>>>(p, nT, d_pm.as<int>(), d_Tb.as<double>(), d_Tt.as<double>());
    LAKGB_CUDA(cudaGetLastError());
    count_launch(2);
  }
  p.ycnt = d_ycnt.as<int>(); p.T_base = d_Tb.as<double>(); p.T_tmp = d_Tt.as<double>();
  DBuf d_out(length * sizeof(double));
  d_out.zero();
  p.out = d_out.as<double>();
  if (defer) {
    BitplaneDeferred d;
    d.p = p;
    d.nT = nT;
    d.host_out = out->lf;
    d.length = length;
    for (DBuf *b : {&mask, &d_at, &d_zt, &d_tt, &d_mw, &d_vS, &d_aA, &d_aZ, &d_oo, &d_to, &d_pm, &d_ycnt, &d_Tb, &d_Tt,
                    &d_out})
      d.keep.push_back(std::move(*b));
    t_bp.push_back(std::move(d));
    defer_register(bitplane_deferred_enqueue, bitplane_deferred_clear);
    return (int)length;
  }
  const size_t smem = std::max((size_t)(kBP_M + kBP_N) * kLd * sizeof(uint32_t),
                               (size_t)kBP_M * (kBP_N + 1) * sizeof(int) + (size_t)kBP_M * kBP_N * sizeof(double));
  static std::once_flag attr;
  std::call_once(attr, [&] {
    LAKGB_CUDA(cudaFuncSetAttribute(bitplane_main_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  });
  if (g_bitplane_impl.load(std::memory_order_relaxed) == LAKGB_IMPL_TENSOR && (B == 8 || B == 16 || B == 32)) {
    launch_bitplane_tc(p, nT, stream());
  } else {
    dim3 grid((npairs + kBP_M - 1) / kBP_M, nT);
    bitplane_main_kernel<<<grid, kBP_T, smem, stream()>>>(p);
    LAKGB_CUDA(cudaGetLastError());
    count_launch();
  }
  copy_back(out->lf, d_out, length);
  return (int)length;
}

extern "C" int wrap_An_ZtSn_ww__run(int *tidx, void **vpra, pthread_t *thread_in, int spacing_a, int spacing_s,
                                    M_handle *M_An, L_handle *lf_ZtSn, M_handle *M_ZtSn, M_handle *M_St,
                                    L_handle **output_p) {
  LAKGB_PROFILE_CALL("wrap_An_ZtSn_ww__run");
  (void)tidx; (void)vpra; (void)thread_in; (void)lf_ZtSn;
  const unsigned long long length_a = spacing_length(spacing_a, M_An);
  const unsigned long long length_s = spacing_length(spacing_s, M_St);
  const unsigned long long length = length_a * length_s;
  L_handle *out = ensure_output(output_p, length, "wrap_An_ZtSn_ww__run");
  if (!out) return (int)length;
  out->spacing_row = spacing_a; out->row_stride = length_a;
  out->spacing_col = spacing_s; out->col_stride = length_s;
  const int n = (int)M_An->rpop_j, nS = (int)M_St->rpop_j;
  if (n == 0 || nS == 0) return (int)length;
  if (M_ZtSn->mc_length != M_An->mc_length || (long long)nS * M_ZtSn->ncols_per_z > M_ZtSn->nrows) {
    set_error(4, "wrap_An_ZtSn_ww__run: planes and rows of unequal length");
    return (int)length;
  }
  std::vector<uint32_t> rowb(M_An->m_b_, M_An->m_b_ + n);
  std::vector<unsigned long long> out_r(n), s_off(nS);
  for (int i = 0; i < n; ++i) out_r[i] = pick_u(spacing_a, i, M_An->m_b_[i], M_An->m_a_[i]);
  for (int s = 0; s < nS; ++s) s_off[s] = pick_u(spacing_s, s, M_St->m_b_[s], M_St->m_a_[s]) * length_a;
  const int nplanes = nS * M_ZtSn->ncols_per_z;
  Stager st;
  const uint8_t *An = (const uint8_t *)resident(M_An->wX, (size_t)M_An->rpop_b * M_An->mc_length);
  const uint8_t *planes = (const uint8_t *)resident(M_ZtSn->wX, (size_t)M_ZtSn->nrows * M_ZtSn->mc_length);
  std::vector<uint32_t> zrow(nplanes), orow(n), ocol(nplanes);
  for (int k = 0; k < nplanes; ++k) zrow[k] = ocol[k] = (uint32_t)k;
  for (int i = 0; i < n; ++i) orow[i] = (uint32_t)i;
  DBuf d_rowb = upload_vec(rowb), d_or = upload_vec(out_r), d_so = upload_vec(s_off);
  DBuf d_zrow = upload_vec(zrow), d_orow = upload_vec(orow), d_ocol = upload_vec(ocol);
  DBuf mask = upload_bytes(M_An->mc_j, M_An->mc_length);
  DBuf d_pos((size_t)n * nplanes * sizeof(double)), d_all((size_t)nplanes * sizeof(long long));
  DBuf d_out(length * sizeof(double));
  d_out.zero();
  st.flush();
  GramParams g{};
  g.wA = An; g.a_rowb = d_rowb.as<uint32_t>(); g.nA = n; g.a_row_bytes = (long long)M_An->mc_length;
  g.wZ = planes; g.z_rowb = d_zrow.as<uint32_t>(); g.nZ = nplanes; g.z_row_bytes = (long long)M_ZtSn->mc_length;
  g.mask = mask.as<uint8_t>(); g.P = (int)(M_An->mc_length / kBlockBytes);
  g.D = nullptr; g.type = 2;  // masked AND counts
  g.out_r = d_orow.as<uint32_t>(); g.out_c = d_ocol.as<uint32_t>(); g.out_stride = n; g.out = d_pos.as<double>();
  launch_gram(g);
  const int nwords = (int)(M_An->mc_length / 4);
  plane_counts_kernel<<<(nplanes * 32 + 255) / 256, 256, 0, stream()>>>(planes, (long long)M_ZtSn->mc_length,
                                                                     mask.as<uint8_t>(), nwords, nplanes,
                                                                     d_all.as<long long>());
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
  AnZtSnFinish p{};
  p.pos = d_pos.as<double>(); p.all = d_all.as<long long>();
  p.n = n; p.nS = nS; p.ncols_per = M_ZtSn->ncols_per_z;
  p.min_d = M_ZtSn->min_d; p.mlt_d = M_ZtSn->mlt_d;
  p.out_r = d_or.as<unsigned long long>(); p.s_off = d_so.as<unsigned long long>();
  p.out = d_out.as<double>();
  an_ztsn_finish_kernel<<<(unsigned)(((long long)n * nS + 255) / 256), 256, 0, stream()>>>(p);
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
  copy_back(out->lf, d_out, length);
  return (int)length;
}

extern "C" int wrap_An_ZtSWn_Yt_ww__run(int *tidx, void **vpra, pthread_t *thread_in, int spacing_a, int spacing_s,
                                        M_handle *M_An, M_handle *M_St, M_handle **M_ZtSWn_, M_handle *M_Wt,
                                        M_handle *M_Yn, double *A_ajdk, double *Y_ajdk, L_handle **output_p) {
  LAKGB_PROFILE_CALL("wrap_An_ZtSWn_Yt_ww__run");
  (void)tidx; (void)vpra; (void)thread_in;
  const unsigned long long length_a = spacing_length(spacing_a, M_An);
  const unsigned long long length_s = spacing_length(spacing_s, M_St);
  const unsigned long long length = length_a * length_s;
  L_handle *out = ensure_output(output_p, length, "wrap_An_ZtSWn_Yt_ww__run");
  if (!out) return (int)length;
  out->spacing_row = spacing_a; out->row_stride = length_a;
  out->spacing_col = spacing_s; out->col_stride = length_s;
  const int nS = (int)M_St->rpop_j;
  const int n = (int)std::min(M_An->rpop_j, M_Yn->rpop_j);
  const int nW = (int)M_Wt->rpop_j;
  if (nS == 0 || n == 0 || nW == 0) return (int)length;  // empty sums: the zeros ensure_output wrote
  if (!M_ZtSWn_ || !A_ajdk || !Y_ajdk) {
    set_error(4, "wrap_An_ZtSWn_Yt_ww__run: planes or allele weights missing");
    return (int)length;
  }
  const int ncols_per = M_ZtSWn_[0] ? M_ZtSWn_[0]->ncols_per_z : 0, B = ncols_per - 1;
  for (int s = 0; s < nS; ++s) {
    const M_handle *Z = M_ZtSWn_[s];
    if (!Z || Z->ncols_per_z != ncols_per || B < 1 || B > 62 || Z->mc_length != M_An->mc_length ||
        (long long)nW * ncols_per > Z->nrows) {
      set_error(4, "wrap_An_ZtSWn_Yt_ww__run: planes of St row %d missing, of unequal length or B_MLT out of range", s);
      return (int)length;
    }
  }
  if ((long long)M_Yn->mc_length * 8 < M_Wt->nrows) {
    set_error(4, "wrap_An_ZtSWn_Yt_ww__run: Yn rows shorter than the Wt rows they index");
    return (int)length;
  }
  const int P = (int)(M_An->mc_length / kBlockBytes);
  const int A_pcols = (int)lakbcc::psize(M_An->ncols), Y_pcols = (int)lakbcc::psize(M_Yn->ncols);
  const double *D01 = A_ajdk + (size_t)lakbcc::AJDK_0_1 * A_pcols;
  const double *D11 = A_ajdk + (size_t)lakbcc::AJDK_1_1 * A_pcols;
  const double *D_Yn = Y_ajdk + (size_t)lakbcc::AJDK_0_1 * Y_pcols;
  const double *a_Yn = Y_ajdk + (size_t)lakbcc::AJDK_1_0 * Y_pcols;

  std::vector<uint32_t> a_rowb(n), y_rowb(n), w_a(nW);
  std::vector<unsigned long long> out_r(n), s_off(nS);
  std::vector<double> wD(nW), wa(nW), mins(nS), mlts(nS);
  std::vector<double> d01(D01, D01 + P), d11(D11, D11 + P);
  for (int i = 0; i < n; ++i) {
    a_rowb[i] = M_An->m_b_[i]; y_rowb[i] = M_Yn->m_b_[i];
    out_r[i] = pick_u(spacing_a, i, M_An->m_b_[i], M_An->m_a_[i]);
  }
  for (int w = 0; w < nW; ++w) {
    w_a[w] = M_Wt->m_a_[w];
    wD[w] = D_Yn[w_a[w] / lakbcc::POPLENGTH];
    wa[w] = a_Yn[w_a[w] / lakbcc::POPLENGTH];
  }
  AnZtSWnParams p{};
  Stager st;
  std::vector<const uint8_t *> planes(nS);
  for (int s = 0; s < nS; ++s) {
    s_off[s] = pick_u(spacing_s, s, M_St->m_b_[s], M_St->m_a_[s]) * length_a;
    const M_handle *Z = M_ZtSWn_[s];
    planes[s] = (const uint8_t *)resident(Z->wX, (size_t)Z->nrows * Z->mc_length);
    mins[s] = Z->min_d; mlts[s] = Z->mlt_d;
  }
  p.An = (const uint8_t *)resident(M_An->wX, (size_t)M_An->rpop_b * M_An->mc_length);
  p.a_row_bytes = (long long)M_An->mc_length; p.n = n;
  p.Yn = (const uint8_t *)resident(M_Yn->wX, (size_t)M_Yn->rpop_b * M_Yn->mc_length);
  p.y_row_bytes = (long long)M_Yn->mc_length;
  DBuf mask = upload_bytes(M_An->mc_j, M_An->mc_length);
  p.mask = mask.as<uint8_t>(); p.P = P;
  DBuf d_pl = upload_vec(planes), d_min = upload_vec(mins), d_mlt = upload_vec(mlts);
  p.planes = d_pl.as<const uint8_t *const>(); p.plane_bytes = (long long)M_An->mc_length;
  p.min_d = d_min.as<double>(); p.mlt_d = d_mlt.as<double>();
  p.nS = nS; p.ncols_per = ncols_per; p.B = B; p.nW = nW;
  DBuf d_d01 = upload_vec(d01), d_d11 = upload_vec(d11);
  p.D01 = d_d01.as<double>(); p.D11 = d_d11.as<double>();
  DBuf d_ar = upload_vec(a_rowb), d_yr = upload_vec(y_rowb), d_wa = upload_vec(w_a);
  DBuf d_wD = upload_vec(wD), d_wal = upload_vec(wa), d_or = upload_vec(out_r), d_so = upload_vec(s_off);
  p.a_rowb = d_ar.as<uint32_t>(); p.y_rowb = d_yr.as<uint32_t>(); p.w_a = d_wa.as<uint32_t>();
  p.wD = d_wD.as<double>(); p.wa = d_wal.as<double>();
  p.out_r = d_or.as<unsigned long long>(); p.s_off = d_so.as<unsigned long long>();

  const long long nq = 1 + (long long)nW * B;
  DBuf d_dq((size_t)nS * nq * sizeof(double)), d_bA((size_t)nS * n * sizeof(double));
  DBuf d_base((size_t)nS * sizeof(double)), d_t((size_t)nS * nW * sizeof(double));
  DBuf d_out(length * sizeof(double));
  d_out.zero();
  p.out = d_out.as<double>();
  st.flush();
  {
    const long long threads = (nq + n) * nS * 32;
    an_ztswn_prep_kernel<<<(unsigned)((threads + 255) / 256), 256, 0, stream()>>>(p, d_dq.as<double>(),
                                                                                d_bA.as<double>());
    LAKGB_CUDA(cudaGetLastError());
    const long long m = (long long)nS * (nW + 1);
    an_ztswn_tsum_kernel<<<(unsigned)((m + 255) / 256), 256, 0, stream()>>>(p, d_dq.as<double>(), d_base.as<double>(),
                                                                            d_t.as<double>());
    LAKGB_CUDA(cudaGetLastError());
    count_launch(2);
  }
  p.base_ = d_base.as<double>(); p.t_ = d_t.as<double>(); p.baseA = d_bA.as<double>();
  static std::once_flag attr;
  std::call_once(attr, [] {
    LAKGB_CUDA(cudaFuncSetAttribute(an_ztswn_ww_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kAnZtSWnSmem));
  });
  // Wt rows in ranges whose X scratch (rows x range x covariates doubles) fits
  // the budget, a whole number of CTA chunks each.
  const int CW = kBP_N / B;
  const long long per_w = (long long)n * nS * (long long)sizeof(double);
  const long long span = std::min<long long>(65535LL * CW,  // grid.y limit
                                             std::max<long long>(CW, (long long)(kAnZtSWnScratch / per_w) / CW * CW));
  const int wspan = (int)std::min<long long>(span, nW);
  DBuf d_X((size_t)wspan * per_w);
  p.X = d_X.as<double>();
  for (int w_lo = 0; w_lo < nW; w_lo += wspan) {
    p.w_lo = w_lo; p.w_hi = std::min(nW, w_lo + wspan);
    dim3 grid((n + kBP_M - 1) / kBP_M, (p.w_hi - w_lo + CW - 1) / CW, nS);
    an_ztswn_ww_kernel<<<grid, kBP_T, kAnZtSWnSmem, stream()>>>(p);
    LAKGB_CUDA(cudaGetLastError());
    const long long e = (long long)n * nS;
    an_ztswn_sum_kernel<<<(unsigned)((e + 255) / 256), 256, 0, stream()>>>(p);
    LAKGB_CUDA(cudaGetLastError());
    count_launch(2);
  }
  copy_back(out->lf, d_out, length);
  return (int)length;
}
