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

#include "abi_common.cuh"
#include "bcc_model.h"
#include "bitplane.cuh"

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

// An_ZtSn_ww: warp per An row.
struct AnZtSnParams {
  const uint8_t *An; const uint32_t *rowb; int n; long long row_bytes;
  const uint8_t *mask; int nwords;
  const uint8_t *planes; long long plane_bytes;
  int nS; int ncols_per;
  double min_d, mlt_d;
  const unsigned long long *out_r; const unsigned long long *s_off;
  double *out;
};

__device__ __forceinline__ long long pm0_row(const uint32_t *a, const uint32_t *y, const uint32_t *m,
                                             int nwords, int lane) {
  int pos = 0, all = 0;
  for (int i = lane; i < nwords; i += 32) {
    const uint32_t ym = __ldg(y + i) & __ldg(m + i);
    pos += __popc(__ldg(a + i) & ym);
    all += __popc(ym);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    pos += __shfl_xor_sync(0xffffffffu, pos, o);
    all += __shfl_xor_sync(0xffffffffu, all, o);
  }
  return 2ll * pos - all;
}

__global__ void an_ztsn_kernel(AnZtSnParams p) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (warp >= p.n) return;
  const uint32_t *a = reinterpret_cast<const uint32_t *>(p.An + (long long)p.rowb[warp] * p.row_bytes);
  const uint32_t *m = reinterpret_cast<const uint32_t *>(p.mask);
  const long long b0 = pm0_row(a, reinterpret_cast<const uint32_t *>(p.planes), m, p.nwords, lane);
  const double base = __dmul_rn(__dmul_rn((double)b0, p.min_d), p.mlt_d);
  for (int s = 0; s < p.nS; ++s) {
    double tmp = 0.0, n2 = 1.0;
    for (int mx = p.ncols_per - 1; mx > 0; --mx) {
      const uint32_t *y = reinterpret_cast<const uint32_t *>(p.planes + (long long)(p.ncols_per * s + mx) * p.plane_bytes);
      const long long v = pm0_row(a, y, m, p.nwords, lane);
      tmp = __dadd_rn(tmp, __dmul_rn(n2, (double)v));
      n2 *= 2.0;
    }
    if (lane == 0) p.out[p.out_r[warp] + p.s_off[s]] = __ddiv_rn(__dadd_rn(base, tmp), p.mlt_d);
  }
}

inline unsigned long long pick_u(int s, unsigned long long j, unsigned long long b, unsigned long long a) {
  return s == LAKGB_SPACING_j ? j : (s == LAKGB_SPACING_b ? b : a);
}

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

  BitplaneParams p{};
  Stager st;
  p.At = (const uint8_t *)resident(M_At->wX, (size_t)M_At->rpop_b * M_At->mc_length);
  p.at_row_bytes = (long long)M_At->mc_length;
  p.Tt = (const uint8_t *)resident(M_Tt->wX, (size_t)M_Tt->rpop_b * M_Tt->mc_length);
  p.tt_row_bytes = (long long)M_Tt->mc_length;
  p.planes = (const uint8_t *)resident(M_YnWt->wX, (size_t)M_YnWt->nrows * M_YnWt->mc_length);
  p.plane_bytes = (long long)M_YnWt->mc_length;
  p.Zt = (const uint8_t *)resident(M_Zt->wX, (size_t)M_Zt->rpop_b * M_Zt->mc_length);
  p.zt_row_bytes = (long long)M_Zt->mc_length;
  DBuf mask = upload_bytes(M_At->mc_j, M_At->mc_length);
  p.mask = mask.as<uint8_t>(); p.P = P; p.npairs = npairs;
  DBuf d_at = upload_vec(at_rowb), d_zt = upload_vec(zt_rowb), d_tt = upload_vec(tt_rowb), d_mw = upload_vec(mw_a);
  DBuf d_vS = upload_vec(vS), d_aA = upload_vec(aA), d_aZ = upload_vec(aZ);
  DBuf d_oo = upload_vec(out_off), d_to = upload_vec(t_off);
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
    st.flush();
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
  AnZtSnParams p{};
  Stager st;
  p.An = (const uint8_t *)resident(M_An->wX, (size_t)M_An->rpop_b * M_An->mc_length);
  p.row_bytes = (long long)M_An->mc_length;
  DBuf d_rowb = upload_vec(rowb), d_or = upload_vec(out_r), d_so = upload_vec(s_off);
  p.rowb = d_rowb.as<uint32_t>(); p.n = n;
  DBuf mask = upload_bytes(M_An->mc_j, M_An->mc_length);
  p.mask = mask.as<uint8_t>(); p.nwords = (int)(M_An->mc_length / 4);
  p.planes = (const uint8_t *)resident(M_ZtSn->wX, (size_t)M_ZtSn->nrows * M_ZtSn->mc_length);
  p.plane_bytes = (long long)M_ZtSn->mc_length;
  p.nS = nS; p.ncols_per = M_ZtSn->ncols_per_z;
  p.min_d = M_ZtSn->min_d; p.mlt_d = M_ZtSn->mlt_d;
  p.out_r = d_or.as<unsigned long long>(); p.s_off = d_so.as<unsigned long long>();
  DBuf d_out(length * sizeof(double));
  d_out.zero();
  p.out = d_out.as<double>();
  st.flush();
  an_ztsn_kernel<<<(n * 32 + 255) / 256, 256, 0, stream()>>>(p);
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
  copy_back(out->lf, d_out, length);
  return (int)length;
}
