// Quantisation of an FP64 matrix into bit planes: get_xcalc / wrap_xcalc
// (dir_c/xcalc.c:5-263).
//
// Given YnWt (rows: the Yn rows selected by mr_b & mr_j; columns: the Wn rows
// selected by mc_b & mc_j), the planes M_X hold, for each retained column
// nc_j, ncols_per = b_mlt + 1 rows of bits over the Yn rows (a-space):
//   plane ncols_per*nc_j + ncols_per-1-nb = bit nb of
//       cz = crop((unsigned long long)(mlt*(x - min)), 1, D_MLT-1)
// and plane 0 additionally marks the rows set in mr_j.  min, max and mlt come
// from the masked extremes (xcalc_setmaxmin, xcalc.c:5-39):
//   min = min_x - (max_x-min_x)/16,  max = max_x + (max_x-min_x)/16,
//   mlt = D_MLT / (max - min).
// The products that read the planes (At_T_YnWt_S_Zn_ww, An_ZtSn_ww) undo the
// scaling exactly as the reference does, so the planes must match bit for bit:
// the conversion is one IEEE subtract, one multiply and a truncation, computed
// here with the same rounding.
//
// Device side: the masked min / max is a grid reduction (exact, order-free);
// the planes are built one warp per (column, 32-row word): every lane
// quantises one row and each plane word is one __ballot_sync, bit-reversed
// into the reference's MSB-first byte order.  The planes stay resident on the
// device for the products that follow, and are copied into M_X->wX for
// callers that read them on the host.
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <mutex>
#include <optional>

#include "abi_common.cuh"
#include "bit_transpose.cuh"
#include "bcc_model.h"
#include "lmirror.cuh"

namespace lakgb {

namespace {

// GLOBAL_D_MLT (default lakcluster_ver18.c:83), per host thread: concurrent
// solves may use different B_MLT.
thread_local long long g_d_mlt = 4294967296LL;

struct XcalcParams {
  const double *lf;
  const long long *row_off;  // per a-row of Yn (nrows_a): element offset, -1 = not retained
  int nrows_a;
  const long long *col_off;  // per retained column nc_j
  int ncols_j;
  double min, mlt;
  unsigned long long dmax;   // D_MLT - 1
  int ncols_per;
  long long brows;           // bytes per plane row
  uint8_t *planes;
  unsigned long long lf_n, planes_n;  // elements of lf, bytes of planes (bounds checks)
  int *bad;                  // set when an index would leave its buffer (access skipped)
  const double *dev_scalars; // a deferred call: device min, max, mlt (then min / mlt above are unused)
};

// The masked min / max compare order keys instead of doubles: GB300's FP64
// pipe issues about two compares per clock per SM, which held a min/max scan
// to a quarter of HBM bandwidth, while the integer pipe compares 64-bit keys
// at memory speed.  The key of x is its bit pattern with the sign bit flipped
// for x >= 0 and every bit flipped for x < 0, so unsigned key order is the
// order of the values, with -0 below +0.  The reference keeps the first of
// equal extremes (xcalc.c:25), so a min or max of zero may differ from it in
// sign only; min, max and mlt (xcalc.c:130) come out the same either way:
// a zero extreme enters them only through differences with the other extreme
// or, when both are zero, through min_data + 1 (xcalc.c:34).
__device__ __forceinline__ unsigned long long order_key(double x) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__device__ __forceinline__ double key_value(unsigned long long k) {
  return __longlong_as_double((long long)((k >> 63) ? (k & 0x7fffffffffffffffull) : ~k));
}

// Grid: blockIdx.x * blockDim.x + threadIdx.x strides the retained rows, each
// thread holding kMinMaxRows row offsets in registers for all its columns;
// blockIdx.y strides the retained columns, kMinMaxCols per pass, so that
// kMinMaxRows * kMinMaxCols loads are in flight per thread.  One partial
// (min, max, any) per block.
constexpr int kMinMaxRows = 4, kMinMaxCols = 2, kMinMaxThreads = 256;

__global__ void xcalc_minmax_kernel(const double *lf, const long long *rows_j, int nr,
                                    const long long *cols_j, int nc, double *pmin, double *pmax,
                                    int *pany) {
  unsigned long long kmn = ~0ull, kmx = 0ull;  // empty: kmn > kmx
  const int stride = gridDim.x * blockDim.x;
  for (int rb = blockIdx.x * blockDim.x + threadIdx.x; rb < nr; rb += kMinMaxRows * stride) {
    long long ro[kMinMaxRows];
    bool rok[kMinMaxRows];
#pragma unroll
    for (int u = 0; u < kMinMaxRows; ++u) {
      const int r = rb + u * stride;
      rok[u] = r < nr;
      ro[u] = rok[u] ? rows_j[r] : 0;
    }
    for (int c = blockIdx.y; c < nc; c += kMinMaxCols * gridDim.y) {
      double x[kMinMaxCols][kMinMaxRows];
      bool cok[kMinMaxCols];
#pragma unroll
      for (int k = 0; k < kMinMaxCols; ++k) {
        const int ck = c + k * gridDim.y;
        cok[k] = ck < nc;
        const long long co = cok[k] ? cols_j[ck] : 0;
#pragma unroll
        for (int u = 0; u < kMinMaxRows; ++u) x[k][u] = (cok[k] && rok[u]) ? __ldg(lf + ro[u] + co) : 0.0;
      }
#pragma unroll
      for (int k = 0; k < kMinMaxCols; ++k)
#pragma unroll
        for (int u = 0; u < kMinMaxRows; ++u)
          if (cok[k] && rok[u]) {
            const unsigned long long q = order_key(x[k][u]);
            kmn = q < kmn ? q : kmn;
            kmx = q > kmx ? q : kmx;
          }
    }
  }
  __shared__ unsigned long long smn[32], smx[32];
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long omn = __shfl_xor_sync(0xffffffffu, kmn, o);
    const unsigned long long omx = __shfl_xor_sync(0xffffffffu, kmx, o);
    kmn = omn < kmn ? omn : kmn;
    kmx = omx > kmx ? omx : kmx;
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { smn[warp] = kmn; smx[warp] = kmx; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      kmn = smn[w] < kmn ? smn[w] : kmn;
      kmx = smx[w] > kmx ? smx[w] : kmx;
    }
    const int b = blockIdx.x + gridDim.x * blockIdx.y;
    const int any = kmn <= kmx;
    pmin[b] = any ? key_value(kmn) : 0.0;
    pmax[b] = any ? key_value(kmx) : 0.0;
    pany[b] = any;
  }
}

// A deferred call's min / max partials reduced on the device (one warp), and
// min, max and mlt formed from them with the host's operations (xcalc.c:34,
// :130): out = {min, max, mlt}.
__global__ void xcalc_scalars_from_partials_kernel(const double *pmin, const double *pmax, const int *pany,
                                                   int blocks, double d_mlt, double *out) {
  unsigned long long kmn = ~0ull, kmx = 0ull;
  for (int i = threadIdx.x; i < blocks; i += 32)
    if (pany[i]) {
      const unsigned long long a = order_key(pmin[i]), b = order_key(pmax[i]);
      kmn = a < kmn ? a : kmn;
      kmx = b > kmx ? b : kmx;
    }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long a = __shfl_xor_sync(0xffffffffu, kmn, o), b = __shfl_xor_sync(0xffffffffu, kmx, o);
    kmn = a < kmn ? a : kmn;
    kmx = b > kmx ? b : kmx;
  }
  if (threadIdx.x == 0) {
    double mn = 0.0, mx = 0.0;
    if (kmn <= kmx) { mn = key_value(kmn); mx = key_value(kmx); }
    if (mn >= mx) mx = __dadd_rn(mn, 1.0);
    const double w = __dsub_rn(mx, mn);
    const double lo = __dsub_rn(mn, __dmul_rn(0.0625, w)), hi = __dadd_rn(mx, __dmul_rn(0.0625, w));
    out[0] = lo;
    out[1] = hi;
    out[2] = __ddiv_rn(d_mlt, __dsub_rn(hi, lo));
  }
}

// Warp per (column, 128-row group): lane l quantises rows 128g + 32k + l,
// k = 0..3 (four independent coalesced loads).  Per k, the 32 x 32 bit
// matrix (row l = bits nb0 .. nb0+31 of lane l's value) is transposed in
// registers, so lane j holds the word of bit nb0+j; lane j then writes its
// plane's four words (128 rows) as one 16-byte store.  Plane rows are
// bsize(nrows) bytes, a multiple of 240 and so of 16, and a group that starts
// inside the rows ends inside the 1920-bit padding, so every store is aligned
// and within its plane row.
__global__ void xcalc_planes_kernel(XcalcParams p) {
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  const int ngroups = (p.nrows_a + 127) >> 7;
  if (warp >= (long long)ngroups * p.ncols_j) return;
  const int g = (int)(warp % ngroups), c = (int)(warp / ngroups);
  const long long co = p.col_off[c];
  unsigned long long cz[4];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    const int r = (g << 7) + (k << 5) + lane;
    cz[k] = 0ull;
    const long long ro = r < p.nrows_a ? p.row_off[r] : -1;
    if (ro >= 0 && (unsigned long long)(ro + co) >= p.lf_n) {
      atomicCAS(p.bad, 0, 1);
    } else if (ro >= 0) {
      const double x = p.lf[ro + co];
      const double pmin = p.dev_scalars ? p.dev_scalars[0] : p.min;
      const double pmlt = p.dev_scalars ? p.dev_scalars[2] : p.mlt;
      unsigned long long v = __double2ull_rz(__dmul_rn(pmlt, __dsub_rn(x, pmin)));
      if (v < 1ull) v = 1ull;
      if (v > p.dmax) v = p.dmax;
      cz[k] = v;
    }
  }
  const int nbits = p.ncols_per - 1;
  for (int nb0 = 0; nb0 < nbits; nb0 += 32) {
    const int nr_ = min(32, nbits - nb0);
    unsigned mine[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) mine[k] = transpose32(__brev((uint32_t)(cz[k] >> nb0)), lane);
    if (lane < nr_ && (mine[0] | mine[1] | mine[2] | mine[3])) {
      // lane j's word has row i at bit 31-i; memory wants row 8m+q at byte m, bit 7-q.
      uint4 v;
      v.x = __byte_perm(mine[0], 0u, 0x0123);
      v.y = __byte_perm(mine[1], 0u, 0x0123);
      v.z = __byte_perm(mine[2], 0u, 0x0123);
      v.w = __byte_perm(mine[3], 0u, 0x0123);
      const long long plane = (long long)p.ncols_per * c + p.ncols_per - 1 - (nb0 + lane);
      const unsigned long long off = (unsigned long long)(plane * p.brows + 16ll * g);
      if (off + 16 > p.planes_n || (off & 15ull)) atomicCAS(p.bad, 0, 2);
      else *reinterpret_cast<uint4 *>(p.planes + off) = v;
    }
  }
}

// --- allocation-free variant ---------------------------------------------
//
// lakgb_xcalc_noalloc runs the same quantisation on caller-owned device
// buffers for callers that cannot allocate device memory.  Its only scratch
// is this file-scope array: per retained column, the column's min, max and a
// "has values" flag (3 x kNoAllocMaxCols doubles), then min / max / mlt of
// the whole matrix (4 doubles) -- 786,464 bytes in all.  Every entry a call
// reads is written earlier in the same call, so nothing needs clearing; the
// array is shared by every call on a device, so calls whose kernels overlap
// on the GPU race.
constexpr int kNoAllocMaxCols = LAKGB_XCALC_NOALLOC_MAX_COLS;
static __device__ __align__(256) double g_xcalc_noalloc_scratch[3 * kNoAllocMaxCols + 4];

// Column-wise min / max of the retained entries: one block per column.
__global__ void xcalc_colminmax_kernel(const double *lf, const long long *rows_j, int nr, const long long *cols_j,
                                       int nc, double *scratch) {
  const int c = blockIdx.x;
  if (c >= nc) return;
  double mn = 0.0, mx = 0.0;
  int any = 0;
  for (int r = threadIdx.x; r < nr; r += blockDim.x) {
    const double x = lf[rows_j[r] + cols_j[c]];
    if (!any) { mn = x; mx = x; any = 1; }
    else { mn = x < mn ? x : mn; mx = x > mx ? x : mx; }
  }
  __shared__ double smn[32], smx[32];
  __shared__ int sany[32];
  for (int o = 16; o > 0; o >>= 1) {
    const double omn = __shfl_xor_sync(0xffffffffu, mn, o);
    const double omx = __shfl_xor_sync(0xffffffffu, mx, o);
    const int oany = __shfl_xor_sync(0xffffffffu, any, o);
    if (oany) {
      if (!any) { mn = omn; mx = omx; any = 1; }
      else { mn = omn < mn ? omn : mn; mx = omx > mx ? omx : mx; }
    }
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { smn[warp] = mn; smx[warp] = mx; sany[warp] = any; }
  __syncthreads();
  if (threadIdx.x == 0) {
    int a = 0;
    double bmn = 0.0, bmx = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      if (!sany[w]) continue;
      if (!a) { bmn = smn[w]; bmx = smx[w]; a = 1; }
      else { bmn = smn[w] < bmn ? smn[w] : bmn; bmx = smx[w] > bmx ? smx[w] : bmx; }
    }
    scratch[c] = bmn;
    scratch[kNoAllocMaxCols + c] = bmx;
    scratch[2 * kNoAllocMaxCols + c] = a ? 1.0 : 0.0;
  }
}

// One thread folds the column partials in column order (min / max are exact,
// so the order does not change the result) and derives min, max and mlt with
// the host formula's operations (xcalc.c:129-130, 240).
__global__ void xcalc_scalars_kernel(int nc, double d_mlt, double *scratch) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double mn = 0.0, mx = 0.0;
  int set = 0;
  for (int c = 0; c < nc; ++c) {
    if (scratch[2 * kNoAllocMaxCols + c] == 0.0) continue;
    const double a = scratch[c], b = scratch[kNoAllocMaxCols + c];
    if (!set) { mn = a; mx = b; set = 1; }
    else { mn = a < mn ? a : mn; mx = b > mx ? b : mx; }
  }
  if (mn >= mx) mx = __dadd_rn(mn, 1.0);
  const double range = __dsub_rn(mx, mn);
  const double lo = __dsub_rn(mn, __dmul_rn(0.0625, range));
  const double hi = __dadd_rn(mx, __dmul_rn(0.0625, range));
  double mlt = __ddiv_rn(d_mlt, __dsub_rn(hi, lo));
  double* out = scratch + 3 * kNoAllocMaxCols;
  out[0] = lo;
  out[1] = hi;
  out[2] = mlt;            // used by the plane kernel
  if (!isfinite(mlt) || mlt <= 0) mlt = 1.0;
  out[3] = mlt;            // the value wrap_xcalc stores as M_X->mlt_d
}

// A warp per (32-row word, column); grid-stride over the warps, so any
// launch size covers every word (the warp index is uniform within a warp, as
// the ballots need).
__global__ void xcalc_planes_dev_kernel(XcalcParams p, const double *scalars) {
  p.min = scalars[0];
  p.mlt = scalars[2];
  const int lane = threadIdx.x & 31;
  const int nwords = (p.nrows_a + 31) >> 5;
  const long long total = (long long)nwords * p.ncols_j;
  const long long step = ((long long)gridDim.x * blockDim.x) >> 5;
  for (long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; warp < total; warp += step) {
    const int w = (int)(warp % nwords), c = (int)(warp / nwords);
    const int r = (w << 5) + lane;
    unsigned long long cz = 0ull;
    if (r < p.nrows_a) {
      const long long ro = p.row_off[r];
      if (ro >= 0) {
        const double x = p.lf[ro + p.col_off[c]];
        cz = __double2ull_rz(__dmul_rn(p.mlt, __dsub_rn(x, p.min)));
        if (cz < 1ull) cz = 1ull;
        if (cz > p.dmax) cz = p.dmax;
      }
    }
    for (int nb = 0; nb < p.ncols_per - 1; ++nb) {
      const unsigned bal = __ballot_sync(0xffffffffu, (unsigned)((cz >> nb) & 1ull));
      if (lane == 0 && bal) {
        const unsigned word = __byte_perm(__brev(bal), 0u, 0x0123);
        const long long plane = (long long)p.ncols_per * c + p.ncols_per - 1 - nb;
        *reinterpret_cast<unsigned *>(p.planes + plane * p.brows + 4ll * w) = word;
      }
    }
  }
}

std::mutex g_noalloc_mu;
void *g_noalloc_scratch[64] = {nullptr};

// Device address of the scratch array on the current device, looked up once
// per device (the lookup is a runtime call that must not run inside a stream
// capture, so callers make their first call before any capture).
double *noalloc_scratch() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
  std::lock_guard<std::mutex> lk(g_noalloc_mu);
  if (!g_noalloc_scratch[dev]) {
    void *ptr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&ptr, g_xcalc_noalloc_scratch);
    if (e != cudaSuccess) {
      set_error(1000 + (int)e, "lakgb_xcalc_noalloc: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
      return nullptr;
    }
    g_noalloc_scratch[dev] = ptr;
  }
  return static_cast<double *>(g_noalloc_scratch[dev]);
}

inline bool bit_on(const unsigned char *b, long n) { return (b[n / 8] >> (7 - n % 8)) & 1; }
inline unsigned long long pick(int s, unsigned long long j, unsigned long long b, unsigned long long a) {
  return s == LAKGB_SPACING_j ? j : (s == LAKGB_SPACING_b ? b : a);
}

}  // namespace

}  // namespace lakgb

using namespace lakgb;

extern "C" void lakgb_set_d_mlt(long long d_mlt) { g_d_mlt = d_mlt; }

namespace lakgb {
namespace {
// Per-thread device flag of the planes kernel's bounds checks.  It is
// zeroed on the thread's own stream: that stream does not wait for the
// legacy default stream (it is created non-blocking), so a plain cudaMemset
// could still be pending when the first read of the flag runs, which would
// then see whatever the allocation held before.
int *bad_flag() {
  thread_local int *d = nullptr;
  if (!d) {
    LAKGB_CUDA(cudaMalloc(&d, sizeof(int)));
    LAKGB_CUDA(cudaMemsetAsync(d, 0, sizeof(int), stream()));
  }
  return d;
}

// Calls inside a deferral scope: their min, max and mlt stay on the device
// (three doubles per call, in chunks of kSlots calls) until the scope ends;
// then M_X's fields are set from them.
constexpr int kSlots = 256;
struct XcalcDeferred { M_handle *M_X; int slot; };
thread_local std::vector<DBuf> t_xs_chunks;
thread_local int t_xs_used = 0;
thread_local std::vector<XcalcDeferred> t_xs;

double *xcalc_slot(int &slot) {
  if (t_xs_used == (int)t_xs_chunks.size() * kSlots) t_xs_chunks.emplace_back((size_t)kSlots * 3 * sizeof(double));
  slot = t_xs_used++;
  return t_xs_chunks[slot / kSlots].as<double>() + (size_t)(slot % kSlots) * 3;
}

void xcalc_deferred_enqueue() {}

// After the scope's wait: the scalars into M_X (xcalc.c:240), the planes
// kernels' bounds flag checked once.
void xcalc_deferred_finish() {
  std::vector<double> h((size_t)t_xs_used * 3);
  for (size_t c = 0; c < t_xs_chunks.size(); ++c) {
    const int n = std::min(kSlots, t_xs_used - (int)c * kSlots);
    if (n > 0)
      LAKGB_CUDA(cudaMemcpyAsync(h.data() + c * kSlots * 3, t_xs_chunks[c].p, (size_t)n * 3 * sizeof(double),
                                 cudaMemcpyDeviceToHost, stream()));
  }
  int hbad = 0;
  LAKGB_CUDA(cudaMemcpyAsync(&hbad, bad_flag(), sizeof(int), cudaMemcpyDeviceToHost, stream()));
  LAKGB_CUDA(cudaStreamSynchronize(stream()));
  for (const XcalcDeferred &d : t_xs) {
    const double *v = h.data() + (size_t)d.slot * 3;
    d.M_X->min_d = v[0]; d.M_X->max_d = v[1]; d.M_X->mlt_d = v[2];
    if (!isfinite(d.M_X->mlt_d) || d.M_X->mlt_d <= 0) d.M_X->mlt_d = 1;
  }
  if (hbad) {
    printf(" %% Warning! wrap_xcalc: a call skipped an out-of-range index (code %d)\n", hbad);
    set_error(5, "wrap_xcalc: a call skipped an out-of-range index (code %d)", hbad);
    LAKGB_CUDA(cudaMemsetAsync(bad_flag(), 0, sizeof(int), stream()));
  }
  t_xs.clear();
  t_xs_chunks.clear();
  t_xs_used = 0;
}
}  // namespace
}  // namespace lakgb

extern "C" void wrap_xcalc(int *tidx, void **vpra, pthread_t *thread_in, unsigned char *mr_j,
                           unsigned char *mr_b, unsigned char *mc_j, unsigned char *mc_b,
                           L_handle *lf_YnWt, double *YnWt, int *Yn_nrows_p, int *Wn_nrows_p,
                           M_handle **M_X_p, int *b_mlt_p, int trm_flag) {
  LAKGB_PROFILE_CALL("wrap_xcalc");
  (void)tidx; (void)vpra; (void)thread_in;
  const int Yn_nrows = *Yn_nrows_p, Wn_nrows = *Wn_nrows_p, b_mlt = *b_mlt_p;
  if (!M_X_p || !*M_X_p) {
    set_error(3, "wrap_xcalc: *M_X_p must be pre-allocated");
    return;
  }
  if (!mr_j || !mr_b || !mc_j || !mc_b) printf(" %% Warning! null mask in get_xcalc\n");
  M_handle *M_X = *M_X_p;
  const long ylen = lakbcc::bsize(Yn_nrows), wlen = lakbcc::bsize(Wn_nrows);
  const int rpop_j = popcount_bytes(mr_j, ylen), rpop_b = popcount_bytes(mr_b, ylen);
  const int cpop_j = popcount_bytes(mc_j, wlen);
  const long long length = (long long)Yn_nrows * Wn_nrows;
  const int ncols_per = b_mlt + 1;
  if (ncols_per > 63) printf(" %% Warning! overflow in get_xcalc!\n");

  // Retained rows / columns and their element offsets (L2_lf_get, L_init.c:188-200).
  const int sr = lf_YnWt ? lf_YnWt->spacing_row : 0, sc = lf_YnWt ? lf_YnWt->spacing_col : 0;
  const unsigned long long rs = lf_YnWt ? lf_YnWt->row_stride : 0;
  std::vector<long long> row_off_a((size_t)(Yn_nrows > 0 ? Yn_nrows : 1), -1), rows_j, cols_j;
  {
    unsigned long long j = 0, b = 0;
    for (int a = 0; a < Yn_nrows; ++a) {
      if (!bit_on(mr_b, a)) continue;
      if (bit_on(mr_j, a)) {
        const long long o = trm_flag ? (long long)(pick(sc, j, b, a) * rs) : (long long)pick(sr, j, b, a);
        row_off_a[a] = o;
        rows_j.push_back(o);
        ++j;
      }
      ++b;
    }
    j = 0; b = 0;
    for (int a = 0; a < Wn_nrows; ++a) {
      if (!bit_on(mc_b, a)) continue;
      if (bit_on(mc_j, a)) {
        cols_j.push_back(trm_flag ? (long long)pick(sr, j, b, a) : (long long)(pick(sc, j, b, a) * rs));
        ++j;
      }
      ++b;
    }
  }
  long long max_off = 0;
  for (long long o : rows_j) max_off = o > max_off ? o : max_off;
  long long max_coff = 0;
  for (long long o : cols_j) max_coff = o > max_coff ? o : max_coff;
  const size_t lf_elems = (size_t)(max_off + max_coff + 1);

  std::optional<Stager> st;
  DBuf d_lf, d_rows, d_cols, d_roff_all;
  double min_data = 0.0, max_data = 0.0;
  const int nr = (int)rows_j.size(), nc = (int)cols_j.size();
  // A mirrored matrix (lmirror.cu) is read in place.
  Mirror *mlf = (lf_YnWt && YnWt == lf_YnWt->lf) ? find_mirror(lf_YnWt) : nullptr;
  const double *plf = nullptr;
  // Inside a deferral scope (and when no host copy of the planes is wanted)
  // min, max and mlt stay on the device: the planes kernel reads them there
  // and M_X's fields are set when the scope ends, so the call does not wait.
  const bool deferred = defer_active() && !host_planes_wanted();
  double *dev_scalars = nullptr;
  int slot = -1;
  if (nr > 0 && nc > 0 && YnWt) {
    if (mlf && lf_elems <= mlf->n) {
      plf = mlf->d;
    } else {
      d_lf = DBuf(lf_elems * sizeof(double));
      d_lf.upload(YnWt, lf_elems * sizeof(double));
      plf = d_lf.as<double>();
    }
    // The Stager lives to the end of the call: arrays of 1 MB or more go to
    // buffers it owns, which must outlive the kernels below.
    st.emplace();
    d_rows = upload_vec(rows_j);
    d_cols = upload_vec(cols_j);
    d_roff_all = upload_vec(row_off_a);
    st->flush();
    // About 16 blocks per SM: rows across blockIdx.x (kMinMaxRows per
    // thread), columns across blockIdx.y.
    const int gx = std::min((nr + kMinMaxRows * kMinMaxThreads - 1) / (kMinMaxRows * kMinMaxThreads), 2432);
    const int gy = std::max(1, std::min(nc, 2432 / gx));
    const int blocks = gx * gy;
    DBuf d_min(blocks * sizeof(double)), d_max(blocks * sizeof(double)), d_any(blocks * sizeof(int));
    xcalc_minmax_kernel<<<dim3(gx, gy), kMinMaxThreads, 0, stream()>>>(plf, d_rows.as<long long>(), nr,
                                                       d_cols.as<long long>(), nc, d_min.as<double>(),
                                                       d_max.as<double>(), d_any.as<int>());
    LAKGB_CUDA(cudaGetLastError());
    count_launch();
    if (deferred) {
      dev_scalars = xcalc_slot(slot);
      xcalc_scalars_from_partials_kernel<<<1, 32, 0, stream()>>>(d_min.as<double>(), d_max.as<double>(),
                                                                 d_any.as<int>(), blocks, (double)g_d_mlt, dev_scalars);
      LAKGB_CUDA(cudaGetLastError());
      count_launch();
    } else {
      std::vector<double> hmin(blocks), hmax(blocks);
      std::vector<int> hany(blocks);
      int hbad = 0;  // an earlier call's planes kernel met an index outside its buffers
      LAKGB_CUDA(cudaMemcpyAsync(&hbad, bad_flag(), sizeof(int), cudaMemcpyDeviceToHost, stream()));
      LAKGB_CUDA(cudaMemcpyAsync(hmin.data(), d_min.p, blocks * sizeof(double), cudaMemcpyDeviceToHost, stream()));
      LAKGB_CUDA(cudaMemcpyAsync(hmax.data(), d_max.p, blocks * sizeof(double), cudaMemcpyDeviceToHost, stream()));
      LAKGB_CUDA(cudaMemcpyAsync(hany.data(), d_any.p, blocks * sizeof(int), cudaMemcpyDeviceToHost, stream()));
      LAKGB_CUDA(cudaStreamSynchronize(stream()));
      if (hbad) {
        printf(" %% Warning! wrap_xcalc: an earlier call skipped an out-of-range index (code %d)\n", hbad);
        set_error(5, "wrap_xcalc: an earlier call skipped an out-of-range index (code %d)", hbad);
        LAKGB_CUDA(cudaMemsetAsync(bad_flag(), 0, sizeof(int), stream()));
      }
      bool set = false;
      for (int i = 0; i < blocks; ++i) {
        if (!hany[i]) continue;
        if (!set) { min_data = hmin[i]; max_data = hmax[i]; set = true; }
        else { min_data = hmin[i] < min_data ? hmin[i] : min_data; max_data = hmax[i] > max_data ? hmax[i] : max_data; }
      }
    }
  }
  if (min_data >= max_data) max_data = min_data + 1;
  const double min = min_data - 0.0625 * (max_data - min_data);
  const double max = max_data + 0.0625 * (max_data - min_data);
  const double mlt = (double)g_d_mlt / (max - min);

  int ncols_bZ = 0, nrows_bZ = 0;
  long long brows = 0;
  if (length > 0 && lf_YnWt != nullptr) {
    ncols_bZ = ncols_per * cpop_j;
    nrows_bZ = Yn_nrows;
    brows = lakbcc::bsize(nrows_bZ);
    const size_t nbytes = (size_t)ncols_bZ * (size_t)brows;
    if (!M_X->Ara) {
      M_X->Ara = (unsigned char *)calloc(nbytes + kBlockBytes, 1);
      if (!M_X->Ara) { set_error(2, "wrap_xcalc: out of host memory"); return; }
    }
    DBuf planes(nbytes);
    planes.zero();
    // Plane 0: the rows set in mr_j (xcalc.c:141).
    std::vector<unsigned char> row0((size_t)brows, 0);
    for (int a = 0; a < Yn_nrows; ++a)
      if (bit_on(mr_j, a)) row0[a / 8] |= (unsigned char)(1 << (7 - a % 8));
    if (nbytes) planes.upload(row0.data(), (size_t)brows);
    if (nr > 0 && nc > 0 && YnWt) {
      XcalcParams p{};
      p.lf = plf;
      p.row_off = d_roff_all.as<long long>(); p.nrows_a = Yn_nrows;
      p.col_off = d_cols.as<long long>(); p.ncols_j = nc;
      p.min = min; p.mlt = mlt; p.dmax = (unsigned long long)(g_d_mlt - 1);
      p.dev_scalars = dev_scalars;
      p.ncols_per = ncols_per; p.brows = brows; p.planes = planes.as<uint8_t>();
      p.lf_n = (plf == d_lf.p) ? (unsigned long long)lf_elems : (unsigned long long)mlf->n;
      p.planes_n = (unsigned long long)nbytes;
      p.bad = bad_flag();
      const long long warps = (long long)((Yn_nrows + 127) / 128) * nc;
      const int blocks = (int)((warps * 32 + 255) / 256);
      xcalc_planes_kernel<<<blocks, 256, 0, stream()>>>(p);
      LAKGB_CUDA(cudaGetLastError());
      count_launch();
    }
    if (host_planes_wanted()) {
      if (nbytes) LAKGB_CUDA(cudaMemcpyAsync(M_X->Ara, planes.p, nbytes, cudaMemcpyDeviceToHost, stream()));
      LAKGB_CUDA(cudaStreamSynchronize(stream()));
    }
    resident_put(M_X->Ara, nbytes, std::move(planes));
  }
  // M_X fields (xcalc.c:231-241).
  M_X->nrows = ncols_bZ; M_X->ncols = nrows_bZ;
  M_X->nrows_extend = (lakbcc::BITJ - (M_X->nrows % lakbcc::BITJ)) % lakbcc::BITJ;
  M_X->mr_length = lakbcc::bsize(M_X->nrows);
  M_X->ncols_extend = (lakbcc::BITJ - (M_X->ncols % lakbcc::BITJ)) % lakbcc::BITJ;
  M_X->mc_length = lakbcc::bsize(M_X->ncols);
  for (int j = 0; j < ncols_bZ; ++j) { lakbcc::bset_on(M_X->mr_b, j); lakbcc::bset_on(M_X->mr_j, j); }
  M_X->rpop_b = ncols_bZ; M_X->rpop_j = ncols_bZ;
  for (unsigned long i = 0; i < M_X->mc_length; ++i) { M_X->mc_b[i] = mr_b[i]; M_X->mc_j[i] = mr_j[i]; }
  M_X->cpop_b = rpop_b; M_X->cpop_j = rpop_j;
  M_X->wX = M_X->Ara;
  M_X->ncols_per_z = ncols_per;
  if (dev_scalars) {
    t_xs.push_back(XcalcDeferred{M_X, slot});
    defer_register(xcalc_deferred_enqueue, xcalc_deferred_finish);
  } else {
    M_X->max_d = max; M_X->min_d = min; M_X->mlt_d = mlt;
    if (!isfinite(M_X->mlt_d) || M_X->mlt_d <= 0) M_X->mlt_d = 1;
  }
  lakbcc::mhandle_mxget(M_X);
}

extern "C" int lakgb_xcalc_noalloc(const struct lakgb_xcalc_noalloc_args *a) {
  if (!a || !a->planes || !a->min_max_mlt || (a->n_rows_j > 0 && a->n_cols_j > 0 && (!a->lf || !a->rows_j ||
      !a->cols_j || !a->row_off_a))) {
    set_error(2, "lakgb_xcalc_noalloc: null argument");
    return 2;
  }
  if (a->n_cols_j < 0 || a->n_rows_j < 0 || a->nrows_a < 0) {
    set_error(2, "lakgb_xcalc_noalloc: negative count (nrows_a %d, n_rows_j %d, n_cols_j %d)", a->nrows_a,
              a->n_rows_j, a->n_cols_j);
    return 2;
  }
  if (a->n_cols_j > kNoAllocMaxCols) {
    set_error(2, "lakgb_xcalc_noalloc: %d retained columns exceed the scratch limit of %d", a->n_cols_j,
              kNoAllocMaxCols);
    return 2;
  }
  if (a->b_mlt < 1 || a->b_mlt > 62 || a->d_mlt < 2) {
    set_error(2, "lakgb_xcalc_noalloc: b_mlt %d outside [1, 62] or d_mlt %lld below 2", a->b_mlt, a->d_mlt);
    return 2;
  }
  // The plane kernel stores whole 4-byte words at planes + plane * brows + 4 * w.
  if (a->brows < (long long)((a->nrows_a + 31) / 32) * 4 || (a->brows & 3) ||
      (reinterpret_cast<uintptr_t>(a->planes) & 3)) {
    set_error(2, "lakgb_xcalc_noalloc: plane rows of %lld bytes too short or not a multiple of 4, or planes "
              "not 4-byte aligned", a->brows);
    return 2;
  }
  double *scratch = noalloc_scratch();
  if (!scratch) return 3;
  cudaStream_t s = static_cast<cudaStream_t>(a->stream);
  const int ncols_per = a->b_mlt + 1;
  const size_t nbytes = (size_t)ncols_per * (size_t)a->n_cols_j * (size_t)a->brows;
  if (nbytes) LAKGB_CUDA(cudaMemsetAsync(a->planes, 0, nbytes, s));
  if (nbytes && a->row0) LAKGB_CUDA(cudaMemcpyAsync(a->planes, a->row0, (size_t)a->brows, cudaMemcpyDeviceToDevice, s));
  const int nc = (a->n_rows_j > 0) ? a->n_cols_j : 0;
  if (nc > 0) {
    xcalc_colminmax_kernel<<<nc, 128, 0, s>>>(a->lf, a->rows_j, a->n_rows_j, a->cols_j, nc, scratch);
    LAKGB_CUDA(cudaGetLastError());
  }
  xcalc_scalars_kernel<<<1, 32, 0, s>>>(nc, (double)a->d_mlt, scratch);
  LAKGB_CUDA(cudaGetLastError());
  count_launch(nc > 0 ? 2 : 1);
  if (nc > 0) {
    XcalcParams p{};
    p.lf = a->lf; p.row_off = a->row_off_a; p.nrows_a = a->nrows_a;
    p.col_off = a->cols_j; p.ncols_j = nc;
    p.dmax = (unsigned long long)(a->d_mlt - 1); p.ncols_per = ncols_per; p.brows = a->brows;
    p.planes = a->planes;
    const long long warps = (long long)((a->nrows_a + 31) / 32) * nc;
    const long long blocks = std::min<long long>((warps * 32 + 255) / 256, 1ll << 20);  // the kernel grid-strides
    xcalc_planes_dev_kernel<<<(unsigned)blocks, 256, 0, s>>>(p, scratch + 3 * kNoAllocMaxCols);
    LAKGB_CUDA(cudaGetLastError());
    count_launch();
  }
  double sc[4];
  LAKGB_CUDA(cudaMemcpyAsync(sc, scratch + 3 * kNoAllocMaxCols, sizeof(sc), cudaMemcpyDeviceToHost, s));
  LAKGB_CUDA(cudaStreamSynchronize(s));
  a->min_max_mlt[0] = sc[0];
  a->min_max_mlt[1] = sc[1];
  a->min_max_mlt[2] = sc[3];
  return 0;
}
