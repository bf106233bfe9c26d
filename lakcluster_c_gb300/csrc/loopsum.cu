// Loop-sum products over FP64 score matrices, and the SNP x SNP product AtTYn.
//
// AnZt_S_WnYt_vv (dir_c/AnZt_S_WnYt_vv.c:5-101, wrapper :103-145):
//   out[ma, s] = sum over Zn rows mz, in order, of (AnZt[ma,mz] * vS(s,mz)) * YnWt[ma,mz]
// AtTYn____WtSZn_vv (dir_c/AtTYn____WtSZn_vv.c:5-115, wrapper :117-159): over
// paired rows (na with nz) and paired inner rows (ny with nw), in order,
//   out[na, s] = sum (AtTYn[na,ny,s] * D_Yn[ny]) * ZtSWn[nz,nw,s]
// Both are sequential FP64 sums; one thread per output element runs the
// reference's recurrence (left-to-right, no FMA), with adjacent threads on
// adjacent rows so the column-major loads coalesce.
//
// AtTYn_vv (dir_c/AtTYn_vv.c:5-202, wrapper :204-235):
//   out[na, ny, t] = ((hhAY - hhAy*aY) - aA*hhaY) + (aA*hhay)*aY
//   hhAY = cpop_j(At) - 2*popcount(~(At_na ^ Tt_t ^ Yt_ny) & mc_j(At))
//        = 2*popcount((At_na ^ Tt_t ^ Yt_ny) & mc_j) - cpop_j
//   hhAy = AtTn[na,t], hhaY = YtTn[ny,t] (integers read from FP64),
//   hhay = -cpop_j(Tt) + 2*popcount(Tt_t & mc_j(Tt)), aA / aY the column
//   means of the At / Yt rows' 1920-bit blocks.
// The popcount is a tiled XOR Gram: per 1920-bit block the CTA stages
// (At ^ Tt) & mask for 64 At rows and Yt & mask for 64 Yt rows, and each
// thread accumulates a 4 x 4 tile of integer counts over all blocks.
#include <optional>

#include "abi_common.cuh"
#include "lmirror.cuh"
#include "bcc_model.h"

namespace lakgb {

namespace {

inline unsigned long long pick_u(int s, unsigned long long j, unsigned long long b, unsigned long long a) {
  return s == LAKGB_SPACING_j ? j : (s == LAKGB_SPACING_b ? b : a);
}

// Number of values in the populated part of an L_handle (2-D or 3-D).
unsigned long long populated(const L_handle *L, bool three_d) {
  unsigned long long n = L->row_stride * L->col_stride * (three_d ? L->lyr_stride : 1);
  return n > L->length ? L->length : n;
}

unsigned long long max_index(const std::vector<unsigned long long> &v) {
  unsigned long long m = 0;
  for (unsigned long long x : v) m = x > m ? x : m;
  return m;
}

// Upload the populated part of an L_handle's values.
DBuf upload_L(const L_handle *L, bool three_d) {
  const unsigned long long n = populated(L, three_d);
  DBuf d((size_t)(n ? n : 1) * sizeof(double));
  if (n) d.upload(L->lf, (size_t)n * sizeof(double));
  return d;
}

// One CTA per 16 rows: all 256 threads compute the products of a 16 x 128
// (row, mz) tile into shared memory -- reads of consecutive rows for one mz are
// contiguous in the column-major matrix -- then 16 threads add their row's
// products in mz order.  The additions stay sequential per row; the loads
// and multiplies run 256 wide.
constexpr int kSW_R = 16, kSW_Z = 128, kSW_T = 256;
struct SwnytCall {
  const double *A; const unsigned long long *a_r, *a_c;
  const double *Y; const unsigned long long *y_r, *y_c;
  const int8_t *vS; int nA, nZ, nS;
  const unsigned long long *out_r, *s_off;
  double *out;
  int tile0;  // grouped launch: first CTA of this call
};

// CTA (row tile rt, covariate s) of one call.
__device__ __forceinline__ void anzt_s_wnyt_tile(const SwnytCall &c, int rt, int s) {
  __shared__ double prod[kSW_Z][kSW_R + 1];
  const int r0 = rt * kSW_R;
  const int8_t *vs = c.vS + (long long)s * c.nZ;
  const int lr = threadIdx.x % kSW_R, lz = threadIdx.x / kSW_R;   // 16 rows x 16 columns per pass
  const int ma = r0 + lr;
  const unsigned long long ar = ma < c.nA ? c.a_r[ma] : 0, yr = ma < c.nA ? c.y_r[ma] : 0;
  double acc = 0.0;
  for (int z0 = 0; z0 < c.nZ; z0 += kSW_Z) {
    const int zn = min(kSW_Z, c.nZ - z0);
    __syncthreads();
    for (int z = lz; z < zn; z += kSW_T / kSW_R) {
      double v = 0.0;
      if (ma < c.nA) {
        const int mz = z0 + z;
        v = __dmul_rn(__dmul_rn(c.A[ar + c.a_c[mz]], (double)vs[mz]), c.Y[yr + c.y_c[mz]]);
      }
      prod[z][lr] = v;
    }
    __syncthreads();
    if (threadIdx.x < kSW_R)
      for (int z = 0; z < zn; ++z) acc = __dadd_rn(acc, prod[z][threadIdx.x]);
  }
  if (threadIdx.x < kSW_R && r0 + threadIdx.x < c.nA) c.out[c.out_r[r0 + threadIdx.x] + c.s_off[s]] = acc;
}

__global__ void __launch_bounds__(kSW_T) anzt_s_wnyt_kernel(SwnytCall c) {
  anzt_s_wnyt_tile(c, blockIdx.x, blockIdx.y);
}

// Several calls in one launch (a deferred group, lakgb_defer_end): CTA k
// belongs to the last call whose tile0 <= k; within it, row tile (k - tile0)
// % row tiles, covariate (k - tile0) / row tiles.
__global__ void __launch_bounds__(kSW_T) anzt_s_wnyt_group_kernel(const SwnytCall *calls, int n) {
  const int k = blockIdx.x;
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (calls[mid].tile0 <= k) lo = mid; else hi = mid - 1;
  }
  const SwnytCall &c = calls[lo];
  const int rtiles = (c.nA + kSW_R - 1) / kSW_R;
  const int j = k - c.tile0;
  anzt_s_wnyt_tile(c, j % rtiles, j / rtiles);
}

// The calls a deferral scope holds back (this host thread): their device
// inputs and outputs, and where each output goes on the host.
struct SwnytDeferred {
  SwnytCall c{};
  std::vector<DBuf> keep;   // uploads and the device output
  double *host_out = nullptr;
  unsigned long long length = 0;
};

struct WtszCall {
  const double *AY; const unsigned long long *ay_a, *ay_y, *ay_s;
  const double *ZW; const unsigned long long *zw_z, *zw_w, *zw_s;
  const double *Dy; int npairs, ninner, nS;
  const unsigned long long *out_r, *s_off;
  double *out;
  int tile0;  // grouped launch: first CTA of this call
};
constexpr int kWZ_T = 128;

// Thread = (pair i, covariate s): the sum over the inner rows in order.
__device__ __forceinline__ void attyn_wtszn_one(const WtszCall &c, int i, int s) {
  if (i >= c.npairs || s >= c.nS) return;
  const unsigned long long a0 = c.ay_a[i] + c.ay_s[s], z0 = c.zw_z[i] + c.zw_s[s];
  double acc = 0.0;
  for (int k = 0; k < c.ninner; ++k)
    acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(c.AY[a0 + c.ay_y[k]], c.Dy[k]), c.ZW[z0 + c.zw_w[k]]));
  c.out[c.out_r[i] + c.s_off[s]] = acc;
}

__global__ void attyn_wtszn_kernel(WtszCall c) {
  attyn_wtszn_one(c, blockIdx.x * blockDim.x + threadIdx.x, blockIdx.y);
}

__global__ void attyn_wtszn_group_kernel(const WtszCall *calls, int n) {
  const int k = blockIdx.x;
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (calls[mid].tile0 <= k) lo = mid; else hi = mid - 1;
  }
  const WtszCall &c = calls[lo];
  const int ptiles = (c.npairs + kWZ_T - 1) / kWZ_T;
  const int j = k - c.tile0;
  attyn_wtszn_one(c, (j % ptiles) * kWZ_T + threadIdx.x, j / ptiles);
}

struct WtszDeferred {
  WtszCall c{};
  std::vector<DBuf> keep;
  double *host_out = nullptr;
  unsigned long long length = 0;
};
thread_local int t_defer_depth = 0;
thread_local std::vector<SwnytDeferred> t_swnyt;
thread_local std::vector<WtszDeferred> t_wtsz;
struct DeferKind { void (*enqueue)(); void (*clear)(); };
thread_local std::vector<DeferKind> t_kinds;  // groups of other translation units
struct DeferCopy { double *host; DBuf dev; unsigned long long length; };
thread_local std::vector<DeferCopy> t_copies;  // other calls' outputs

// Page-locked host chunks and their device twins for held-back calls'
// inputs: bump-allocated, 16-byte aligned; `sent` is how much has been
// copied.  Arrays larger than a chunk get a chunk of their own.  Reset (not
// freed) when the outermost scope ends.
struct UpChunk { uint8_t *h = nullptr; uint8_t *d = nullptr; size_t cap = 0, used = 0, sent = 0; };
constexpr size_t kUpChunk = 4u << 20;
thread_local std::vector<UpChunk> t_up;
thread_local size_t t_up_cur = 0;

constexpr int kLd = kBlockWords + 1;
constexpr int kTY_M = 64, kTY_N = 64, kTY_TM = 4, kTY_TN = 4, kTY_T = 256;

struct AtTYnParams {
  const uint8_t *At; const uint32_t *a_rowb; int nA; long long a_row_bytes;
  const uint8_t *Yt; const uint32_t *y_rowb; int nY; long long y_row_bytes;
  const uint8_t *Tt; const uint32_t *t_rowb; long long t_row_bytes;
  const uint8_t *mask; int P; long long cpop;
  const double *hhAy;   // [t][na]
  const double *hhaY;   // [t][ny]
  const double *hhay;   // [t]
  const double *aA; const double *aY;
  const unsigned long long *out_a; const unsigned long long *out_y; const unsigned long long *out_t;
  double *out;
  // AtTAn (Yt = At): pairs na <= ny only, each also stored at
  // out_a2[ny] + out_y2[na] (the transposed position).
  int symmetric;
  const unsigned long long *out_a2; const unsigned long long *out_y2;
};

__global__ void __launch_bounds__(kTY_T, 2) attyn_kernel(AtTYnParams p) {
  extern __shared__ __align__(16) uint32_t smem[];
  uint32_t *As = smem, *Ys = smem + kTY_M * kLd;
  __shared__ long long a_off[kTY_M], y_off[kTY_N];
  const int t = blockIdx.z;
  const int n0 = blockIdx.x * kTY_N, m0 = blockIdx.y * kTY_M;
  if (p.symmetric && m0 > n0 + kTY_N - 1) return;  // wholly below the diagonal
  const int tid = threadIdx.x, tx = tid % (kTY_N / kTY_TN), ty = tid / (kTY_N / kTY_TN);
  for (int i = tid; i < kTY_M; i += kTY_T) a_off[i] = m0 + i < p.nA ? (long long)p.a_rowb[m0 + i] * p.a_row_bytes : -1;
  for (int i = tid; i < kTY_N; i += kTY_T) y_off[i] = n0 + i < p.nY ? (long long)p.y_rowb[n0 + i] * p.y_row_bytes : -1;
  const uint8_t *trow = p.Tt + (long long)p.t_rowb[t] * p.t_row_bytes;
  int c[kTY_TM][kTY_TN];
#pragma unroll
  for (int i = 0; i < kTY_TM; ++i)
#pragma unroll
    for (int j = 0; j < kTY_TN; ++j) c[i][j] = 0;
  for (int blk = 0; blk < p.P; ++blk) {
    __syncthreads();
    const long long boff = (long long)blk * kBlockBytes;
    const uint4 *mk = reinterpret_cast<const uint4 *>(p.mask + boff);
    const uint4 *tk = reinterpret_cast<const uint4 *>(trow + boff);
    for (int idx = tid; idx < kTY_M * 15; idx += kTY_T) {
      const int r = idx / 15, v = idx - r * 15;
      uint4 x = make_uint4(0u, 0u, 0u, 0u);
      if (a_off[r] >= 0) {
        const uint4 a = __ldg(reinterpret_cast<const uint4 *>(p.At + a_off[r] + boff) + v);
        const uint4 tt = __ldg(tk + v), m = __ldg(mk + v);
        x.x = (a.x ^ tt.x) & m.x; x.y = (a.y ^ tt.y) & m.y; x.z = (a.z ^ tt.z) & m.z; x.w = (a.w ^ tt.w) & m.w;
      }
      uint32_t *d = As + r * kLd + 4 * v;
      d[0] = x.x; d[1] = x.y; d[2] = x.z; d[3] = x.w;
    }
    for (int idx = tid; idx < kTY_N * 15; idx += kTY_T) {
      const int r = idx / 15, v = idx - r * 15;
      uint4 x = make_uint4(0u, 0u, 0u, 0u);
      if (y_off[r] >= 0) {
        const uint4 y = __ldg(reinterpret_cast<const uint4 *>(p.Yt + y_off[r] + boff) + v);
        const uint4 m = __ldg(mk + v);
        x.x = y.x & m.x; x.y = y.y & m.y; x.z = y.z & m.z; x.w = y.w & m.w;
      }
      uint32_t *d = Ys + r * kLd + 4 * v;
      d[0] = x.x; d[1] = x.y; d[2] = x.z; d[3] = x.w;
    }
    __syncthreads();
#pragma unroll 4
    for (int w = 0; w < kBlockWords; ++w) {
      uint32_t a[kTY_TM], y[kTY_TN];
#pragma unroll
      for (int i = 0; i < kTY_TM; ++i) a[i] = As[(ty + 16 * i) * kLd + w];
#pragma unroll
      for (int j = 0; j < kTY_TN; ++j) y[j] = Ys[(tx + 16 * j) * kLd + w];
#pragma unroll
      for (int i = 0; i < kTY_TM; ++i)
#pragma unroll
        for (int j = 0; j < kTY_TN; ++j) c[i][j] += __popc(a[i] ^ y[j]);
    }
  }
  const double hhay = p.hhay[t];
#pragma unroll
  for (int i = 0; i < kTY_TM; ++i) {
    const int na = m0 + ty + 16 * i;
    if (na >= p.nA) continue;
    const double hhAy = p.hhAy[(long long)t * p.nA + na], aA = p.aA[na];
#pragma unroll
    for (int j = 0; j < kTY_TN; ++j) {
      const int ny = n0 + tx + 16 * j;
      if (ny >= p.nY || (p.symmetric && na > ny)) continue;
      const double hhaY = p.hhaY[(long long)t * p.nY + ny], aY = p.aY[ny];
      const double hhAY = (double)(2ll * c[i][j] - p.cpop);
      const double v = __dadd_rn(__dsub_rn(__dsub_rn(hhAY, __dmul_rn(hhAy, aY)), __dmul_rn(aA, hhaY)),
                                 __dmul_rn(__dmul_rn(aA, hhay), aY));
      p.out[p.out_a[na] + p.out_y[ny] + p.out_t[t]] = v;
      if (p.symmetric) p.out[p.out_a2[ny] + p.out_y2[na] + p.out_t[t]] = v;
    }
  }
}

}  // namespace

bool defer_active() { return t_defer_depth > 0; }

const void *defer_put(const void *h, size_t n) {
  const size_t need = (n + 15) & ~(size_t)15;
  while (t_up_cur < t_up.size() && t_up[t_up_cur].used + need > t_up[t_up_cur].cap) ++t_up_cur;
  if (t_up_cur == t_up.size()) {
    if (!t_up.empty()) defer_flush();  // the earlier chunks' pending bytes go first
    UpChunk c;
    c.cap = std::max(kUpChunk, need);
    LAKGB_CUDA(cudaHostAlloc((void **)&c.h, c.cap, cudaHostAllocDefault));
    LAKGB_CUDA(cudaMalloc((void **)&c.d, c.cap));
    t_up.push_back(c);
  }
  UpChunk &c = t_up[t_up_cur];
  if (n) memcpy(c.h + c.used, h, n);
  const void *d = c.d + c.used;
  c.used += need;
  return d;
}

void defer_flush() {
  for (UpChunk &c : t_up) {
    if (c.used > c.sent)
      LAKGB_CUDA(cudaMemcpyAsync(c.d + c.sent, c.h + c.sent, c.used - c.sent, cudaMemcpyHostToDevice, stream()));
    c.sent = c.used;
  }
}

void defer_copy(double *host, DBuf &&dev, unsigned long long length) {
  t_copies.push_back(DeferCopy{host, std::move(dev), length});
}

void defer_register(void (*enqueue)(), void (*clear)()) {
  for (const DeferKind &k : t_kinds)
    if (k.enqueue == enqueue) return;
  t_kinds.push_back({enqueue, clear});
}

}  // namespace lakgb

using namespace lakgb;

extern "C" int wrap_AnZt_S_WnYt_vv__run(int *tidx, void **vpra, pthread_t *thread_in, int output_spacing_a,
                                        int output_spacing_s, M_handle *M_An, M_handle *M_St, M_handle *M_Zn,
                                        L_handle *lf_AnZt, L_handle *lf_YnWt, L_handle **output_p) {
  LAKGB_PROFILE_CALL("wrap_AnZt_S_WnYt_vv__run");
  (void)tidx; (void)vpra; (void)thread_in;
  const unsigned long long length_a = spacing_length(output_spacing_a, M_An);
  const unsigned long long length_s = spacing_length(output_spacing_s, M_St);
  const unsigned long long length = length_a * length_s;
  L_handle *out = ensure_output(output_p, length, "wrap_AnZt_S_WnYt_vv__run");
  if (!out) return (int)length;
  out->spacing_row = output_spacing_a; out->row_stride = length_a;
  out->spacing_col = output_spacing_s; out->col_stride = length_s;
  const int nA = (int)M_An->rpop_j, nZ = (int)M_Zn->rpop_j, nS = (int)M_St->rpop_j;
  if (!lf_AnZt || !lf_YnWt || nA == 0 || nS == 0) return (int)length;
  std::vector<unsigned long long> a_r(nA), y_r(nA), out_r(nA), a_c(nZ), y_c(nZ), s_off(nS);
  for (int i = 0; i < nA; ++i) {
    a_r[i] = pick_u(lf_AnZt->spacing_row, i, M_An->m_b_[i], M_An->m_a_[i]);
    y_r[i] = pick_u(lf_YnWt->spacing_row, i, M_An->m_b_[i], M_An->m_a_[i]);
    out_r[i] = pick_u(output_spacing_a, i, M_An->m_b_[i], M_An->m_a_[i]);
  }
  for (int k = 0; k < nZ; ++k) {
    a_c[k] = pick_u(lf_AnZt->spacing_col, k, M_Zn->m_b_[k], M_Zn->m_a_[k]) * lf_AnZt->row_stride;
    y_c[k] = pick_u(lf_YnWt->spacing_col, k, M_Zn->m_b_[k], M_Zn->m_a_[k]) * lf_YnWt->row_stride;
  }
  std::vector<int8_t> vS((size_t)nS * (nZ > 0 ? nZ : 1));
  for (int s = 0; s < nS; ++s) {
    s_off[s] = pick_u(output_spacing_s, s, M_St->m_b_[s], M_St->m_a_[s]) * length_a;
    const unsigned char *st = M_St->wX + (size_t)M_St->m_b_[s] * M_St->mc_length;
    for (int k = 0; k < nZ; ++k) {
      vS[(size_t)s * nZ + k] = (int8_t)lakbcc::bget_pm(st, M_Zn->m_a_[k]);
      if (!lakbcc::bget_on(M_St->mc_j, M_Zn->m_a_[k]))
        printf(" %% Warning! bit %d,%d,%d off in M_St->mc_j\n", k, (int)M_Zn->m_b_[k], (int)M_Zn->m_a_[k]);
    }
  }
  if (max_index(a_r) + max_index(a_c) >= populated(lf_AnZt, false) ||
      max_index(y_r) + max_index(y_c) >= populated(lf_YnWt, false)) {
    set_error(4, "wrap_AnZt_S_WnYt_vv__run: L_handle smaller than the rows and columns it is indexed by");
    return (int)length;
  }
  // Mirrored matrices (lmirror.cu) are read in place.
  Mirror *mA = find_mirror(lf_AnZt), *mY = find_mirror(lf_YnWt);
  // Inside a deferral scope the uploads are owned buffers (they must outlive
  // the call), and the kernel runs at the end of the scope.
  const bool defer = t_defer_depth > 0;
  std::optional<Stager> st;
  if (!defer) st.emplace();
  DBuf dA = mA ? DBuf() : upload_L(lf_AnZt, false);
  DBuf dY = (mY || lf_YnWt == lf_AnZt) ? DBuf() : upload_L(lf_YnWt, false);
  const double *pA = mA ? mA->d : dA.as<double>();
  const double *pY = mY ? mY->d : ((lf_YnWt == lf_AnZt) ? pA : dY.as<double>());
  auto up = [&](const auto &v) { return defer ? defer_upload(v) : upload_vec(v); };
  DBuf d_ar = up(a_r), d_yr = up(y_r), d_ac = up(a_c), d_yc = up(y_c);
  DBuf d_vS = up(vS), d_or = up(out_r), d_so = up(s_off);
  if (defer) defer_flush();
  DBuf d_out(length * sizeof(double));
  d_out.zero();
  SwnytCall c{};
  c.A = pA; c.a_r = d_ar.as<unsigned long long>(); c.a_c = d_ac.as<unsigned long long>();
  c.Y = pY; c.y_r = d_yr.as<unsigned long long>(); c.y_c = d_yc.as<unsigned long long>();
  c.vS = d_vS.as<int8_t>(); c.nA = nA; c.nZ = nZ; c.nS = nS;
  c.out_r = d_or.as<unsigned long long>(); c.s_off = d_so.as<unsigned long long>(); c.out = d_out.as<double>();
  if (defer) {
    SwnytDeferred d;
    d.c = c;
    d.host_out = out->lf;
    d.length = length;
    for (DBuf *b : {&dA, &dY, &d_ar, &d_yr, &d_ac, &d_yc, &d_vS, &d_or, &d_so, &d_out}) d.keep.push_back(std::move(*b));
    t_swnyt.push_back(std::move(d));
    return (int)length;
  }
  st->flush();
  anzt_s_wnyt_kernel<<<dim3((nA + kSW_R - 1) / kSW_R, nS), kSW_T, 0, stream()>>>(c);
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
  copy_back(out->lf, d_out, length);
  return (int)length;
}

// Deferral scope: AnZt_S_WnYt and AtTYn____WtSZn calls made inside it (the
// reference runs them on thread slots and joins them afterwards,
// GLOBAL_pthread_tuc) are held back and run together when the outermost scope
// ends -- one grouped launch per kind, then every output copied into its host
// L_handle.  Outputs are not to be read before the scope ends.
extern "C" void lakgb_defer_begin(void) { ++t_defer_depth; }

extern "C" void lakgb_defer_end(void) {
  if (t_defer_depth <= 0 || --t_defer_depth > 0) return;
  if (t_swnyt.empty() && t_wtsz.empty() && t_kinds.empty() && t_copies.empty()) return;
  LAKGB_PROFILE_CALL("lakgb_defer_end");
  std::vector<SwnytCall> c1;
  std::vector<WtszCall> c2;
  int tiles1 = 0, tiles2 = 0;
  for (auto &d : t_swnyt) {
    d.c.tile0 = tiles1;
    tiles1 += ((d.c.nA + kSW_R - 1) / kSW_R) * d.c.nS;
    c1.push_back(d.c);
  }
  for (auto &d : t_wtsz) {
    d.c.tile0 = tiles2;
    tiles2 += ((d.c.npairs + kWZ_T - 1) / kWZ_T) * d.c.nS;
    c2.push_back(d.c);
  }
  {
    DBuf d_c1, d_c2;
    if (!c1.empty()) {
      d_c1 = defer_upload(c1);
      defer_flush();
      anzt_s_wnyt_group_kernel<<<tiles1, kSW_T, 0, stream()>>>(d_c1.as<SwnytCall>(), (int)c1.size());
      LAKGB_CUDA(cudaGetLastError());
      count_launch();
    }
    if (!c2.empty()) {
      d_c2 = defer_upload(c2);
      defer_flush();
      attyn_wtszn_group_kernel<<<tiles2, kWZ_T, 0, stream()>>>(d_c2.as<WtszCall>(), (int)c2.size());
      LAKGB_CUDA(cudaGetLastError());
      count_launch();
    }
    for (const DeferKind &k : t_kinds) k.enqueue();
    if (profile_calls_on()) {
      LAKGB_PROFILE_CALL("(kernel wait)");
      LAKGB_CUDA(cudaStreamSynchronize(stream()));
    }
    LAKGB_PROFILE_CALL("(copy back + sync)");
    for (auto &d : t_swnyt)
      if (d.length)
        LAKGB_CUDA(cudaMemcpyAsync(d.host_out, d.c.out, d.length * sizeof(double), cudaMemcpyDeviceToHost, stream()));
    for (auto &d : t_wtsz)
      if (d.length)
        LAKGB_CUDA(cudaMemcpyAsync(d.host_out, d.c.out, d.length * sizeof(double), cudaMemcpyDeviceToHost, stream()));
    for (auto &c : t_copies)
      if (c.length)
        LAKGB_CUDA(cudaMemcpyAsync(c.host, c.dev.p, c.length * sizeof(double), cudaMemcpyDeviceToHost, stream()));
    LAKGB_CUDA(cudaStreamSynchronize(stream()));
  }
  t_copies.clear();
  for (UpChunk &c : t_up) c.used = c.sent = 0;  // the stream has drained: reuse the chunks
  t_up_cur = 0;
  t_swnyt.clear();
  t_wtsz.clear();
  for (const DeferKind &k : t_kinds) k.clear();
  t_kinds.clear();
}

extern "C" int wrap_AtTYn____WtSZn_vv__run(int *tidx, void **vpra, pthread_t *thread_in, int output_spacing_a,
                                           int output_spacing_s, M_handle *M_At, M_handle *M_Tt, M_handle *M_Yt,
                                           M_handle *M_Wt, M_handle *M_St, M_handle *M_Zt, double *Y_ajdk,
                                           L_handle *lf_AtTYn, L_handle *lf_ZtSWn, L_handle **output_p) {
  LAKGB_PROFILE_CALL("wrap_AtTYn____WtSZn_vv__run");
  (void)tidx; (void)vpra; (void)thread_in; (void)M_Tt;
  const unsigned long long length_a = spacing_length(output_spacing_a, M_At);
  const unsigned long long length_s = spacing_length(output_spacing_s, M_St);
  const unsigned long long length = length_a * length_s;
  L_handle *out = ensure_output(output_p, length, "wrap_AtTYn____WtSZn_vv__run");
  if (!out) return (int)length;
  out->spacing_row = output_spacing_a; out->row_stride = length_a;
  out->spacing_col = output_spacing_s; out->col_stride = length_s;
  const int npairs = (int)std::min(M_At->rpop_j, M_Zt->rpop_j);
  const int ninner = (int)std::min(M_Yt->rpop_j, M_Wt->rpop_j);
  const int nS = (int)M_St->rpop_j;
  // no pairs, covariates or inner rows: every sum is empty (the zeros written above)
  if (npairs == 0 || nS == 0 || ninner == 0) return (int)length;
  const int Y_pcols = (int)lakbcc::psize(M_Yt->nrows);
  const double *D_Yn = Y_ajdk + (size_t)lakbcc::AJDK_0_1 * Y_pcols;
  const L_handle *LA = lf_AtTYn, *LZ = lf_ZtSWn;
  std::vector<unsigned long long> ay_a(npairs), zw_z(npairs), out_r(npairs), ay_y(ninner > 0 ? ninner : 1),
      zw_w(ninner > 0 ? ninner : 1), ay_s(nS), zw_s(nS), s_off(nS);
  std::vector<double> Dy(ninner > 0 ? ninner : 1);
  for (int i = 0; i < npairs; ++i) {
    ay_a[i] = pick_u(LA->spacing_row, i, M_At->m_b_[i], M_At->m_a_[i]);
    zw_z[i] = pick_u(LZ->spacing_row, i, M_Zt->m_b_[i], M_Zt->m_a_[i]);
    out_r[i] = pick_u(output_spacing_a, i, M_At->m_b_[i], M_At->m_a_[i]);
  }
  for (int k = 0; k < ninner; ++k) {
    ay_y[k] = pick_u(LA->spacing_col, k, M_Yt->m_b_[k], M_Yt->m_a_[k]) * LA->row_stride;
    zw_w[k] = pick_u(LZ->spacing_col, k, M_Wt->m_b_[k], M_Wt->m_a_[k]) * LZ->row_stride;
    Dy[k] = D_Yn[M_Yt->m_a_[k] / lakbcc::POPLENGTH];
  }
  for (int s = 0; s < nS; ++s) {
    ay_s[s] = pick_u(LA->spacing_lyr, s, M_St->m_b_[s], M_St->m_a_[s]) * LA->row_stride * LA->col_stride;
    zw_s[s] = pick_u(LZ->spacing_lyr, s, M_St->m_b_[s], M_St->m_a_[s]) * LZ->row_stride * LZ->col_stride;
    s_off[s] = pick_u(output_spacing_s, s, M_St->m_b_[s], M_St->m_a_[s]) * length_a;
  }
  if (max_index(ay_a) + max_index(ay_y) + max_index(ay_s) >= populated(LA, true) ||
      max_index(zw_z) + max_index(zw_w) + max_index(zw_s) >= populated(LZ, true)) {
    set_error(4, "wrap_AtTYn____WtSZn_vv__run: L_handle smaller than the rows and columns it is indexed by");
    return (int)length;
  }
  // Mirrored inputs (lmirror.cu) are read in place; inside a deferral scope
  // the uploads are owned buffers and the kernel runs when the scope ends.
  Mirror *mLA = find_mirror(LA), *mLZ = find_mirror(LZ);
  const bool defer = t_defer_depth > 0;
  std::optional<Stager> st;
  if (!defer) st.emplace();
  DBuf dA = mLA ? DBuf() : upload_L(LA, true);
  DBuf dZ = (mLZ || LZ == LA) ? DBuf() : upload_L(LZ, true);
  const double *pA = mLA ? mLA->d : dA.as<double>();
  const double *pZ = mLZ ? mLZ->d : ((LZ == LA) ? pA : dZ.as<double>());
  auto up = [&](const auto &v) { return defer ? defer_upload(v) : upload_vec(v); };
  DBuf d_aa = up(ay_a), d_ay = up(ay_y), d_as = up(ay_s);
  DBuf d_zz = up(zw_z), d_zw = up(zw_w), d_zs = up(zw_s);
  DBuf d_D = up(Dy), d_or = up(out_r), d_so = up(s_off);
  if (defer) defer_flush();
  DBuf d_out(length * sizeof(double));
  d_out.zero();
  WtszCall c{};
  c.AY = pA; c.ay_a = d_aa.as<unsigned long long>(); c.ay_y = d_ay.as<unsigned long long>();
  c.ay_s = d_as.as<unsigned long long>();
  c.ZW = pZ; c.zw_z = d_zz.as<unsigned long long>(); c.zw_w = d_zw.as<unsigned long long>();
  c.zw_s = d_zs.as<unsigned long long>();
  c.Dy = d_D.as<double>(); c.npairs = npairs; c.ninner = ninner; c.nS = nS;
  c.out_r = d_or.as<unsigned long long>(); c.s_off = d_so.as<unsigned long long>(); c.out = d_out.as<double>();
  if (defer) {
    WtszDeferred d;
    d.c = c;
    d.host_out = out->lf;
    d.length = length;
    for (DBuf *b : {&dA, &dZ, &d_aa, &d_ay, &d_as, &d_zz, &d_zw, &d_zs, &d_D, &d_or, &d_so, &d_out})
      d.keep.push_back(std::move(*b));
    t_wtsz.push_back(std::move(d));
    return (int)length;
  }
  st->flush();
  attyn_wtszn_kernel<<<dim3((npairs + kWZ_T - 1) / kWZ_T, nS), kWZ_T, 0, stream()>>>(c);
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
  copy_back(out->lf, d_out, length);
  return (int)length;
}

namespace {

int attyn_entry(bool symmetric, const char *who, int output_spacing_a, int output_spacing_y, int output_spacing_t,
                M_handle *M_At, M_handle *M_Tt, M_handle *M_Yt, double *A_ajdk, double *Y_ajdk,
                L_handle *lf_AtTn, L_handle *lf_YtTn, L_handle **output_p) {
  const unsigned long long la = spacing_length(output_spacing_a, M_At);
  const unsigned long long ly = spacing_length(output_spacing_y, M_Yt);
  const unsigned long long lt = spacing_length(output_spacing_t, M_Tt);
  const unsigned long long length = la * ly * lt;
  // A mirrored output (lmirror.cu) is produced on the device only.
  Mirror *mo = *output_p ? find_mirror(*output_p) : nullptr;
  L_handle *out = nullptr;
  HostOutputFill fill;
  if (mo) {
    out = *output_p;
    if (out->length < length || mo->n < length) {
      set_error(2, "output length %llu < %llu in %s", out->length, length, who);
      return (int)length;
    }
    if (length) LAKGB_CUDA(cudaMemsetAsync(mo->d, 0, length * sizeof(double), stream()));
    mo->host_stale = true;
  } else {
    out = ensure_output(output_p, length, who, false);
    fill.L = out;
    fill.n = length;
  }
  if (!out) return (int)length;
  out->spacing_row = output_spacing_a; out->row_stride = la;
  out->spacing_col = output_spacing_y; out->col_stride = ly;
  out->spacing_lyr = output_spacing_t; out->lyr_stride = lt;
  const int nA = (int)M_At->rpop_j, nY = (int)M_Yt->rpop_j, nT = (int)M_Tt->rpop_j;
  if (nA == 0 || nY == 0 || nT == 0) return (int)length;
  if (M_Yt->mc_length != M_At->mc_length || M_Tt->mc_length != M_At->mc_length) {
    set_error(4, "%s: rows of unequal length", who);
    return (int)length;
  }
  const int A_pcols = (int)lakbcc::psize(M_At->nrows), Y_pcols = (int)lakbcc::psize(M_Yt->nrows);
  const double *a_An = A_ajdk + (size_t)lakbcc::AJDK_1_0 * A_pcols;
  const double *a_Yn = Y_ajdk + (size_t)lakbcc::AJDK_1_0 * Y_pcols;
  std::vector<uint32_t> a_rowb(M_At->m_b_, M_At->m_b_ + nA), y_rowb(M_Yt->m_b_, M_Yt->m_b_ + nY), t_rowb(nT);
  std::vector<double> hhAy((size_t)nT * nA), hhaY((size_t)nT * nY), hhay(nT), aA(nA), aY(nY);
  std::vector<unsigned long long> out_a(nA), out_y(nY), out_t(nT);
  for (int i = 0; i < nA; ++i) {
    aA[i] = a_An[M_At->m_a_[i] / lakbcc::POPLENGTH];
    out_a[i] = pick_u(output_spacing_a, i, M_At->m_b_[i], M_At->m_a_[i]);
  }
  for (int k = 0; k < nY; ++k) {
    aY[k] = a_Yn[M_Yt->m_a_[k] / lakbcc::POPLENGTH];
    out_y[k] = pick_u(output_spacing_y, k, M_Yt->m_b_[k], M_Yt->m_a_[k]) * la;
  }
  for (int t = 0; t < nT; ++t) {
    const unsigned tb = M_Tt->m_b_[t], ta = M_Tt->m_a_[t];
    t_rowb[t] = tb;
    out_t[t] = pick_u(output_spacing_t, t, tb, ta) * la * ly;
    hhay[t] = (double)(-M_Tt->cpop_j + 2ll * popcount_bytes_masked(M_Tt->wX + (size_t)tb * M_Tt->mc_length, M_Tt->mc_j, (long)M_Tt->mc_length));
    for (int i = 0; i < nA; ++i)
      hhAy[(size_t)t * nA + i] = (double)(long long)(*lakbcc::L2_get(lf_AtTn, i, M_At->m_b_[i], M_At->m_a_[i], t, tb, ta));
    for (int k = 0; k < nY; ++k)
      hhaY[(size_t)t * nY + k] = (double)(long long)(*lakbcc::L2_get(lf_YtTn, k, M_Yt->m_b_[k], M_Yt->m_a_[k], t, tb, ta));
  }
  AtTYnParams p{};
  Stager st;
  p.At = (const uint8_t *)resident(M_At->wX, (size_t)M_At->rpop_b * M_At->mc_length);
  p.Yt = (const uint8_t *)resident(M_Yt->wX, (size_t)M_Yt->rpop_b * M_Yt->mc_length);
  p.Tt = (const uint8_t *)resident(M_Tt->wX, (size_t)M_Tt->rpop_b * M_Tt->mc_length);
  p.a_row_bytes = p.y_row_bytes = p.t_row_bytes = (long long)M_At->mc_length;
  DBuf d_ar = upload_vec(a_rowb), d_yr = upload_vec(y_rowb), d_tr = upload_vec(t_rowb);
  p.a_rowb = d_ar.as<uint32_t>(); p.y_rowb = d_yr.as<uint32_t>(); p.t_rowb = d_tr.as<uint32_t>();
  p.nA = nA; p.nY = nY;
  DBuf mask = upload_bytes(M_At->mc_j, M_At->mc_length);
  p.mask = mask.as<uint8_t>(); p.P = (int)(M_At->mc_length / kBlockBytes); p.cpop = M_At->cpop_j;
  DBuf d_hAy = upload_vec(hhAy), d_haY = upload_vec(hhaY), d_hay = upload_vec(hhay), d_aA = upload_vec(aA), d_aY = upload_vec(aY);
  DBuf d_oa = upload_vec(out_a), d_oy = upload_vec(out_y), d_ot = upload_vec(out_t);
  p.hhAy = d_hAy.as<double>(); p.hhaY = d_haY.as<double>(); p.hhay = d_hay.as<double>();
  p.aA = d_aA.as<double>(); p.aY = d_aY.as<double>();
  p.out_a = d_oa.as<unsigned long long>(); p.out_y = d_oy.as<unsigned long long>(); p.out_t = d_ot.as<unsigned long long>();
  DBuf d_oa2, d_oy2;
  if (symmetric) {
    // transposed positions: Yt row k as an output row, At row i as a column
    std::vector<unsigned long long> out_a2(nY), out_y2(nA);
    for (int k = 0; k < nY; ++k) out_a2[k] = pick_u(output_spacing_a, k, M_Yt->m_b_[k], M_Yt->m_a_[k]);
    for (int i = 0; i < nA; ++i) out_y2[i] = pick_u(output_spacing_y, i, M_At->m_b_[i], M_At->m_a_[i]) * la;
    d_oa2 = upload_vec(out_a2);
    d_oy2 = upload_vec(out_y2);
    p.symmetric = 1;
    p.out_a2 = d_oa2.as<unsigned long long>();
    p.out_y2 = d_oy2.as<unsigned long long>();
  }
  DBuf d_out;
  if (mo) {
    p.out = mo->d;
  } else {
    d_out = DBuf(length * sizeof(double));
    d_out.zero();
    p.out = d_out.as<double>();
  }
  const size_t smem = (size_t)(kTY_M + kTY_N) * kLd * sizeof(uint32_t);
  dim3 grid((nY + kTY_N - 1) / kTY_N, (nA + kTY_M - 1) / kTY_M, nT);
  st.flush();
  attyn_kernel<<<grid, kTY_T, smem, stream()>>>(p);
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
  if (mo) return (int)length;
  copy_back(out->lf, d_out, length, &fill);
  return (int)length;
}

}  // namespace

extern "C" int wrap_AtTYn_vv__run(int *tidx, void **vpra, pthread_t *thread_in, int output_spacing_a,
                                  int output_spacing_y, int output_spacing_t, M_handle *M_At, M_handle *M_Tt,
                                  M_handle *M_Yt, double *A_ajdk, double *Y_ajdk, L_handle *lf_AtTn,
                                  L_handle *lf_YtTn, L_handle **output_p) {
  LAKGB_PROFILE_CALL("wrap_AtTYn_vv__run");
  (void)tidx; (void)vpra; (void)thread_in;
  return attyn_entry(false, "wrap_AtTYn_vv__run", output_spacing_a, output_spacing_y, output_spacing_t, M_At, M_Tt,
                     M_Yt, A_ajdk, Y_ajdk, lf_AtTn, lf_YtTn, output_p);
}

extern "C" int wrap_AtTAn_vv__run(int *tidx, void **vpra, pthread_t *thread_in, int output_spacing_a,
                                  int output_spacing_y, int output_spacing_t, M_handle *M_At, M_handle *M_Tt,
                                  M_handle *M_Yt, double *A_ajdk, double *Y_ajdk, L_handle *lf_AtTn,
                                  L_handle *lf_YtTn, L_handle **output_AtTAn_p) {
  LAKGB_PROFILE_CALL("wrap_AtTAn_vv__run");
  (void)tidx; (void)vpra; (void)thread_in;
  return attyn_entry(true, "wrap_AtTAn_vv__run", output_spacing_a, output_spacing_y, output_spacing_t, M_At, M_Tt,
                     M_Yt, A_ajdk, Y_ajdk, lf_AtTn, lf_YtTn, output_AtTAn_p);
}
