// The "condense" row strategy's two entry points (GLOBAL_QR_strategy
// "YnWt condense", bcc_lrup_QR_YnWt_stage_2, dir_c/bcc_lrup.c:772-861):
//
//   wrap_M_At_to_L2_run / wrap_M_An_to_L2_run (dir_c/M_Ax_to_L2.c:5-315):
//     a bit matrix expanded into a dense FP64 matrix, each retained entry
//     (b - a_k) * sqrt(d_k) -- b = +1/-1 (TYPE_pm) or 1/0 (TYPE_00), a_k and
//     d_k the column terms A_ajdk of the entry's SNP k -- or plain b without
//     A_ajdk;
//   wrap_AnZt_mm__run (dir_c/AnZt_mm.c:6-109): the FP64 product of two such
//     matrices, C(i,j) = sum_k At(k,i) * Zt(k,j).
//
// The reference computes the product with cblas_dgemm and links GSL's CBLAS
// (-lgslcblas in its makefiles).  That dgemm, for this call (column-major,
// A transposed, B not), forms every element as one running sum from +0 over
// k = 0, 1, ..., K-1 with the product and the sum each rounded once; the
// kernel below keeps exactly that order (__dmul_rn then __dadd_rn, no fused
// multiply-add), so the product matches the reference bit for bit.  It is a
// plain CUDA-core FP64 kernel: the values are arbitrary doubles, so there is
// nothing for the tensor cores, and the FP64 pipe bounds it.
#include <math.h>
#include <stdint.h>

#include <algorithm>
#include <vector>

#include "abi_common.cuh"
#include "bcc_model.h"
#include "lmirror.cuh"

namespace lakgb {

namespace {

struct ToL2Params {
  const uint8_t *rows;          // row data, rpop_b rows of row_bytes
  long long row_bytes;
  const uint32_t *row_b;        // per retained row: its b-index (data row)
  const unsigned long long *out_r;  // per retained row: output row index
  const uint32_t *col_a;        // per retained column: its a-index (bit)
  const unsigned long long *out_c;  // per retained column: output column offset (index * row stride)
  int nr, nc;
  int bits01;                   // 1: values 1/0 (TYPE_00), 0: +1/-1 (TYPE_pm)
  const double *a, *sd;         // centring terms per row (by_row) or per column, or null
  int by_row;
  double *out;
};

// One thread per retained entry, rows fastest: a warp writes consecutive
// output rows (the output's contiguous index when rows are j-spaced).
// Columns stride over blockIdx.y (gridDim.y is at most 65535).
__global__ void m_to_l2_kernel(ToL2Params p) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= p.nr) return;
  const uint8_t *row = p.rows + (long long)p.row_b[r] * p.row_bytes;
  const unsigned long long orow = p.out_r[r];
  for (int c = blockIdx.y; c < p.nc; c += gridDim.y) {
    const uint32_t na = p.col_a[c];
    const int bit = (row[na >> 3] >> (7 - (na & 7))) & 1;
    double v = p.bits01 ? (double)bit : (double)(2 * bit - 1);
    if (p.a) {
      const int k = p.by_row ? r : c;
      v = __dmul_rn(__dsub_rn(v, p.a[k]), p.sd[k]);
    }
    p.out[orow + p.out_c[c]] = v;
  }
}

constexpr int kMmTile = 64, kMmK = 16, kMmThreads = 256;  // 16 x 16 threads, 4 x 4 outputs each

// C(i,j) = sum_k A[k + i*lda] * B[k + j*ldb], k ascending, from +0; thread
// (tx, ty) of a 64 x 64 tile holds rows ty + 16r and columns tx + 16c.
__global__ void __launch_bounds__(kMmThreads) anzt_mm_kernel(const double *__restrict__ A, long long lda,
                                                              const double *__restrict__ B, long long ldb,
                                                              int m, int n, int K, double *__restrict__ C,
                                                              long long ldc) {
  __shared__ double As[kMmK][kMmTile], Bs[kMmK][kMmTile];
  const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
  const int i0 = blockIdx.x * kMmTile, j0 = blockIdx.y * kMmTile;
  double acc[4][4];
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) acc[r][c] = 0.0;
  for (int k0 = 0; k0 < K; k0 += kMmK) {
    const int kn = min(kMmK, K - k0);
    // 16 consecutive k of one column per 16 threads (coalesced reads)
#pragma unroll
    for (int q = 0; q < 4; ++q) {
      const int kk = threadIdx.x & 15, col = (threadIdx.x >> 4) + 16 * q;
      const int i = i0 + col, j = j0 + col;
      As[kk][col] = (kk < kn && i < m) ? A[(long long)(k0 + kk) + (long long)i * lda] : 0.0;
      Bs[kk][col] = (kk < kn && j < n) ? B[(long long)(k0 + kk) + (long long)j * ldb] : 0.0;
    }
    __syncthreads();
    for (int kk = 0; kk < kn; ++kk) {
      double a[4], b[4];
#pragma unroll
      for (int r = 0; r < 4; ++r) a[r] = As[kk][ty + 16 * r];
#pragma unroll
      for (int c = 0; c < 4; ++c) b[c] = Bs[kk][tx + 16 * c];
#pragma unroll
      for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = __dadd_rn(acc[r][c], __dmul_rn(a[r], b[c]));
    }
    __syncthreads();
  }
#pragma unroll
  for (int r = 0; r < 4; ++r)
#pragma unroll
    for (int c = 0; c < 4; ++c) {
      const int i = i0 + ty + 16 * r, j = j0 + tx + 16 * c;
      if (i < m && j < n) C[(long long)i + (long long)j * ldc] = acc[r][c];
    }
}

// Device data of an input L_handle: its mirror when it has one (the values
// live there), else an upload of the host array.
const double *l_input(const L_handle *L, unsigned long long n, DBuf &hold) {
  if (Mirror *m = find_mirror(L)) {
    if (m->n >= n) return m->d;
  }
  hold = upload_bytes(L->lf, n * sizeof(double));
  return hold.as<double>();
}

// M_An_to_L2 (rows = M rows, centring by column) and M_At_to_L2 (rows = M
// rows = SNPs, centring by row): dir_c/M_Ax_to_L2.c:5-100 and :137-280.
int m_to_l2_entry(bool at, const char *who, int type_flag, int spacing_r, int spacing_c, M_handle *M,
                  double *A_ajdk, L_handle **output_L_p) {
  const unsigned long long lr = spacing_length(spacing_r, M);
  unsigned long long lc = 0;
  switch (spacing_c) {
    case LAKGB_SPACING_j: lc = (unsigned long long)M->cpop_j; break;
    case LAKGB_SPACING_b: lc = (unsigned long long)M->cpop_b; break;
    case LAKGB_SPACING_a: lc = (unsigned long long)M->ncols; break;
    default: break;
  }
  const unsigned long long length = lr * lc;
  if (type_flag == LAKGB_TYPE_p0) printf(" %% Warning! TYPE_p0 not implemented within %s\n", who);
  Mirror *mo = *output_L_p ? find_mirror(*output_L_p) : nullptr;
  L_handle *L = nullptr;
  if (mo) {
    L = *output_L_p;
    if (L->length < length || mo->n < L->length) {
      set_error(2, "output length %llu < %llu in %s", L->length, length, who);
      return (int)length;
    }
    // the whole handle is zeroed (L_zero, L_init.c:31), not only the product
    if (L->length) LAKGB_CUDA(cudaMemsetAsync(mo->d, 0, L->length * sizeof(double), stream()));
    mo->host_stale = true;
  } else {
    L = ensure_output(output_L_p, length, who);
    if (!L) return (int)length;
    memset(L->lf, 0, L->length * sizeof(double));
  }
  L->spacing_row = spacing_r; L->row_stride = lr;
  L->spacing_col = spacing_c; L->col_stride = lc;
  L->spacing_lyr = LAKGB_SPACING_b; L->lyr_stride = 0;
  const int nr = (int)M->rpop_j, nc = (int)M->cpop_j;
  if (nr == 0 || nc == 0 || type_flag == LAKGB_TYPE_p0 || length == 0) return (int)length;
  std::vector<uint32_t> row_b(nr), col_a(nc);
  std::vector<unsigned long long> out_r(nr), out_c(nc);
  for (int r = 0; r < nr; ++r) {
    row_b[r] = M->m_b_[r];
    out_r[r] = lakbcc::pick(spacing_r, r, M->m_b_[r], M->m_a_[r]);
  }
  for (int c = 0; c < nc; ++c) {
    col_a[c] = M->n_a_[c];
    out_c[c] = lakbcc::pick(spacing_c, c, M->n_b_[c], M->n_a_[c]) * lr;
  }
  std::vector<double> a, sd;
  if (A_ajdk) {
    // the SNP of an entry is its row (At) or its column (An)
    const int pcols = (int)lakbcc::psize(at ? M->nrows : M->ncols);
    const int n = at ? nr : nc;
    a.resize(n);
    sd.resize(n);
    for (int k = 0; k < n; ++k) {
      const unsigned snp = at ? M->m_a_[k] : M->n_a_[k];
      a[k] = A_ajdk[snp / lakbcc::POPLENGTH + (size_t)lakbcc::AJDK_1_0 * pcols];
      sd[k] = sqrt(A_ajdk[snp / lakbcc::POPLENGTH + (size_t)lakbcc::AJDK_0_1 * pcols]);
    }
  }
  Stager st;
  ToL2Params p{};
  p.rows = (const uint8_t *)resident(M->wX, (size_t)M->rpop_b * M->mc_length);
  p.row_bytes = (long long)M->mc_length;
  DBuf d_rb = upload_vec(row_b), d_or = upload_vec(out_r), d_ca = upload_vec(col_a), d_oc = upload_vec(out_c);
  DBuf d_a, d_sd;
  if (A_ajdk) {
    d_a = upload_vec(a);
    d_sd = upload_vec(sd);
    p.a = d_a.as<double>();
    p.sd = d_sd.as<double>();
  }
  p.row_b = d_rb.as<uint32_t>(); p.out_r = d_or.as<unsigned long long>();
  p.col_a = d_ca.as<uint32_t>(); p.out_c = d_oc.as<unsigned long long>();
  p.nr = nr; p.nc = nc;
  p.bits01 = type_flag == LAKGB_TYPE_00;
  p.by_row = at;
  DBuf d_out;
  if (mo) {
    p.out = mo->d;
  } else {
    d_out = DBuf(length * sizeof(double));
    d_out.zero();
    p.out = d_out.as<double>();
  }
  st.flush();
  m_to_l2_kernel<<<dim3((nr + 127) / 128, std::min(nc, 65535)), 128, 0, stream()>>>(p);
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
  if (!mo) copy_back(L->lf, d_out, length);
  return (int)length;
}

}  // namespace
}  // namespace lakgb

using namespace lakgb;

extern "C" int wrap_M_At_to_L2_run(int *tidx, void **vpra, pthread_t *thread_in, int type_flag, int output_spacing_r,
                                   int output_spacing_c, M_handle *M_At, double *A_ajdk, L_handle **output_L_p) {
  LAKGB_PROFILE_CALL("wrap_M_At_to_L2_run");
  (void)tidx; (void)vpra; (void)thread_in;
  return m_to_l2_entry(true, "wrap_M_At_to_L2_run", type_flag, output_spacing_r, output_spacing_c, M_At, A_ajdk,
                       output_L_p);
}

extern "C" int wrap_M_An_to_L2_run(int *tidx, void **vpra, pthread_t *thread_in, int type_flag, int output_spacing_r,
                                   int output_spacing_c, M_handle *M_An, double *A_ajdk, L_handle **output_L_p) {
  LAKGB_PROFILE_CALL("wrap_M_An_to_L2_run");
  (void)tidx; (void)vpra; (void)thread_in;
  return m_to_l2_entry(false, "wrap_M_An_to_L2_run", type_flag, output_spacing_r, output_spacing_c, M_An, A_ajdk,
                       output_L_p);
}

extern "C" int wrap_AnZt_mm__run(int *tidx, void **vpra, pthread_t *thread_in, L_handle *lf_At, L_handle *lf_Zt,
                                 L_handle **output_AnZt_p) {
  LAKGB_PROFILE_CALL("wrap_AnZt_mm__run");
  (void)tidx; (void)vpra; (void)thread_in;
  const unsigned long long m = lf_At->col_stride, n = lf_Zt->col_stride, K = lf_At->row_stride;
  const unsigned long long length = m * n;
  Mirror *mo = *output_AnZt_p ? find_mirror(*output_AnZt_p) : nullptr;
  L_handle *out = nullptr;
  HostOutputFill fill;
  if (mo) {
    out = *output_AnZt_p;
    if (out->length < length || mo->n < length) {
      set_error(2, "output length %llu < %llu in wrap_AnZt_mm__run", out->length, length);
      return (int)length;
    }
    if (length) LAKGB_CUDA(cudaMemsetAsync(mo->d, 0, length * sizeof(double), stream()));
    mo->host_stale = true;
  } else {
    out = ensure_output(output_AnZt_p, length, "wrap_AnZt_mm__run", false);
    if (!out) return (int)length;
    fill.L = out;
    fill.n = length;
  }
  out->spacing_row = lf_At->spacing_col; out->row_stride = m;
  out->spacing_col = lf_Zt->spacing_col; out->col_stride = n;
  if (K == 0 || m == 0 || n == 0 || lf_Zt->row_stride == 0) return (int)length;
  // Every column of Zt must hold the K values the product reads (the
  // reference reads K values from each column of ldb = Zt's row stride).
  if (lf_Zt->row_stride < K) {
    set_error(4, "wrap_AnZt_mm__run: Zt has %llu rows per column, fewer than At's %llu",
              lf_Zt->row_stride, K);
    return (int)length;
  }
  if (m > (unsigned long long)INT32_MAX || n > (unsigned long long)INT32_MAX || K > (unsigned long long)INT32_MAX ||
      (m + kMmTile - 1) / kMmTile > 0x7fffffffull || (n + kMmTile - 1) / kMmTile > 65535ull) {
    set_error(4, "wrap_AnZt_mm__run: %llu x %llu x %llu is beyond the kernel's grid", m, n, K);
    return (int)length;
  }
  Stager st;
  DBuf hold_a, hold_b, d_out;
  const double *A = l_input(lf_At, K * m, hold_a);
  const double *B = l_input(lf_Zt, lf_Zt->row_stride * n, hold_b);
  double *C = nullptr;
  if (mo) {
    C = mo->d;
  } else {
    d_out = DBuf(length * sizeof(double));
    C = d_out.as<double>();
  }
  st.flush();
  const dim3 grid((unsigned)((m + kMmTile - 1) / kMmTile), (unsigned)((n + kMmTile - 1) / kMmTile));
  anzt_mm_kernel<<<grid, kMmThreads, 0, stream()>>>(A, (long long)K, B, (long long)lf_Zt->row_stride, (int)m, (int)n,
                                                    (int)K, C, (long long)m);
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
  if (!mo) copy_back(out->lf, d_out, length, &fill);
  return (int)length;
}
