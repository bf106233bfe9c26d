// Reference-compatible C entry points for the bcc kernels.  Each takes the
// reference's host-side M_handle / L_handle structs, moves what the kernel
// needs to the device (bit matrices stay resident between calls), launches the
// sm_103a kernel and writes the result into the caller's L_handle exactly where
// the reference kernel would.
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "gram.cuh"
#include "lakgb_runtime.cuh"
#include "rowvec.cuh"
#include "abi_common.cuh"
#include "lmirror.cuh"

using namespace lakgb;

namespace {

constexpr int kAjdk_0_1 = 5;
constexpr int kAjdk_1_1 = 6;
constexpr int kAjdk_2_1 = 7;

// Host outputs at least this large come back in two parts (gram_entry).
constexpr size_t kSplitDownloadBytes = size_t(8) << 20;

int gram_entry(bool symmetric, int type_flag, int spacing_r, int spacing_c, M_handle *M_An,
               M_handle *M_Zn, double *A_ajdk, L_handle *lf_An_ajdk, L_handle *lf_Zn_ajdk,
               L_handle **out_p, const char *who) {
  const unsigned long long length_r = spacing_length(spacing_r, M_An);
  const unsigned long long length_c = spacing_length(spacing_c, M_Zn);
  const unsigned long long length = length_r * length_c;
  // A mirrored output (lmirror.cu) is produced on the device only.
  Mirror *mo = *out_p ? find_mirror(*out_p) : nullptr;
  L_handle *out = nullptr;
  HostOutputFill fill;
  if (mo) {
    out = *out_p;
    if (out->length < length || mo->n < length) {
      set_error(2, "output length %llu < %llu in %s", out->length, length, who);
      return (int)length;
    }
    if (length) LAKGB_CUDA(cudaMemsetAsync(mo->d, 0, length * sizeof(double), stream()));
    mo->host_stale = true;
  } else {
    out = ensure_output(out_p, length, who, false);
    fill.L = out;
    fill.n = length;
  }
  if (!out) return (int)length;
  out->spacing_row = spacing_r; out->row_stride = length_r;
  out->spacing_col = spacing_c; out->col_stride = length_c;
  if (type_flag == LAKGB_TYPE_p0) {
    printf(" %% Warning! TYPE_p0 not implemented within %s\n", who);
    return (int)length;
  }
  const int P = (int)(M_An->mc_length / kBlockBytes);
  const int nA = (int)M_An->rpop_j, nZ = (int)M_Zn->rpop_j;
  // Column-mask sums (AnZt_vv.c:62-63), host side in block order.
  double a0d1 = 0.0, a2d1 = 0.0;
  for (int nc = 0; nc < P; ++nc) {
    const double c = (double)popcount_bytes(M_An->mc_j + (long)nc * kBlockBytes, kBlockBytes);
    a0d1 += (A_ajdk ? A_ajdk[nc + kAjdk_0_1 * P] : 1.0) * c;
    a2d1 += (A_ajdk ? A_ajdk[nc + kAjdk_2_1 * P] : 0.0) * c;
  }
  if (nA == 0 || nZ == 0 || P == 0) return (int)length;

  Stager st;
  const void *wA = resident(M_An->wX, (size_t)M_An->rpop_b * M_An->mc_length);
  const void *wZ = resident(M_Zn->wX, (size_t)M_Zn->rpop_b * M_Zn->mc_length);
  DBuf mask = upload_bytes(M_An->mc_j, M_An->mc_length);
  std::vector<uint32_t> arow(M_An->m_b_, M_An->m_b_ + nA), zrow(M_Zn->m_b_, M_Zn->m_b_ + nZ);
  DBuf d_arow = upload_vec(arow), d_zrow = upload_vec(zrow);
  const std::vector<uint32_t> outc = spacing_index(spacing_c, M_Zn);
  DBuf d_outr = upload_vec(spacing_index(spacing_r, M_An));
  DBuf d_outc = upload_vec(outc);
  DBuf d_outr2, d_outc2;
  if (symmetric) {
    d_outr2 = upload_vec(spacing_index(spacing_r, M_Zn));
    d_outc2 = upload_vec(spacing_index(spacing_c, M_An));
  }
  DBuf d_D;
  if (A_ajdk) {
    d_D = upload_bytes(A_ajdk + (size_t)kAjdk_0_1 * P, (size_t)P * sizeof(double));
  }
  DBuf d_lfA, d_lfZ;
  if (lf_An_ajdk && lf_Zn_ajdk) {
    std::vector<double> a((size_t)nA), z((size_t)nZ);
    std::vector<uint32_t> ia = spacing_index(lf_An_ajdk->spacing_row, M_An);
    std::vector<uint32_t> iz = spacing_index(lf_Zn_ajdk->spacing_row, M_Zn);
    for (int i = 0; i < nA; ++i) a[i] = lf_An_ajdk->lf[ia[i] + kAjdk_1_1 * lf_An_ajdk->row_stride];
    for (int k = 0; k < nZ; ++k) z[k] = lf_Zn_ajdk->lf[iz[k] + kAjdk_1_1 * lf_Zn_ajdk->row_stride];
    d_lfA = upload_vec(a);
    d_lfZ = upload_vec(z);
  }
  DBuf d_out;
  double *dout = nullptr;
  if (mo) {
    dout = mo->d;
  } else {
    d_out = DBuf(length * sizeof(double));
    d_out.zero();
    dout = d_out.as<double>();
  }

  GramParams p{};
  p.wA = (const uint8_t *)wA; p.a_rowb = d_arow.as<uint32_t>(); p.nA = nA; p.a_row_bytes = (long long)M_An->mc_length;
  p.wZ = (const uint8_t *)wZ; p.z_rowb = d_zrow.as<uint32_t>(); p.nZ = nZ; p.z_row_bytes = (long long)M_Zn->mc_length;
  p.mask = mask.as<uint8_t>(); p.P = P; p.D = d_D.as<double>();
  p.type = (type_flag == LAKGB_TYPE_pm) ? 1 : 2;
  p.a0d1 = a0d1; p.a2d1 = a2d1;
  p.lfA = d_lfA.as<double>(); p.lfZ = d_lfZ.as<double>();
  p.out_r = d_outr.as<uint32_t>(); p.out_c = d_outc.as<uint32_t>();
  p.out_r2 = d_outr2.as<uint32_t>(); p.out_c2 = d_outc2.as<uint32_t>();
  p.out_stride = (long long)length_r; p.out = dout;
  p.symmetric = symmetric ? 1 : 0;
  st.flush();
  // A large host output of a non-symmetric Gram comes back in two parts: the
  // Z rows are split at a multiple of 128 rows (whole tensor-core tiles) into
  // two launches, and the output columns of the first part (a contiguous
  // range: column indices grow with the Z row) are downloaded while the
  // second part computes.  Every element is computed exactly as by one
  // launch.  (A symmetric Gram also writes the mirrored elements, which
  // cross the column split, so it comes back in one piece.)
  const int zsplit = ((nZ / 2) + 127) / 128 * 128;
  if (!mo && !symmetric && length * sizeof(double) >= kSplitDownloadBytes && zsplit > 0 && zsplit < nZ &&
      std::is_sorted(outc.begin(), outc.end())) {
    GramParams q0 = p, q1 = p;
    q0.nZ = zsplit;
    q1.nZ = nZ - zsplit;
    q1.z_rowb = p.z_rowb + zsplit;
    q1.out_c = p.out_c + zsplit;
    if (p.lfZ) q1.lfZ = p.lfZ + zsplit;
    const unsigned long long c_mid = outc[zsplit];  // first output column of the second part
    cudaEvent_t e0;
    LAKGB_CUDA(cudaEventCreateWithFlags(&e0, cudaEventDisableTiming));
    launch_gram(q0);
    LAKGB_CUDA(cudaEventRecord(e0, stream()));
    launch_gram(q1);
    {
      LAKGB_PROFILE_CALL("(copy back + sync)");
      fill.copied = true;
      LAKGB_CUDA(cudaStreamWaitEvent(copy_stream(), e0, 0));
      LAKGB_CUDA(cudaMemcpyAsync(out->lf, dout, c_mid * length_r * sizeof(double), cudaMemcpyDeviceToHost,
                                 copy_stream()));
      LAKGB_CUDA(cudaMemcpyAsync(out->lf + c_mid * length_r, dout + c_mid * length_r,
                                 (length - c_mid * length_r) * sizeof(double), cudaMemcpyDeviceToHost, stream()));
      LAKGB_CUDA(cudaStreamSynchronize(copy_stream()));
      LAKGB_CUDA(cudaStreamSynchronize(stream()));
    }
    LAKGB_CUDA(cudaEventDestroy(e0));
    return (int)length;
  }
  launch_gram(p);
  if (mo) return (int)length;
  copy_back(out->lf, d_out, length, &fill);
  return (int)length;
}

}  // namespace

extern "C" int wrap_AnZt_vv__run(int *tidx, void **vpra, pthread_t *thread_in, int type_flag,
                                 int output_spacing_r, int output_spacing_c, M_handle *M_An,
                                 M_handle *M_Zn, double *A_ajdk, L_handle *lf_An_ajdk,
                                 L_handle *lf_Zn_ajdk, L_handle **output_AnZt_p) {
  LAKGB_PROFILE_CALL("wrap_AnZt_vv__run");
  (void)tidx; (void)vpra; (void)thread_in;
  return gram_entry(false, type_flag, output_spacing_r, output_spacing_c, M_An, M_Zn, A_ajdk,
                    lf_An_ajdk, lf_Zn_ajdk, output_AnZt_p, "wrap_AnZt_vv__run");
}

extern "C" int wrap_AnAt_vv__run(int *tidx, void **vpra, pthread_t *thread_in, int type_flag,
                                 int output_spacing_r, int output_spacing_c, M_handle *M_An,
                                 M_handle *M_Zn, double *A_ajdk, L_handle *lf_An_ajdk,
                                 L_handle *lf_Zn_ajdk, L_handle **output_AnAt_p) {
  LAKGB_PROFILE_CALL("wrap_AnAt_vv__run");
  (void)tidx; (void)vpra; (void)thread_in;
  return gram_entry(true, type_flag, output_spacing_r, output_spacing_c, M_An, M_Zn, A_ajdk,
                    lf_An_ajdk, lf_Zn_ajdk, output_AnAt_p, "wrap_AnAt_vv__run");
}

extern "C" int wrap_An_v__run(int *tidx, void **vpra, pthread_t *thread_in, int type_flag,
                              int output_spacing_r, M_handle *M_An, L_handle **output_An_v_p) {
  LAKGB_PROFILE_CALL("wrap_An_v__run");
  (void)tidx; (void)vpra; (void)thread_in;
  const unsigned long long length = spacing_length(output_spacing_r, M_An);
  L_handle *out = ensure_output(output_An_v_p, length, "wrap_An_v__run");
  if (!out) return (int)length;
  out->spacing_row = output_spacing_r; out->row_stride = length;
  if (type_flag == LAKGB_TYPE_p0) {
    printf(" %% Warning! TYPE_p0 not implemented within get_An_v__run\n");
    return (int)length;
  }
  const int n = (int)M_An->rpop_j;
  if (n == 0) return (int)length;
  const int P = (int)(M_An->mc_length / kBlockBytes);
  Stager st;
  const void *w = resident(M_An->wX, (size_t)M_An->rpop_b * M_An->mc_length);
  DBuf mask = upload_bytes(M_An->mc_j, M_An->mc_length);
  std::vector<uint32_t> rows(M_An->m_b_, M_An->m_b_ + n);
  DBuf d_rows = upload_vec(rows), d_outr = upload_vec(spacing_index(output_spacing_r, M_An));
  st.flush();
  DBuf d_out(length * sizeof(double));
  d_out.zero();
  RowvecParams p{};
  p.w = (const uint8_t *)w; p.rowb = d_rows.as<uint32_t>(); p.n = n; p.row_bytes = (long long)M_An->mc_length;
  p.mask = mask.as<uint8_t>(); p.P = P; p.type = (type_flag == LAKGB_TYPE_pm) ? 1 : 2;
  p.cpop_j = M_An->cpop_j; p.out_r = d_outr.as<uint32_t>(); p.out = d_out.as<double>();
  launch_an_v(p);
  copy_back(out->lf, d_out, length);
  return (int)length;
}

extern "C" int wrap_An_ajdk_v(int *tidx, void **vpra, pthread_t *thread_in, int type_flag,
                              int output_spacing_r, M_handle *M_An, double *A_ajdk,
                              L_handle **output_An_ajdk_p) {
  LAKGB_PROFILE_CALL("wrap_An_ajdk_v");
  (void)tidx; (void)vpra; (void)thread_in;
  const unsigned long long length_r = spacing_length(output_spacing_r, M_An);
  const unsigned long long length = length_r * LAKGB_AJDK_TOT;
  L_handle *out = ensure_output(output_An_ajdk_p, length, "wrap_An_ajdk_v");
  if (!out) return (int)length;
  out->spacing_row = output_spacing_r; out->row_stride = length_r;
  out->spacing_col = LAKGB_SPACING_a; out->col_stride = LAKGB_AJDK_TOT;
  if (type_flag == LAKGB_TYPE_p0) {
    printf(" %% Warning! TYPE_p0 not implemented within get_An_ajdk_v\n");
    return (int)length;
  }
  const int P = (int)(M_An->mc_length / kBlockBytes);
  double base[LAKGB_AJDK_TOT];
  for (int k = 0; k < LAKGB_AJDK_TOT; ++k) {
    double s = 0.0;
    for (int nc = 0; nc < P; ++nc)
      s += A_ajdk[nc + k * P] * (double)popcount_bytes(M_An->mc_j + (long)nc * kBlockBytes, kBlockBytes);
    base[k] = s;
  }
  const int n = (int)M_An->rpop_j;
  if (n == 0) return (int)length;
  Stager st;
  const void *w = resident(M_An->wX, (size_t)M_An->rpop_b * M_An->mc_length);
  DBuf mask = upload_bytes(M_An->mc_j, M_An->mc_length);
  std::vector<uint32_t> rows(M_An->m_b_, M_An->m_b_ + n);
  DBuf d_rows = upload_vec(rows), d_outr = upload_vec(spacing_index(output_spacing_r, M_An));
  DBuf d_ajdk = upload_bytes(A_ajdk, (size_t)P * LAKGB_AJDK_TOT * sizeof(double));
  DBuf d_base = upload_bytes(base, sizeof(base));
  DBuf d_out(length * sizeof(double));
  d_out.zero();
  RowvecParams p{};
  p.w = (const uint8_t *)w; p.rowb = d_rows.as<uint32_t>(); p.n = n; p.row_bytes = (long long)M_An->mc_length;
  p.mask = mask.as<uint8_t>(); p.P = P; p.type = (type_flag == LAKGB_TYPE_pm) ? 1 : 2;
  p.ajdk = d_ajdk.as<double>(); p.base = d_base.as<double>();
  p.out_r = d_outr.as<uint32_t>(); p.out_stride = (long long)length_r; p.out = d_out.as<double>();
  st.flush();
  launch_an_ajdk(p);
  copy_back(out->lf, d_out, length);
  return (int)length;
}
