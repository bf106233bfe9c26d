// Element-wise FP64 loop products, kept as the reference's ground truths for
// the bit-plane and ZtSWn products:
//
// At_T_YnWt_S_Zn_vv (dir_c/At_T_YnWt_S_Zn_vv.c:5-85):
//   out[na, ns] = sum_my (vA - a_An[na]) * vT * I[ns, na, my],
//   I[ns, na, my] = sum_mw YnWt[my, mw] * vS * (vZ - a_An[nz]),
// At row na paired with Zt row nz, vA = At(na, my), vT = Tt(ns, my),
// vS = St(ns, mw), vZ = Zt(nz, mw) as +/-1, both sums in index order.
//
// An_ZtSWn_Yt_vv (dir_c/An_ZtSWn_Yt_vv.c:5-130):
//   out[ma, ns] = sum_ny J[ns, ma, ny],
//   J[ns, ma, ny] = (sum_na (vA - a_An[na]) * D_An[na] * ZtSWn[na, ny, ns]) * (D_Yn[ny] * (vY - a_Yn[ny])),
// An row ma paired with Yn row my, vA = An(ma, na), vY = Yn(my, ny), sums in
// index order.
//
// Each product runs as two kernels: the inner sums, one thread per
// (covariate, output row, outer index) -- the threads of a warp share the
// outer index, so the FP64 matrix element each step reads is a broadcast --
// written to a scratch array laid out [covariate][outer index][row]; then the
// outer sums in order, one thread per (covariate, output row), reading the
// scratch coalesced.  Every operation is the reference's, in its order, with
// separate multiplies and adds.
#include <algorithm>

#include "abi_common.cuh"
#include "bcc_model.h"
#include "lmirror.cuh"

namespace lakgb {

namespace {

__device__ __forceinline__ int bit_pm(const uint8_t *row, unsigned a) {
  return ((row[a >> 3] >> (7 - (a & 7))) & 1) ? 1 : -1;
}

__device__ __forceinline__ unsigned long long pick_d(int s, unsigned long long j, unsigned long long b,
                                                     unsigned long long a) {
  return s == LAKGB_SPACING_j ? j : (s == LAKGB_SPACING_b ? b : a);
}

struct LView {  // an L_handle's addressing on the device
  const double *lf;
  int sr, sc, sl;
  unsigned long long rs, cs;
};

__device__ __forceinline__ double l2(const LView &L, unsigned long long rj, unsigned long long rb,
                                     unsigned long long ra, unsigned long long cj, unsigned long long cb,
                                     unsigned long long ca) {
  return L.lf[pick_d(L.sr, rj, rb, ra) + pick_d(L.sc, cj, cb, ca) * L.rs];
}

__device__ __forceinline__ double l3(const LView &L, unsigned long long rj, unsigned long long rb,
                                     unsigned long long ra, unsigned long long cj, unsigned long long cb,
                                     unsigned long long ca, unsigned long long lj, unsigned long long lb,
                                     unsigned long long la) {
  return L.lf[pick_d(L.sr, rj, rb, ra) + pick_d(L.sc, cj, cb, ca) * L.rs + pick_d(L.sl, lj, lb, la) * L.rs * L.cs];
}

// ---- At_T_YnWt_S_Zn_vv ------------------------------------------------------

struct AtYnWtParams {
  const uint8_t *At; const uint32_t *a_rowb; const uint32_t *a_rowa; long long a_row_bytes;
  const uint8_t *Zt; const uint32_t *z_rowb; const uint32_t *z_rowa; long long z_row_bytes;
  const uint8_t *Tt; const uint8_t *St; const uint32_t *s_rowb; long long t_row_bytes, s_row_bytes;
  int nP, nS;
  const uint32_t *my_a, *my_b; int nMy;   // retained columns of At (patients)
  const uint32_t *mw_a, *mw_b; int nMw;   // retained columns of Zt (controls)
  const double *a_An;
  LView L;                                // YnWt [my, mw]
  double *scratch;                        // [s][my][i]
  const unsigned long long *out_r; const unsigned long long *s_off;
  double *out;
};

__global__ void at_ynwt_inner_kernel(AtYnWtParams p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = blockIdx.z;
  if (i >= p.nP) return;
  const uint8_t *St = p.St + (long long)p.s_rowb[s] * p.s_row_bytes;
  const uint8_t *Zt = p.Zt + (long long)p.z_rowb[i] * p.z_row_bytes;
  const double az = p.a_An[p.z_rowa[i] / lakbcc::POPLENGTH];
  for (int my = blockIdx.y; my < p.nMy; my += gridDim.y) {
    const unsigned ya = p.my_a[my], yb = p.my_b[my];
    double tmp = 0.0;
    for (int mw = 0; mw < p.nMw; ++mw) {
      const unsigned wa = p.mw_a[mw], wb = p.mw_b[mw];
      const int vS = bit_pm(St, wa), vZ = bit_pm(Zt, wa);
      tmp = __dadd_rn(tmp, __dmul_rn(__dmul_rn(l2(p.L, my, yb, ya, mw, wb, wa), (double)vS), __dsub_rn((double)vZ, az)));
    }
    p.scratch[((long long)s * p.nMy + my) * p.nP + i] = tmp;
  }
}

__global__ void at_ynwt_outer_kernel(AtYnWtParams p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = blockIdx.y;
  if (i >= p.nP) return;
  const uint8_t *At = p.At + (long long)p.a_rowb[i] * p.a_row_bytes;
  const uint8_t *Tt = p.Tt + (long long)p.s_rowb[s] * p.t_row_bytes;
  const double aa = p.a_An[p.a_rowa[i] / lakbcc::POPLENGTH];
  double acc = 0.0;
  for (int my = 0; my < p.nMy; ++my) {
    const unsigned ya = p.my_a[my];
    const int vA = bit_pm(At, ya), vT = bit_pm(Tt, ya);
    acc = __dadd_rn(acc, __dmul_rn(__dmul_rn(__dsub_rn((double)vA, aa), (double)vT),
                                   p.scratch[((long long)s * p.nMy + my) * p.nP + i]));
  }
  p.out[p.out_r[i] + p.s_off[s]] = acc;
}

// ---- An_ZtSWn_Yt_vv ---------------------------------------------------------

struct AnZtSWnYtParams {
  const uint8_t *An; const uint32_t *a_rowb; long long a_row_bytes;
  const uint8_t *Yn; const uint32_t *y_rowb; long long y_row_bytes;
  int nP, nS;
  const uint32_t *s_rowj, *s_rowb, *s_rowa;
  const uint32_t *na_a, *na_b; int nNa;   // retained columns of An
  const uint32_t *ny_a, *ny_b; int nNy;   // retained columns of Yn
  const double *a_An, *D_An, *a_Yn, *D_Yn;
  LView L;                                // ZtSWn [na, ny, s]
  double *scratch;                        // [s][ny][i]
  const unsigned long long *out_r; const unsigned long long *s_off;
  double *out;
};

__global__ void an_ztswn_inner_kernel(AnZtSWnYtParams p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = blockIdx.z;
  if (i >= p.nP) return;
  const uint8_t *An = p.An + (long long)p.a_rowb[i] * p.a_row_bytes;
  const uint8_t *Yn = p.Yn + (long long)p.y_rowb[i] * p.y_row_bytes;
  const unsigned sj = p.s_rowj[s], sb = p.s_rowb[s], sa = p.s_rowa[s];
  for (int ny = blockIdx.y; ny < p.nNy; ny += gridDim.y) {
    const unsigned ya = p.ny_a[ny], yb = p.ny_b[ny];
    double tmp = 0.0;
    for (int na = 0; na < p.nNa; ++na) {
      const unsigned xa = p.na_a[na], xb = p.na_b[na];
      const int blk = xa / lakbcc::POPLENGTH;
      const double w = __dmul_rn(__dsub_rn((double)bit_pm(An, xa), p.a_An[blk]), p.D_An[blk]);
      tmp = __dadd_rn(tmp, __dmul_rn(w, l3(p.L, na, xb, xa, ny, yb, ya, sj, sb, sa)));
    }
    const int yblk = ya / lakbcc::POPLENGTH;
    tmp = __dmul_rn(tmp, __dmul_rn(p.D_Yn[yblk], __dsub_rn((double)bit_pm(Yn, ya), p.a_Yn[yblk])));
    p.scratch[((long long)s * p.nNy + ny) * p.nP + i] = tmp;
  }
}

__global__ void an_ztswn_outer_kernel(AnZtSWnYtParams p) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int s = blockIdx.y;
  if (i >= p.nP) return;
  double acc = 0.0;
  for (int ny = 0; ny < p.nNy; ++ny) acc = __dadd_rn(acc, p.scratch[((long long)s * p.nNy + ny) * p.nP + i]);
  p.out[p.out_r[i] + p.s_off[s]] = acc;
}

inline unsigned long long pick_h(int s, unsigned long long j, unsigned long long b, unsigned long long a) {
  return s == LAKGB_SPACING_j ? j : (s == LAKGB_SPACING_b ? b : a);
}

// Device view of an L_handle: its device mirror when it has one, else its
// host values uploaded (kept alive by `buf`).
LView lview(const L_handle *L, DBuf &buf) {
  const double *d = nullptr;
  if (Mirror *m = find_mirror(L)) {
    d = m->d;
  } else {
    buf = upload_bytes(L->lf, L->length * sizeof(double));
    d = buf.as<double>();
  }
  return LView{d, L->spacing_row, L->spacing_col, L->spacing_lyr, L->row_stride, L->col_stride};
}

}  // namespace

}  // namespace lakgb

using namespace lakgb;

extern "C" int wrap_At_T_YnWt_S_Zn_vv__run(int *tidx, void **vpra, pthread_t *thread_in, int output_spacing_a,
                                           int output_spacing_s, M_handle *M_At, M_handle *M_Tt, M_handle *M_St,
                                           M_handle *M_Zt, double *A_ajdk, L_handle *lf_YnWt, L_handle **output_p) {
  LAKGB_PROFILE_CALL("wrap_At_T_YnWt_S_Zn_vv__run");
  (void)tidx; (void)vpra; (void)thread_in;
  const unsigned long long la = spacing_length(output_spacing_a, M_At);
  const unsigned long long ls = spacing_length(output_spacing_s, M_St);
  const unsigned long long length = la * ls;
  L_handle *out = ensure_output(output_p, length, "wrap_At_T_YnWt_S_Zn_vv__run");
  if (!out) return (int)length;
  out->spacing_row = output_spacing_a; out->row_stride = la;
  out->spacing_col = output_spacing_s; out->col_stride = ls;
  const int nP = (int)std::min(M_At->rpop_j, M_Zt->rpop_j), nS = (int)M_St->rpop_j;
  const int nMy = (int)M_At->cpop_j, nMw = (int)M_Zt->cpop_j;
  if (nP == 0 || nS == 0 || !lf_YnWt) return (int)length;
  const int A_pcols = (int)lakbcc::psize(M_At->nrows);
  std::vector<uint32_t> a_rowb(nP), a_rowa(nP), z_rowb(nP), z_rowa(nP), s_rowb(nS);
  std::vector<unsigned long long> out_r(nP), s_off(nS);
  for (int i = 0; i < nP; ++i) {
    a_rowb[i] = M_At->m_b_[i]; a_rowa[i] = M_At->m_a_[i];
    z_rowb[i] = M_Zt->m_b_[i]; z_rowa[i] = M_Zt->m_a_[i];
    out_r[i] = pick_h(output_spacing_a, i, M_At->m_b_[i], M_At->m_a_[i]);
  }
  for (int s = 0; s < nS; ++s) {
    s_rowb[s] = M_St->m_b_[s];
    s_off[s] = pick_h(output_spacing_s, s, M_St->m_b_[s], M_St->m_a_[s]) * la;
  }
  Stager st;
  AtYnWtParams p{};
  p.At = (const uint8_t *)resident(M_At->wX, (size_t)M_At->rpop_b * M_At->mc_length);
  p.Zt = (const uint8_t *)resident(M_Zt->wX, (size_t)M_Zt->rpop_b * M_Zt->mc_length);
  p.Tt = (const uint8_t *)resident(M_Tt->wX, (size_t)M_Tt->rpop_b * M_Tt->mc_length);
  p.St = (const uint8_t *)resident(M_St->wX, (size_t)M_St->rpop_b * M_St->mc_length);
  p.a_row_bytes = (long long)M_At->mc_length; p.z_row_bytes = (long long)M_Zt->mc_length;
  p.t_row_bytes = (long long)M_Tt->mc_length; p.s_row_bytes = (long long)M_St->mc_length;
  DBuf d_ab = upload_vec(a_rowb), d_aa = upload_vec(a_rowa), d_zb = upload_vec(z_rowb), d_za = upload_vec(z_rowa);
  DBuf d_sb = upload_vec(s_rowb), d_or = upload_vec(out_r), d_so = upload_vec(s_off);
  DBuf d_mya = upload_bytes(M_At->n_a_, nMy * sizeof(uint32_t)), d_myb = upload_bytes(M_At->n_b_, nMy * sizeof(uint32_t));
  DBuf d_mwa = upload_bytes(M_Zt->n_a_, nMw * sizeof(uint32_t)), d_mwb = upload_bytes(M_Zt->n_b_, nMw * sizeof(uint32_t));
  DBuf d_aj = upload_bytes(A_ajdk + (size_t)lakbcc::AJDK_1_0 * A_pcols, (size_t)A_pcols * sizeof(double));
  DBuf d_L;
  p.L = lview(lf_YnWt, d_L);
  p.a_rowb = d_ab.as<uint32_t>(); p.a_rowa = d_aa.as<uint32_t>();
  p.z_rowb = d_zb.as<uint32_t>(); p.z_rowa = d_za.as<uint32_t>(); p.s_rowb = d_sb.as<uint32_t>();
  p.nP = nP; p.nS = nS;
  p.my_a = d_mya.as<uint32_t>(); p.my_b = d_myb.as<uint32_t>(); p.nMy = nMy;
  p.mw_a = d_mwa.as<uint32_t>(); p.mw_b = d_mwb.as<uint32_t>(); p.nMw = nMw;
  p.a_An = d_aj.as<double>();
  p.out_r = d_or.as<unsigned long long>(); p.s_off = d_so.as<unsigned long long>();
  DBuf scratch((size_t)nS * std::max(nMy, 1) * nP * sizeof(double));
  DBuf d_out(length * sizeof(double));
  d_out.zero();
  p.scratch = scratch.as<double>();
  p.out = d_out.as<double>();
  st.flush();
  const int T = 128;
  if (nMy > 0) {
    at_ynwt_inner_kernel<<<dim3((nP + T - 1) / T, std::min(nMy, 65535), nS), T, 0, stream()>>>(p);
    LAKGB_CUDA(cudaGetLastError());
  }
  at_ynwt_outer_kernel<<<dim3((nP + T - 1) / T, nS), T, 0, stream()>>>(p);
  LAKGB_CUDA(cudaGetLastError());
  count_launch(nMy > 0 ? 2 : 1);
  copy_back(out->lf, d_out, length);
  return (int)length;
}

extern "C" int wrap_An_ZtSWn_Yt_vv__run(int *tidx, void **vpra, pthread_t *thread_in, int output_spacing_a,
                                        int output_spacing_s, M_handle *M_An, M_handle *M_St, M_handle *M_Yn,
                                        double *A_ajdk, double *Y_ajdk, L_handle *lf_ZtSWn, L_handle **output_p) {
  LAKGB_PROFILE_CALL("wrap_An_ZtSWn_Yt_vv__run");
  (void)tidx; (void)vpra; (void)thread_in;
  const unsigned long long la = spacing_length(output_spacing_a, M_An);
  const unsigned long long ls = spacing_length(output_spacing_s, M_St);
  const unsigned long long length = la * ls;
  L_handle *out = ensure_output(output_p, length, "wrap_An_ZtSWn_Yt_vv__run");
  if (!out) return (int)length;
  out->spacing_row = output_spacing_a; out->row_stride = la;
  out->spacing_col = output_spacing_s; out->col_stride = ls;
  if (!lf_ZtSWn) {
    printf(" %% Warning! lf_ZtSWn==NULL in get_An_ZtSWn_Yt_vv\n");
    return (int)length;
  }
  const int nP = (int)std::min(M_An->rpop_j, M_Yn->rpop_j), nS = (int)M_St->rpop_j;
  const int nNa = (int)M_An->cpop_j, nNy = (int)M_Yn->cpop_j;
  if (nP == 0 || nS == 0) return (int)length;
  const int A_pcols = (int)lakbcc::psize(M_An->ncols), Y_pcols = (int)lakbcc::psize(M_Yn->ncols);
  std::vector<uint32_t> a_rowb(nP), y_rowb(nP), s_rowj(nS), s_rowb(nS), s_rowa(nS);
  std::vector<unsigned long long> out_r(nP), s_off(nS);
  for (int i = 0; i < nP; ++i) {
    a_rowb[i] = M_An->m_b_[i];
    y_rowb[i] = M_Yn->m_b_[i];
    out_r[i] = pick_h(output_spacing_a, i, M_An->m_b_[i], M_An->m_a_[i]);
  }
  for (int s = 0; s < nS; ++s) {
    s_rowj[s] = s; s_rowb[s] = M_St->m_b_[s]; s_rowa[s] = M_St->m_a_[s];
    s_off[s] = pick_h(output_spacing_s, s, M_St->m_b_[s], M_St->m_a_[s]) * la;
  }
  Stager st;
  AnZtSWnYtParams p{};
  p.An = (const uint8_t *)resident(M_An->wX, (size_t)M_An->rpop_b * M_An->mc_length);
  p.Yn = (const uint8_t *)resident(M_Yn->wX, (size_t)M_Yn->rpop_b * M_Yn->mc_length);
  p.a_row_bytes = (long long)M_An->mc_length; p.y_row_bytes = (long long)M_Yn->mc_length;
  DBuf d_ab = upload_vec(a_rowb), d_yb = upload_vec(y_rowb), d_or = upload_vec(out_r), d_so = upload_vec(s_off);
  DBuf d_sj = upload_vec(s_rowj), d_sb = upload_vec(s_rowb), d_sa = upload_vec(s_rowa);
  DBuf d_naa = upload_bytes(M_An->n_a_, nNa * sizeof(uint32_t)), d_nab = upload_bytes(M_An->n_b_, nNa * sizeof(uint32_t));
  DBuf d_nya = upload_bytes(M_Yn->n_a_, nNy * sizeof(uint32_t)), d_nyb = upload_bytes(M_Yn->n_b_, nNy * sizeof(uint32_t));
  DBuf d_aA = upload_bytes(A_ajdk + (size_t)lakbcc::AJDK_1_0 * A_pcols, (size_t)A_pcols * sizeof(double));
  DBuf d_DA = upload_bytes(A_ajdk + (size_t)lakbcc::AJDK_0_1 * A_pcols, (size_t)A_pcols * sizeof(double));
  DBuf d_aY = upload_bytes(Y_ajdk + (size_t)lakbcc::AJDK_1_0 * Y_pcols, (size_t)Y_pcols * sizeof(double));
  DBuf d_DY = upload_bytes(Y_ajdk + (size_t)lakbcc::AJDK_0_1 * Y_pcols, (size_t)Y_pcols * sizeof(double));
  DBuf d_L;
  p.L = lview(lf_ZtSWn, d_L);
  p.a_rowb = d_ab.as<uint32_t>(); p.y_rowb = d_yb.as<uint32_t>();
  p.nP = nP; p.nS = nS;
  p.s_rowj = d_sj.as<uint32_t>(); p.s_rowb = d_sb.as<uint32_t>(); p.s_rowa = d_sa.as<uint32_t>();
  p.na_a = d_naa.as<uint32_t>(); p.na_b = d_nab.as<uint32_t>(); p.nNa = nNa;
  p.ny_a = d_nya.as<uint32_t>(); p.ny_b = d_nyb.as<uint32_t>(); p.nNy = nNy;
  p.a_An = d_aA.as<double>(); p.D_An = d_DA.as<double>(); p.a_Yn = d_aY.as<double>(); p.D_Yn = d_DY.as<double>();
  p.out_r = d_or.as<unsigned long long>(); p.s_off = d_so.as<unsigned long long>();
  DBuf scratch((size_t)nS * std::max(nNy, 1) * nP * sizeof(double));
  DBuf d_out(length * sizeof(double));
  d_out.zero();
  p.scratch = scratch.as<double>();
  p.out = d_out.as<double>();
  st.flush();
  const int T = 128;
  if (nNy > 0) {
    an_ztswn_inner_kernel<<<dim3((nP + T - 1) / T, std::min(nNy, 65535), nS), T, 0, stream()>>>(p);
    LAKGB_CUDA(cudaGetLastError());
  }
  an_ztswn_outer_kernel<<<dim3((nP + T - 1) / T, nS), T, 0, stream()>>>(p);
  LAKGB_CUDA(cudaGetLastError());
  count_launch(nNy > 0 ? 2 : 1);
  copy_back(out->lf, d_out, length);
  return (int)length;
}
