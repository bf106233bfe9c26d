// bcc solve for the YnWt row/column strategies (lakcluster_driver,
// dir_c/lakcluster_driver.c:14-251), restated over the reference data model.
//
// Every heavy product goes through the reference-compatible kernel entry
// points (wrap_AnZt_vv__run, wrap_xcalc, wrap_At_T_YnWt_S_Zn_ww__run, ...),
// which this library implements on the GPU.  The remaining per-row and
// per-column FP64 bookkeeping (corrections for collapsed loops, score
// normalisation, the tie-ordered sort and the elimination schedule) is
// evaluated here in exactly the reference's operation order so that the
// elimination trace is bit-identical.  Host code must be compiled without
// FP contraction.
//
// Scope of this restatement: no extra column blocks (Y/W absent); covariate
// matrices T / S of any width (one column of ones when absent) with every
// covariate column retained, and the MDS correction of bcc_sumscores_ifT;
// any GLOBAL_Ireq (the per-bin normalisation, sort and selection of
// bcc_sumscores_nrm/srt/xij when it is positive).  Other settings are
// rejected with an error rather than computed differently.
#include "bcc_driver.h"
#include "bcc_sort.h"

#include <math.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <memory>
#include <thread>

namespace lakbcc {

namespace {

int g_tidx = 0;
void *g_vpra[128];
pthread_t g_thread;
#define TARGS &g_tidx, g_vpra, &g_thread

// Optional wall-clock profile per stage (LAKBCC_PROFILE=1): printed to
// stderr when the solve ends.
struct StageClock {
  bool on = false;
  std::chrono::steady_clock::time_point last;
  std::vector<std::pair<std::string, double>> acc;
  void tick(const char *stage) {
    if (!on) return;
    const auto now = std::chrono::steady_clock::now();
    const double dt = std::chrono::duration<double>(now - last).count();
    last = now;
    for (auto &kv : acc)
      if (kv.first == stage) { kv.second += dt; return; }
    acc.emplace_back(stage, dt);
  }
};
thread_local StageClock g_clock;

// ---------------------------------------------------------------------------
// State (the subset of bcc_ajdk / bcc_single / bcc_double used on this path)

struct Single {
  int nb = 0;
  int A_nrows = 0, A_rbother = 0;
  long A_mr_length = 0;
  std::vector<unsigned char> A_bmr_b, A_bmr_j, A_bmr_j_rmv, A_bmr_j_rtn;
  std::vector<unsigned char> A_umr_j, A_umr_j_rmv, A_umr_j_rtn;
  unsigned A_rpop_b = 0, A_rpop_j = 0, A_rpop_j_rmv = 0, A_rpop_j_rtn = 0;
  int Z_nrows = 0, Z_rbother = 0;
  long Z_mr_length = 0;
  std::vector<unsigned char> Z_bmr_b, Z_bmr_j;
  unsigned Z_rpop_b = 0, Z_rpop_j = 0;
  // packed data
  std::vector<unsigned char> An_w, At_w, Zn_w, Zt_w, Tn_w, Tt_w, Sn_w, St_w;
  MH *M_An = nullptr, *M_At = nullptr, *M_Zn = nullptr, *M_Zt = nullptr;
  MH *M_Tn = nullptr, *M_Tt = nullptr, *M_Sn = nullptr, *M_St = nullptr;
  MH *M_an = nullptr, *M_at = nullptr, *M_jn = nullptr, *M_jt = nullptr, *M_kn = nullptr, *M_kt = nullptr;
  MH *M_hn = nullptr, *M_ht = nullptr, *M_zn = nullptr, *M_zt = nullptr, *M_vn = nullptr, *M_vt = nullptr;
  MH *M_tt = nullptr, *M_rt = nullptr, *M_1 = nullptr;
  MH *M_An_a1d1 = nullptr, *M_a2d2_ZtSn = nullptr, *M_a2d2_AtTn = nullptr;
  L_handle *lf_At_rsum = nullptr, *lf_Zt_rsum = nullptr;
  L_handle *lf_An_ajdk = nullptr, *lf_Zn_ajdk = nullptr, *lf_AtTn = nullptr, *lf_ZtSn = nullptr;
  L_handle *lf_jn_ajdk = nullptr, *lf_vn_ajdk = nullptr, *lf_kn_ajdk = nullptr, *lf_zn_ajdk = nullptr;
  // dense removed columns of the condense row strategy (SNPs x rows)
  L_handle *lf_jn = nullptr, *lf_vn = nullptr;
  L_handle *lf_hn_ajdk = nullptr, *lf_an_ajdk = nullptr;
  L_handle *lf_attn = nullptr, *lf_jttn = nullptr, *lf_ktrn = nullptr, *lf_htrn = nullptr;
  L_handle *lf_ztsn = nullptr, *lf_vtsn = nullptr, *lf_ztsvn = nullptr, *lf_attjn = nullptr, *lf_ktrhn = nullptr;
  L_handle *lf_a1d2_Zt_Sn, *lf_a2d2_Zt_Sn, *lf_a3d2_Zt_Sn, *lf_a1d2_At_Tn, *lf_a2d2_At_Tn, *lf_a3d2_At_Tn;
  L_handle *lf_et_Tn, *lf_et_Sn, *lf_et_An, *lf_a1d1_At_en, *lf_a1d2_At_en, *lf_a3d2_At_en;
  L_handle *lf_et_An_a1d1, *lf_Tt_An_a1d1, *lf_T_AnAt_AnAt;
  L_handle *lf_An_a1d1 = nullptr, *lf_At_An_a1d1 = nullptr, *lf_a2d2_ZtSn = nullptr, *lf_a2d2_AtTn = nullptr;
  // SNP x SNP x covariate products of the ZtSWn column strategy
  L_handle *lf_AtTAn = nullptr, *lf_ZtSZn = nullptr, *lf_ktrkn = nullptr;
  // dexcluster single-study terms (dcc_single_init_lf, dir_c/dcc.c:667-725)
  L_handle *lf_A_a0d1 = nullptr, *lf_A_a2d1 = nullptr, *lf_a1d1_ZtSn = nullptr, *lf_a1d1_AtTn = nullptr;
  L_handle *lf_a0d1_ZtSn = nullptr, *lf_a0d1_AtTn = nullptr;
  MH *M_a0d1_ZtSn = nullptr, *M_a0d1_AtTn = nullptr;
  std::vector<double> QR_AnZtSZnAt_nrm, QR_AnAtTAnAt_nrm;
  std::vector<int> QR_index_global_mr_a, QR_index_global_mr_b, QR_index_global_mr_j;
};

struct Double {
  int nb1 = 0, nb2 = 0;
  // dexcluster bin-pair terms (dcc_double_init_lf, dir_c/dcc.c:775-828)
  L_handle *lf_An_a0d1_ZtSn = nullptr, *lf_An_a0d1_AtTn = nullptr, *lf_TAnZtS_ww = nullptr, *lf_TAnAtT_ww = nullptr;
  L_handle *lf_D_AtTn_ZtSn_vv = nullptr, *lf_D_AtTn_AtTn_vv = nullptr;
  L_handle *lf_AnZt = nullptr, *lf_AnAt = nullptr;
  MH *M_AnZt = nullptr, *M_AnAt = nullptr;
  int M_AnZt_trm = 0, M_AnAt_trm = 0;
  L_handle *lf_jnvt = nullptr, *lf_jnjt = nullptr;
  L_handle *lf_knzt = nullptr, *lf_hnvt = nullptr, *lf_ankt = nullptr, *lf_knat = nullptr, *lf_knkt = nullptr;
  MH *M_knzt = nullptr, *M_hnvt = nullptr, *M_ankt = nullptr, *M_knkt = nullptr;
  int M_knzt_trm = 0, M_hnvt_trm = 0, M_ankt_trm = 0, M_knkt_trm = 0;
  L_handle *lf_kt_r_knzt_s_zn, *lf_kt_r_hnvt_s_zn, *lf_at_t_ankt_r_kn, *lf_kt_r_knat_t_an, *lf_kt_r_knkt_r_kn;
  L_handle *lf_attjn____vtszn, *lf_attjn____jttan, *lf_attjn____htrkn, *lf_ktrhn____jttan, *lf_ktrhn____htrkn;
  L_handle *lf_AnZt_S_ZnAt, *lf_AnAt_T_AnAt;
  L_handle *lf_At_T_AnZt_S_Zn, *lf_At_T_AnAt_T_An;
  L_handle *lf_AtTAn____ZtSZn = nullptr, *lf_AtTAn____AtTAn = nullptr;  // ZtSWn column strategy
  L_handle *lf_An_a2d2_Zt_Sn, *lf_An_a2d2_At_Tn;
  L_handle *QR_AnZtSZnAt, *QR_AnAtTAnAt, *QC_AtTAnZtSZn, *QC_AtTAnAtTAn;
};

struct State {
  Params P;
  int nbins = 0;
  int A_ncols = 0, A_cbother = 0, A_pcols = 0;
  long A_mc_length = 0;
  std::vector<unsigned char> A_bmc_b, A_bmc_j, A_bmc_j_rmv, A_bmc_j_rtn;
  std::vector<unsigned char> A_umc_j, A_umc_j_rmv, A_umc_j_rtn;
  unsigned A_cpop_b = 0, A_cpop_j = 0, A_cpop_j_rmv = 0, A_cpop_j_rtn = 0;
  int T_ncols = 1;
  long T_mc_length = 0;
  std::vector<unsigned char> T_bmc_b, T_bmc_j;
  unsigned T_cpop_b = 0, T_cpop_j = 0;
  int A_nrows_total = 0; unsigned A_rpop_b_total = 0, A_rpop_j_total = 0;
  int Z_nrows_total = 0; unsigned Z_rpop_b_total = 0, Z_rpop_j_total = 0;
  std::vector<double> AZ_rsum, A_p, A_ajdk;
  std::vector<double> QC_AtTAnZtSZn_nrm, QC_AtTAnAtTAn_nrm;
  std::vector<double> QC_svalue, QR_svalue;
  std::vector<int> QC_index_local_mc_a, QC_index_local_mc_b, QC_index_local_mc_j;
  std::vector<int> QR_index_local_mr_a, QR_index_local_mr_b, QR_index_local_mr_j, QR_index_local_nb;
  std::vector<int> QR_index_global_mr_a, QR_index_global_mr_b, QR_index_global_mr_j;
  int Irem = 0, Ireq = 0;
  std::vector<std::unique_ptr<Single>> E;
  std::vector<std::unique_ptr<Double>> F;  // F[nb1 + nb2*nbins]
  std::vector<MH *> all_mh;
  std::vector<L_handle *> all_lh;
  Output *out = nullptr;

  const Hooks *hooks = nullptr;

  Double *f(int nb1, int nb2) { return F[nb1 + nb2 * nbins].get(); }
  L_handle *L(unsigned long long n) { L_handle *h = lh_make(n); all_lh.push_back(h); return h; }
  MH *keep(MH *m) { all_mh.push_back(m); return m; }
  void release(L_handle *L) {
    if (L && hooks && hooks->release_L) hooks->release_L(L);
  }
  void forget(const std::vector<unsigned char> &v) {
    if (!v.empty() && hooks && hooks->forget_host) hooks->forget_host(v.data());
  }
  std::vector<L_handle *> mirrored;
  void mirror(L_handle *L) {
    if (!hooks || !hooks->L_mirror || !L) return;
    if (std::find(mirrored.begin(), mirrored.end(), L) != mirrored.end()) return;
    hooks->L_mirror(L);
    mirrored.push_back(L);
  }
  // Mirror a freshly allocated (all-zero) L without uploading it.
  void mirror_zero(L_handle *L) {
    if (!hooks || !hooks->L_mirror || !L) return;
    if (std::find(mirrored.begin(), mirrored.end(), L) != mirrored.end()) return;
    if (hooks->L_mirror_zero)
      hooks->L_mirror_zero(L);
    else
      hooks->L_mirror(L);
    mirrored.push_back(L);
  }
  void to_host(L_handle *L) {
    if (hooks && hooks->L_to_host && L) hooks->L_to_host(L);
  }
  void sub(L_handle *dst, const L_handle *src) {
    if (hooks && hooks->L_sub) { hooks->L_sub(dst, src); return; }
    for (unsigned long long i = 0; i < dst->length; ++i) dst->lf[i] -= src->lf[i];
  }
  void defer_begin() {
    if (hooks && hooks->defer_begin) hooks->defer_begin();
  }
  void defer_end() {
    if (hooks && hooks->defer_end) hooks->defer_end();
  }
  void transpose(L_handle *dst, const L_handle *src) {
    if (hooks && hooks->L_transpose) { hooks->L_transpose(dst, src); return; }
    lh_transpose(dst, src);
  }
  ~State() {
    if (hooks && hooks->L_release_mirror)
      for (L_handle *L : mirrored) hooks->L_release_mirror(L);
    // Outputs the kernel entry points allocated on first use.
    for (auto &E : this->E) {
      for (L_handle *L : {E->lf_An_ajdk, E->lf_Zn_ajdk, E->lf_AtTn, E->lf_ZtSn, E->lf_jn_ajdk, E->lf_vn_ajdk,
                          E->lf_kn_ajdk, E->lf_zn_ajdk, E->lf_hn_ajdk, E->lf_an_ajdk, E->lf_attn, E->lf_jttn,
                          E->lf_ktrn, E->lf_htrn, E->lf_ztsn, E->lf_vtsn, E->lf_ztsvn, E->lf_attjn, E->lf_ktrhn,
                          E->lf_At_An_a1d1, E->lf_AtTAn, E->lf_ZtSZn, E->lf_ktrkn})
        release(L);
      for (auto *v : {&E->An_w, &E->At_w, &E->Zn_w, &E->Zt_w, &E->Tn_w, &E->Tt_w, &E->Sn_w, &E->St_w}) forget(*v);
    }
    for (auto *m : all_mh) { forget(m->own_rows); delete m; }
    for (auto *h : all_lh) lh_free(h);
  }
};

// ---------------------------------------------------------------------------
// small reference helpers restated

void ura_from_bits(std::vector<unsigned char> &u, const std::vector<unsigned char> &b, int n) {
  for (int i = 0; i < n; ++i) u[i] = (unsigned char)bget_on(b.data(), i);
}
void bits_from_ura(std::vector<unsigned char> &b, const std::vector<unsigned char> &u, int n) {
  std::fill(b.begin(), b.end(), 0);
  for (int i = 0; i < n; ++i)
    if (u[i] > 0) bset_on(b.data(), i);
}

// get_xdrop, dir_c/xdrop.c:5-64
void get_xdrop(const Params &P, double lrij, double lcij, int *rdrop_p, int *cdrop_p) {
  if (lrij > lcij) { get_xdrop(P, lcij, lrij, cdrop_p, rdrop_p); return; }
  const double dbl1 = 1.000000 - 0.000001;
  const double gamma = P.gamma;
  double gamma_tmp_row = 0, ammag_tmp_row = 0, gamma_tmp_col = 0, ammag_tmp_col = 0;
  int rdrop = 0, cdrop = 0;
  if (lrij <= 2) {
    rdrop = (int)lrij; cdrop = (int)lcij;
  } else {
    if (gamma > 0) {
      gamma_tmp_row = std::max(gamma, dbl1 / std::max(1.0, lrij));
      ammag_tmp_row = std::min(1 - gamma, (lrij - 1) / std::max(1.0, lrij));
    } else {
      gamma_tmp_row = dbl1 / std::max(1.0, lrij);
      ammag_tmp_row = (lrij - 1) / std::max(1.0, lrij);
    }
    switch (P.gamma_type) {
      case 0: ammag_tmp_col = exp(log(ammag_tmp_row) * log(lcij) / std::max(1.0, log(std::max(1.0, lrij)))); break;
      case 1: ammag_tmp_col = sqrt(ammag_tmp_row * lrij) * sqrt(lcij) / std::max(1.0, sqrt(std::max(1.0, lrij))) /
                              ((double)std::max(1.0, lcij)); break;
      case 2: ammag_tmp_col = ammag_tmp_row; break;
      case 3: ammag_tmp_col = 0; break;
      default: break;
    }
    gamma_tmp_col = dbl1 - ammag_tmp_col;
    rdrop = (int)ceil(gamma_tmp_row * lrij);
    cdrop = (int)ceil(gamma_tmp_col * lcij);
    if (P.gamma_type == 3) cdrop = 0;
  }
  rdrop = (int)std::min((double)rdrop, lrij);
  cdrop = (int)std::min((double)cdrop, lcij);
  if (rdrop_p) *rdrop_p = rdrop;
  if (cdrop_p) *cdrop_p = cdrop;
}

// ---------------------------------------------------------------------------
// load (bcc_load, dir_c/bcc.c:1482-1540 and the functions it calls)

// rows: a-space rows of a (nrows x ncols) matrix, bsize(ncols) bytes each.
// Returns the compacted-by-mask rows (M_handle_v_make / M_load semantics).
std::vector<unsigned char> compact_rows(const std::vector<unsigned char> &rows, int nrows, long row_bytes,
                                        const std::vector<unsigned char> &mr_b) {
  std::vector<unsigned char> out;
  out.reserve(rows.size());
  for (int r = 0; r < nrows; ++r)
    if (bget_on(mr_b.data(), r)) out.insert(out.end(), rows.begin() + (long)r * row_bytes, rows.begin() + (long)(r + 1) * row_bytes);
  out.resize(out.size() + POPLENGTH / BIT8, 0);  // one block of slack (see mh_init)
  return out;
}

// Transpose a-space rows (nrows x ncols) into a-space rows of the transpose,
// 8 x 8 bit blocks at a time (byte k of row r holds columns 8k..8k+7,
// most significant bit first).
inline uint64_t transpose8(uint64_t x) {
  // Bit-matrix transpose of an 8 x 8 block held one row per byte (row i in
  // byte i, column j in bit 7-j): three rounds of block swaps.
  uint64_t t;
  t = (x ^ (x >> 7)) & 0x00AA00AA00AA00AAull; x = x ^ t ^ (t << 7);
  t = (x ^ (x >> 14)) & 0x0000CCCC0000CCCCull; x = x ^ t ^ (t << 14);
  t = (x ^ (x >> 28)) & 0x00000000F0F0F0F0ull; x = x ^ t ^ (t << 28);
  return x;
}

// Column blocks [k0, k1) of transpose_rows, in tiles of 64 x 64 bytes (512
// rows x 512 columns) so that the rows read and the columns written stay in
// cache while a tile is done.
void transpose_tiles(const unsigned char *rows, unsigned char *t, int nrows, int ncols, long rb, long tb, int k0,
                     int k1) {
  const int rblocks = (nrows + 7) / 8;
  for (int kb = k0; kb < k1; kb += 64)
    for (int ib = 0; ib < rblocks; ib += 64) {
      const int ke = std::min(k1, kb + 64), ie = std::min(rblocks, ib + 64);
      for (int i = ib; i < ie; ++i)
        for (int k = kb; k < ke; ++k) {
          uint64_t x = 0;
          for (int q = 0; q < 8; ++q) {
            const int r = 8 * i + q;
            const uint64_t byte = r < nrows ? rows[(size_t)r * rb + k] : 0;
            x |= byte << (8 * (7 - q));
          }
          if (!x) continue;
          x = transpose8(x);
          for (int q = 0; q < 8; ++q) {
            const int c = 8 * k + q;
            if (c < ncols) t[(size_t)c * tb + i] = (unsigned char)(x >> (8 * (7 - q)));
          }
        }
    }
}

// The bit transpose of a packed row-major matrix (8 x 8 blocks).  Matrices of
// 64 MB or more are split over up to 8 host threads by column blocks (each
// writes its own output rows).
std::vector<unsigned char> transpose_rows(const std::vector<unsigned char> &rows, int nrows, int ncols) {
  const long rb = bsize(ncols), tb = bsize(nrows);
  std::vector<unsigned char> t((size_t)std::max(1, ncols) * (size_t)tb, 0);
  const int cblocks = (ncols + 7) / 8;
  const int nth = (size_t)nrows * (size_t)rb >= (size_t(64) << 20)
                      ? (int)std::max(1u, std::min(8u, std::thread::hardware_concurrency()))
                      : 1;
  if (nth <= 1) {
    transpose_tiles(rows.data(), t.data(), nrows, ncols, rb, tb, 0, cblocks);
    return t;
  }
  const int per = ((cblocks + nth - 1) / nth + 63) / 64 * 64;
  std::vector<std::thread> th;
  for (int k0 = 0; k0 < cblocks; k0 += per)
    th.emplace_back(transpose_tiles, rows.data(), t.data(), nrows, ncols, rb, tb, k0, std::min(cblocks, k0 + per));
  for (auto &x : th) x.join();
  return t;
}

// GLOBAL_TEST_TYPE dexcluster_driver: the dcc method (dir_c/dexcluster_driver.c)
// on the same state.
bool dcc_mode(const Params &P) { return P.test_type.rfind("dexcluster", 0) == 0; }

// GLOBAL_QR_strategy / GLOBAL_QC_strategy (substrings, as the reference tests
// them with strstr).  Rows: "YnWt", optionally "condense" (lrup_QR_condense).
// Columns: "YnWt" and / or "ZtSWn"; "store one" loops the covariates one at a
// time through one-covariate forms of the same products (AttYn_vv,
// AttYn____WtsZn_vv, bcc_lrup.c:483-590) to save host memory: each product
// element is the same sum in the same order as in "store all", so the
// store-all stages give its results and it needs nothing else here.
bool qr_condense(const Params &P) { return P.QR_strategy.find("condense") != std::string::npos; }
bool strategies_supported(const Params &P) {
  return P.QR_strategy.find("YnWt") != std::string::npos && P.QR_strategy.find("ZtSWn") == std::string::npos &&
         (P.QC_strategy.find("YnWt") != std::string::npos || P.QC_strategy.find("ZtSWn") != std::string::npos);
}
const char *const kStrategyError =
    "supported strategies: rows YnWt (optionally condense); columns YnWt and / or ZtSWn";

// n1b_cap / n2b_cap (default n1b / n2b): the largest counts the planes must
// hold, when more rows can be removed in one step than the transposition
// flag was chosen for.
MH *xcalc_out(State &S, int n1a, int n1b, int n2a, int n2b, int *trm, int n1b_cap = -1, int n2b_cap = -1) {
  // bcc_double_init_lf_excerpt / M_handle_w_make (bcc.c:992-1003, M_init.c:418-430)
  if (n1b_cap < 0) n1b_cap = n1b;
  if (n2b_cap < 0) n2b_cap = n2b;
  int nrows_bZ, ncols_tmp;
  if (n2b <= n1b) { *trm = 0; nrows_bZ = n1a; ncols_tmp = n2b_cap; }
  else { *trm = 1; nrows_bZ = n2a; ncols_tmp = n1b_cap; }
  const int ncols_bZ = (1 + S.P.B_MLT) * ncols_tmp;
  return S.keep(mh_make_owned(ncols_bZ, nrows_bZ));
}

int load(State &S, const Input &I, std::string &err) {
  const Params &P = S.P;
  S.nbins = (int)I.bins.size();
  if (S.nbins <= 0) { err = "NBINS must be positive"; return 2; }
  // bcc_ajdk_load (bcc.c:54-115)
  S.A_ncols = I.ncols;
  S.A_cbother = S.A_ncols > 0;
  S.A_mc_length = bsize(S.A_ncols);
  S.A_bmc_b.assign(S.A_mc_length, 0);
  if (!I.mc_b.empty()) memcpy(S.A_bmc_b.data(), I.mc_b.data(), std::min<size_t>(I.mc_b.size(), S.A_mc_length));
  else for (int c = 0; c < S.A_ncols; ++c) bset_on(S.A_bmc_b.data(), c);
  S.A_bmc_j = S.A_bmc_b;
  S.A_bmc_j_rmv.assign(S.A_mc_length, 0);
  S.A_bmc_j_rtn.assign(S.A_mc_length, 0);
  S.A_cpop_b = popcount_bytes(S.A_bmc_b.data(), S.A_mc_length);
  S.A_cpop_j = popcount_bytes(S.A_bmc_j.data(), S.A_mc_length);
  S.A_umc_j.assign(std::max(1, S.A_ncols), 0);
  S.A_umc_j_rmv.assign(std::max(1, S.A_ncols), 0);
  S.A_umc_j_rtn.assign(std::max(1, S.A_ncols), 0);
  ura_from_bits(S.A_umc_j, S.A_bmc_j, S.A_ncols);
  S.T_ncols = I.T_ncols;
  S.T_mc_length = bsize(S.T_ncols);
  S.T_bmc_b.assign(S.T_mc_length, 0);
  for (int c = 0; c < S.T_ncols; ++c) bset_on(S.T_bmc_b.data(), c);
  S.T_bmc_j = S.T_bmc_b;
  S.T_cpop_b = popcount_bytes(S.T_bmc_b.data(), S.T_mc_length);
  S.T_cpop_j = S.T_cpop_b;
  const long row_bytes = bsize(S.A_ncols);

  // bcc_single_load_M_An (bcc.c:270-413), per bin
  for (int nb = 0; nb < S.nbins; ++nb) {
    const BinInput &B = I.bins[nb];
    auto E = std::make_unique<Single>();
    E->nb = nb;
    E->A_nrows = B.A_nrows;
    E->A_rbother = E->A_nrows > 0;
    E->A_mr_length = bsize(E->A_nrows);
    E->A_bmr_b.assign(E->A_mr_length, 0);
    if (!B.A_mr_b.empty()) memcpy(E->A_bmr_b.data(), B.A_mr_b.data(), std::min<size_t>(B.A_mr_b.size(), E->A_mr_length));
    else for (int r = 0; r < E->A_nrows; ++r) bset_on(E->A_bmr_b.data(), r);
    E->A_bmr_j = E->A_bmr_b;
    E->A_bmr_j_rmv.assign(E->A_mr_length, 0);
    E->A_bmr_j_rtn.assign(E->A_mr_length, 0);
    E->A_rpop_b = popcount_bytes(E->A_bmr_b.data(), E->A_mr_length);
    E->A_rpop_j = popcount_bytes(E->A_bmr_j.data(), E->A_mr_length);
    E->A_umr_j.assign(std::max(1, E->A_nrows), 0);
    E->A_umr_j_rmv.assign(std::max(1, E->A_nrows), 0);
    E->A_umr_j_rtn.assign(std::max(1, E->A_nrows), 0);
    ura_from_bits(E->A_umr_j, E->A_bmr_j, E->A_nrows);
    E->Z_nrows = B.Z_nrows;
    E->Z_rbother = E->Z_nrows > 0;
    E->Z_mr_length = bsize(E->Z_nrows);
    E->Z_bmr_b.assign(E->Z_mr_length, 0);
    if (!B.Z_mr_b.empty()) memcpy(E->Z_bmr_b.data(), B.Z_mr_b.data(), std::min<size_t>(B.Z_mr_b.size(), E->Z_mr_length));
    else for (int r = 0; r < E->Z_nrows; ++r) bset_on(E->Z_bmr_b.data(), r);
    E->Z_bmr_j = E->Z_bmr_b;
    E->Z_rpop_b = popcount_bytes(E->Z_bmr_b.data(), E->Z_mr_length);
    E->Z_rpop_j = popcount_bytes(E->Z_bmr_j.data(), E->Z_mr_length);
    // packed data: An rows compacted by A_bmr_b; At rows (SNPs) compacted by A_bmc_b
    E->An_w = compact_rows(B.A_rows, E->A_nrows, row_bytes, E->A_bmr_b);
    E->At_w = compact_rows(transpose_rows(B.A_rows, E->A_nrows, S.A_ncols), S.A_ncols, bsize(E->A_nrows), S.A_bmc_b);
    E->M_An = S.keep(mh_make(E->A_nrows, S.A_ncols, E->An_w.data(), E->A_bmr_b.data(), S.A_bmc_b.data()));
    E->M_At = S.keep(mh_make(S.A_ncols, E->A_nrows, E->At_w.data(), S.A_bmc_b.data(), E->A_bmr_b.data()));
    if (E->Z_nrows > 0) {
      E->Zn_w = compact_rows(B.Z_rows, E->Z_nrows, row_bytes, E->Z_bmr_b);
      E->Zt_w = compact_rows(transpose_rows(B.Z_rows, E->Z_nrows, S.A_ncols), S.A_ncols, bsize(E->Z_nrows), S.A_bmc_b);
    } else {
      E->Zn_w.assign(POPLENGTH / BIT8, 0);
      E->Zt_w.assign(POPLENGTH / BIT8, 0);
    }
    E->M_Zn = S.keep(mh_make(E->Z_nrows, S.A_ncols, E->Zn_w.data(), E->Z_bmr_b.data(), S.A_bmc_b.data()));
    E->M_Zt = S.keep(mh_make(S.A_ncols, E->Z_nrows, E->Zt_w.data(), S.A_bmc_b.data(), E->Z_bmr_b.data()));
    // T and S (bcc.c:360-399): the covariate matrices when given (rows
    // compacted by the row mask, their transposes by the covariate mask),
    // otherwise one covariate column of ones.
    const long tb = bsize(S.T_ncols);
    if (!B.T_rows.empty()) {
      E->Tn_w = compact_rows(B.T_rows, E->A_nrows, tb, E->A_bmr_b);
      E->Tt_w = compact_rows(transpose_rows(B.T_rows, E->A_nrows, S.T_ncols), S.T_ncols, bsize(E->A_nrows), S.T_bmc_b);
    } else {
      E->Tn_w.assign((size_t)std::max(1, E->A_nrows) * (size_t)bsize(1), 0);
      for (int r = 0; r < E->A_nrows; ++r) E->Tn_w[(size_t)r * bsize(1)] |= (1 << 7);
      E->Tt_w.assign((size_t)bsize(E->A_nrows) + POPLENGTH / BIT8, 0);
      for (int r = 0; r < E->A_nrows; ++r) bset_on(E->Tt_w.data(), r);
    }
    E->M_Tn = S.keep(mh_make(E->A_nrows, S.T_ncols, E->Tn_w.data(), E->A_bmr_b.data(), S.T_bmc_b.data()));
    E->M_Tt = S.keep(mh_make(S.T_ncols, E->A_nrows, E->Tt_w.data(), S.T_bmc_b.data(), E->A_bmr_b.data()));
    if (!B.S_rows.empty() && E->Z_nrows > 0) {
      E->Sn_w = compact_rows(B.S_rows, E->Z_nrows, tb, E->Z_bmr_b);
      E->St_w = compact_rows(transpose_rows(B.S_rows, E->Z_nrows, S.T_ncols), S.T_ncols, bsize(E->Z_nrows), S.T_bmc_b);
    } else {
      E->Sn_w.assign((size_t)std::max(1, E->Z_nrows) * (size_t)bsize(1), 0);
      for (int r = 0; r < E->Z_nrows; ++r) E->Sn_w[(size_t)r * bsize(1)] |= (1 << 7);
      E->St_w.assign((size_t)bsize(E->Z_nrows) * (size_t)std::max(1, S.T_ncols) + POPLENGTH / BIT8, 0);
      for (int r = 0; r < E->Z_nrows; ++r) bset_on(E->St_w.data(), r);
    }
    E->M_Sn = S.keep(mh_make(E->Z_nrows, S.T_ncols, E->Sn_w.data(), E->Z_bmr_b.data(), S.T_bmc_b.data()));
    E->M_St = S.keep(mh_make(S.T_ncols, E->Z_nrows, E->St_w.data(), S.T_bmc_b.data(), E->Z_bmr_b.data()));
    // low-rank-update views share the packed data with their base handles
    M_handle &An = E->M_An->h, &At = E->M_At->h, &Zn = E->M_Zn->h, &Zt = E->M_Zt->h, &Tt = E->M_Tt->h;
    auto view = [&](M_handle &base) {
      return S.keep(mh_make(base.nrows, base.ncols, base.wX, base.mr_b, base.mc_b));
    };
    E->M_an = view(An); E->M_jn = view(An); E->M_kn = view(An); E->M_hn = view(An);
    E->M_at = view(At); E->M_jt = view(At); E->M_kt = view(At); E->M_ht = view(At);
    E->M_zn = view(Zn); E->M_vn = view(Zn);
    E->M_zt = view(Zt); E->M_vt = view(Zt);
    E->M_tt = view(Tt); E->M_rt = view(Tt);
    S.E.push_back(std::move(E));
  }
  // bcc_X_nrows_total (bcc.c:1179-1192)
  for (auto &E : S.E) {
    S.A_nrows_total += E->A_nrows; S.A_rpop_b_total += E->A_rpop_b; S.A_rpop_j_total += E->A_rpop_j;
    S.Z_nrows_total += E->Z_nrows; S.Z_rpop_b_total += E->Z_rpop_b; S.Z_rpop_j_total += E->Z_rpop_j;
  }
  // bcc_single_init_lf (bcc.c:652-990): buffers used on this path
  for (auto &Ep : S.E) {
    Single *E = Ep.get();
    E->lf_At_rsum = S.L(S.A_ncols);
    E->lf_Zt_rsum = S.L(S.A_ncols);
    const int T = S.T_ncols;
    E->lf_a1d2_Zt_Sn = S.L(T); E->lf_a2d2_Zt_Sn = S.L(T); E->lf_a3d2_Zt_Sn = S.L(T);
    E->lf_a1d2_At_Tn = S.L(T); E->lf_a2d2_At_Tn = S.L(T); E->lf_a3d2_At_Tn = S.L(T);
    E->lf_et_Tn = S.L(T); E->lf_et_Sn = S.L(T);
    E->lf_et_An = S.L(S.A_ncols); E->lf_a1d1_At_en = S.L(S.A_ncols);
    E->lf_a1d2_At_en = S.L(S.A_ncols); E->lf_a3d2_At_en = S.L(S.A_ncols);
    E->lf_et_An_a1d1 = S.L(1); E->lf_Tt_An_a1d1 = S.L(T);
    E->lf_T_AnAt_AnAt = S.L((unsigned long long)T * E->A_nrows);
    E->M_1 = S.keep(mh_make_owned(1, 1));
    E->lf_An_a1d1 = S.L((unsigned long long)E->A_rpop_b * 1);
    E->M_An_a1d1 = S.keep(mh_make_owned((1 + P.B_MLT) * 1, E->A_nrows));
    E->lf_a2d2_ZtSn = S.L((unsigned long long)S.A_cpop_b * S.T_cpop_b);
    E->M_a2d2_ZtSn = S.keep(mh_make_owned((1 + P.B_MLT) * (int)S.T_cpop_b, S.A_ncols));
    E->lf_a2d2_AtTn = S.L((unsigned long long)S.A_cpop_b * S.T_cpop_b);
    E->M_a2d2_AtTn = S.keep(mh_make_owned((1 + P.B_MLT) * (int)S.T_cpop_b, S.A_ncols));
    if (dcc_mode(P)) {
      E->lf_A_a0d1 = S.L(1); E->lf_A_a2d1 = S.L(1);
      E->lf_a1d1_ZtSn = S.L(T); E->lf_a1d1_AtTn = S.L(T);
      E->lf_a0d1_ZtSn = S.L((unsigned long long)S.A_cbother * S.A_cpop_b * S.T_cpop_b);
      E->lf_a0d1_AtTn = S.L((unsigned long long)S.A_cbother * S.A_cpop_b * S.T_cpop_b);
      E->M_a0d1_ZtSn = S.keep(mh_make_owned((1 + P.B_MLT) * (int)S.T_cpop_b, S.A_cbother * S.A_ncols));
      E->M_a0d1_AtTn = S.keep(mh_make_owned((1 + P.B_MLT) * (int)S.T_cpop_b, S.A_cbother * S.A_ncols));
    }
  }
  // bcc_single_init_lf (bcc.c:762-792, "store all"): the SNP x SNP x covariate
  // products of the column low-rank update, sized for ckeep retained x cdrop
  // removed columns (a scorebox removes up to ceil(col_max / (col_num - 1))
  // columns per step)
  if (P.QC_strategy.find("YnWt") != std::string::npos) {
    int cdrop = 0;
    get_xdrop(P, (double)S.A_rpop_j_total, (double)S.A_cpop_j, nullptr, &cdrop);
    if (P.test_type.find("scorebox") != std::string::npos && P.scorebox_col_num > 1 && P.scorebox_col_max > 0)
      cdrop = (int)ceil((double)P.scorebox_col_max / (double)(P.scorebox_col_num - 1));
    const unsigned long long ckeep = (unsigned long long)std::max(0, (int)S.A_cpop_j - cdrop);
    const unsigned long long n = ckeep * (unsigned long long)cdrop * (unsigned long long)S.T_ncols;
    for (auto &E : S.E) {  // released with the entry points' outputs (~State)
      E->lf_ztsvn = lh_make(E->Z_rbother ? n : 0);
      E->lf_attjn = lh_make(E->A_rbother ? n : 0);
      E->lf_ktrhn = lh_make(E->A_rbother ? n : 0);
    }
  }
  // bcc_single_init_lf (bcc.c:750-761, "condense"): the removed columns as
  // dense matrices, up to cdrop SNPs x the bin's rows
  if (qr_condense(P)) {
    int cdrop = 0;
    get_xdrop(P, (double)S.A_rpop_j_total, (double)S.A_cpop_j, nullptr, &cdrop);
    if (P.test_type.find("scorebox") != std::string::npos && P.scorebox_col_num > 1 && P.scorebox_col_max > 0)
      cdrop = (int)ceil((double)P.scorebox_col_max / (double)(P.scorebox_col_num - 1));
    for (auto &E : S.E) {
      E->lf_jn = S.L((unsigned long long)E->A_rbother * E->A_nrows * cdrop);
      E->lf_vn = S.L((unsigned long long)E->Z_rbother * E->Z_nrows * cdrop);
      S.mirror_zero(E->lf_jn);
      S.mirror_zero(E->lf_vn);
    }
  }
  // bcc_double_init_lf (bcc.c:1005-1150)
  int rdrop = 0;
  get_xdrop(P, (double)S.A_rpop_j_total, (double)S.A_cpop_j, &rdrop, nullptr);
  // The transposition flags of the removed-row products follow rdrop2 from
  // the gamma schedule (bcc.c:1027).  A scorebox removes up to
  // ceil(row_max / (row_num - 1)) rows per step; the reference sets that
  // count after rdrop2 (bcc.c:1028), so its buffers do not grow with it and a
  // larger step writes past them.  Here the buffers hold the larger step.
  const int rdrop2 = std::max(2, rdrop);
  int rcap = rdrop2;
  if (P.test_type.find("scorebox") != std::string::npos && P.scorebox_row_num > 1 && P.scorebox_row_max > 0)
    rcap = std::max(rcap, (int)ceil((double)P.scorebox_row_max / (double)(P.scorebox_row_num - 1)));
  S.F.resize((size_t)S.nbins * S.nbins);
  for (int nb1 = 0; nb1 < S.nbins; ++nb1) {
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      auto F = std::make_unique<Double>();
      F->nb1 = nb1; F->nb2 = nb2;
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      const int A1a = E1->M_An->h.nrows, A1b = (int)E1->M_An->h.rpop_b;
      const int A2a = E2->M_An->h.nrows, A2b = (int)E2->M_An->h.rpop_b;
      const int Z2a = E2->M_Zn->h.nrows, Z2b = (int)E2->M_Zn->h.rpop_b;
      if (dcc_mode(P)) {  // the half loop needs no row x row products
        const unsigned long long NT = (unsigned long long)E1->A_nrows * S.T_ncols;
        const unsigned long long AT = (unsigned long long)S.A_ncols * S.T_ncols;
        F->lf_An_a0d1_ZtSn = S.L(NT); F->lf_An_a0d1_AtTn = S.L(NT);
        F->lf_TAnZtS_ww = S.L(NT); F->lf_TAnAtT_ww = S.L(NT);
        F->lf_D_AtTn_ZtSn_vv = S.L(AT); F->lf_D_AtTn_AtTn_vv = S.L(AT);
        F->QR_AnZtSZnAt = S.L(NT); F->QR_AnAtTAnAt = S.L(NT);
        F->QC_AtTAnZtSZn = S.L(AT); F->QC_AtTAnAtTAn = S.L(AT);
        S.F[nb1 + nb2 * S.nbins] = std::move(F);
        continue;
      }
      F->lf_AnZt = S.L((unsigned long long)A1b * Z2b);
      F->M_AnZt = xcalc_out(S, A1a, A1b, Z2a, Z2b, &F->M_AnZt_trm);
      F->lf_AnAt = S.L((unsigned long long)A1b * A2b);
      F->M_AnAt = xcalc_out(S, A1a, A1b, A2a, A2b, &F->M_AnAt_trm);
      F->lf_jnvt = S.L((unsigned long long)A1b * Z2b);
      F->lf_jnjt = S.L((unsigned long long)A1b * A2b);
      const int c = S.A_cbother;
      const int n1b = c * std::min(rdrop2, A1b), n1c = c * std::min(rcap, A1b);
      const int n2k = c * std::min(rdrop2, A2b), n2c = c * std::min(rcap, A2b);
      F->lf_knzt = S.L((unsigned long long)n1c * (c * Z2b));
      F->M_knzt = xcalc_out(S, c * A1a, n1b, c * Z2a, c * Z2b, &F->M_knzt_trm, n1c);
      F->lf_hnvt = S.L((unsigned long long)n1c * (c * Z2b));
      F->M_hnvt = xcalc_out(S, c * A1a, n1b, c * Z2a, c * Z2b, &F->M_hnvt_trm, n1c);
      F->lf_ankt = S.L((unsigned long long)(c * A1b) * n2c);
      F->M_ankt = xcalc_out(S, c * A1a, c * A1b, c * A2a, n2k, &F->M_ankt_trm, -1, n2c);
      F->lf_knat = S.L((unsigned long long)n1c * (c * A2b));
      F->lf_knkt = S.L((unsigned long long)n1c * n2c);
      F->M_knkt = xcalc_out(S, c * A1a, n1b, c * A2a, n2k, &F->M_knkt_trm, n1c, n2c);
      const unsigned long long AT = (unsigned long long)S.A_ncols * S.T_ncols;
      F->lf_kt_r_knzt_s_zn = S.L(AT); F->lf_kt_r_hnvt_s_zn = S.L(AT); F->lf_at_t_ankt_r_kn = S.L(AT);
      F->lf_kt_r_knat_t_an = S.L(AT); F->lf_kt_r_knkt_r_kn = S.L(AT);
      F->lf_attjn____vtszn = S.L(AT); F->lf_attjn____jttan = S.L(AT); F->lf_attjn____htrkn = S.L(AT);
      F->lf_ktrhn____jttan = S.L(AT); F->lf_ktrhn____htrkn = S.L(AT);
      const unsigned long long NT = (unsigned long long)E1->M_An->h.nrows * S.T_ncols;
      F->lf_AnZt_S_ZnAt = S.L(NT); F->lf_AnAt_T_AnAt = S.L(NT);
      F->lf_At_T_AnZt_S_Zn = S.L(AT); F->lf_At_T_AnAt_T_An = S.L(AT);
      F->lf_AtTAn____ZtSZn = S.L(AT); F->lf_AtTAn____AtTAn = S.L(AT);
      F->lf_An_a2d2_Zt_Sn = S.L((unsigned long long)E1->A_nrows * S.T_ncols);
      F->lf_An_a2d2_At_Tn = S.L((unsigned long long)E1->A_nrows * S.T_ncols);
      F->QR_AnZtSZnAt = S.L((unsigned long long)E1->A_nrows * S.T_ncols);
      F->QR_AnAtTAnAt = S.L((unsigned long long)E1->A_nrows * S.T_ncols);
      F->QC_AtTAnZtSZn = S.L(AT); F->QC_AtTAnAtTAn = S.L(AT);
      S.mirror_zero(F->lf_AnZt); S.mirror_zero(F->lf_AnAt); S.mirror_zero(F->lf_jnvt); S.mirror_zero(F->lf_jnjt);
      S.mirror_zero(F->lf_knzt); S.mirror_zero(F->lf_hnvt); S.mirror_zero(F->lf_ankt); S.mirror_zero(F->lf_knat);
      S.mirror_zero(F->lf_knkt);
      S.F[nb1 + nb2 * S.nbins] = std::move(F);
    }
  }
  // bcc_load_A_p (bcc.c:1197-1313)
  S.A_pcols = (int)psize(S.A_ncols);
  S.AZ_rsum.assign(std::max(1, S.A_ncols), 0.0);
  S.A_p.assign(std::max(1, S.A_pcols), 0.0);
  for (auto &E : S.E) {
    memset(E->lf_At_rsum->lf, 0, sizeof(double) * S.A_ncols);
    wrap_An_v__run(TARGS, LAKGB_TYPE_00, SP_a, E->M_At->p(), &E->lf_At_rsum);
    memset(E->lf_Zt_rsum->lf, 0, sizeof(double) * S.A_ncols);
    wrap_An_v__run(TARGS, LAKGB_TYPE_00, SP_a, E->M_Zt->p(), &E->lf_Zt_rsum);
  }
  for (auto &E : S.E) {
    for (int c = 0; c < S.A_ncols; ++c) S.AZ_rsum[c] += E->lf_At_rsum->lf[c];
    for (int c = 0; c < S.A_ncols; ++c) S.AZ_rsum[c] += E->lf_Zt_rsum->lf[c];
  }
  for (int p = 0; p < S.A_pcols; ++p) {
    S.A_p[p] = 0.5;
    if (!P.test_sparse) continue;
    const int nc_start = std::min(S.A_ncols - 1, std::max(0, p * POPLENGTH));
    const int nc_final = std::min(S.A_ncols - 1, std::max(0, (p + 1) * POPLENGTH - 1));
    double tmp_sum = 0, tmp_num = 0;
    for (int nc = nc_start; nc <= nc_final; ++nc)
      if (bget_on(S.A_bmc_b.data(), nc)) { tmp_sum += S.AZ_rsum[nc]; tmp_num += 1; }
    if (tmp_num == 0) S.A_p[p] = 0.5;
    else {
      double v = tmp_sum / (tmp_num * (double)(S.A_rpop_b_total + S.Z_rpop_b_total));
      S.A_p[p] = v < 0.01 ? 0.01 : (v > 0.99 ? 0.99 : v);
    }
  }
  // calc_A_ajdk (An_ajdk_v.c:5-30)
  S.A_ajdk.assign((size_t)AJDK_TOT * std::max(1, S.A_pcols), 0.0);
  for (int k = 0; k < 3; ++k)
    for (int j = 0; j < 5; ++j)
      for (int nc = 0; nc < S.A_pcols; ++nc) {
        const double p = S.A_p[nc];
        S.A_ajdk[nc + (j + 5 * k) * S.A_pcols] =
            pow(p - (1 - p), j) * pow(1.0 / std::max(0.01, (4.0 * p * (1 - p))), k);
      }
  // bcc_init_QX (bcc.c:1369-1412)
  const size_t QC = (size_t)S.A_ncols * S.T_ncols * S.nbins * S.nbins;
  S.QC_AtTAnZtSZn_nrm.assign(std::max<size_t>(1, QC), 0.0);
  S.QC_AtTAnAtTAn_nrm.assign(std::max<size_t>(1, QC), 0.0);
  S.QC_svalue.assign(std::max(1, S.A_ncols), 0.0);
  S.QC_index_local_mc_a.assign(std::max(1, S.A_ncols), 0);
  S.QC_index_local_mc_b.assign(std::max(1, S.A_ncols), 0);
  S.QC_index_local_mc_j.assign(std::max(1, S.A_ncols), 0);
  const int NR = std::max(1, S.A_nrows_total);
  S.QR_svalue.assign(NR, 0.0);
  S.QR_index_global_mr_a.assign(NR, 0); S.QR_index_global_mr_b.assign(NR, 0); S.QR_index_global_mr_j.assign(NR, 0);
  S.QR_index_local_mr_a.assign(NR, 0); S.QR_index_local_mr_b.assign(NR, 0);
  S.QR_index_local_mr_j.assign(NR, 0); S.QR_index_local_nb.assign(NR, 0);
  int mx_a = 0, mx_b = 0, mx_j = 0;
  for (auto &E : S.E) {
    E->QR_index_global_mr_a.assign(std::max(1, E->A_nrows), 0);
    E->QR_index_global_mr_b.assign(std::max(1, E->A_nrows), 0);
    E->QR_index_global_mr_j.assign(std::max(1, E->A_nrows), 0);
    for (int mr_a = 0; mr_a < E->A_nrows; ++mr_a) {
      E->QR_index_global_mr_a[mr_a] = mx_a;
      if (bget_on(E->A_bmr_b.data(), mr_a)) {
        E->QR_index_global_mr_b[mr_a] = mx_b;
        if (bget_on(E->A_bmr_j.data(), mr_a)) { E->QR_index_global_mr_j[mr_a] = mx_j; mx_j++; }
        mx_b++;
      }
      mx_a++;
    }
    const size_t n = (size_t)E->A_nrows * S.T_ncols * S.nbins;
    E->QR_AnZtSZnAt_nrm.assign(std::max<size_t>(1, n), 0.0);
    E->QR_AnAtTAnAt_nrm.assign(std::max<size_t>(1, n), 0.0);
  }
  return 0;
}

// bcc_M_mxset (bcc.c:1414-1438)
void M_mxset_all(State &S) {
  S.A_cpop_j = popcount_bytes(S.A_bmc_j.data(), S.A_mc_length);
  S.T_cpop_j = popcount_bytes(S.T_bmc_j.data(), S.T_mc_length);
  S.A_rpop_j_total = 0; S.Z_rpop_j_total = 0;
  for (auto &E : S.E) {
    E->A_rpop_j = popcount_bytes(E->A_bmr_j.data(), E->A_mr_length); S.A_rpop_j_total += E->A_rpop_j;
    E->Z_rpop_j = popcount_bytes(E->Z_bmr_j.data(), E->Z_mr_length); S.Z_rpop_j_total += E->Z_rpop_j;
    mh_mxset(E->M_An, E->A_bmr_j.data(), S.A_bmc_j.data()); mh_mxset(E->M_At, S.A_bmc_j.data(), E->A_bmr_j.data());
    mh_mxset(E->M_Zn, E->Z_bmr_j.data(), S.A_bmc_j.data()); mh_mxset(E->M_Zt, S.A_bmc_j.data(), E->Z_bmr_j.data());
    mh_mxset(E->M_Tn, E->A_bmr_j.data(), S.T_bmc_j.data()); mh_mxset(E->M_Tt, S.T_bmc_j.data(), E->A_bmr_j.data());
    mh_mxset(E->M_Sn, E->Z_bmr_j.data(), S.T_bmc_j.data()); mh_mxset(E->M_St, S.T_bmc_j.data(), E->Z_bmr_j.data());
  }
}

// bcc_lrup_mxset (bcc_lrup.c:1101-1126)
void lrup_mxset(State &S) {
  for (auto &E : S.E) {
    unsigned char *rtn = E->A_bmr_j_rtn.data(), *rmv = E->A_bmr_j_rmv.data();
    unsigned char *crtn = S.A_bmc_j_rtn.data(), *crmv = S.A_bmc_j_rmv.data();
    mh_mxset(E->M_an, rtn, crtn); mh_mxset(E->M_at, crtn, rtn);
    mh_mxset(E->M_jn, rtn, crmv); mh_mxset(E->M_jt, crmv, rtn);
    mh_mxset(E->M_kn, rmv, crtn); mh_mxset(E->M_kt, crtn, rmv);
    mh_mxset(E->M_hn, rmv, crmv); mh_mxset(E->M_ht, crmv, rmv);
    mh_mxset(E->M_zn, E->Z_bmr_j.data(), crtn); mh_mxset(E->M_zt, crtn, E->Z_bmr_j.data());
    mh_mxset(E->M_vn, E->Z_bmr_j.data(), crmv); mh_mxset(E->M_vt, crmv, E->Z_bmr_j.data());
    mh_mxset(E->M_tt, S.T_bmc_j.data(), rtn);
    mh_mxset(E->M_rt, S.T_bmc_j.data(), rmv);
  }
}

// ---------------------------------------------------------------------------
// stages

// The stages below run their independent calls as one joined group (a
// deferral scope): no call reads another's output before the stage ends.
void An_ajdk_all(State &S) {  // bcc_An_ajdk (bcc_lf.c:7-51)
  S.defer_begin();
  for (auto &E : S.E) {
    if (E->A_rbother && S.A_cbother) wrap_An_ajdk_v(TARGS, T_pm, SP_a, E->M_An->p(), S.A_ajdk.data(), &E->lf_An_ajdk);
    if (E->Z_rbother && S.A_cbother) wrap_An_ajdk_v(TARGS, T_pm, SP_a, E->M_Zn->p(), S.A_ajdk.data(), &E->lf_Zn_ajdk);
  }
  S.defer_end();
}

void lf_ZtSn_all(State &S) {  // bcc_lf_ZtSn (bcc_lf.c:53-100)
  S.defer_begin();
  for (auto &E : S.E) {
    if (E->A_rbother && S.A_cbother)
      wrap_AnZt_vv__run(TARGS, T_pm, SP_a, SP_a, E->M_At->p(), E->M_Tt->p(), nullptr, nullptr, nullptr, &E->lf_AtTn);
    if (E->Z_rbother && S.A_cbother)
      wrap_AnZt_vv__run(TARGS, T_pm, SP_a, SP_a, E->M_Zt->p(), E->M_St->p(), nullptr, nullptr, nullptr, &E->lf_ZtSn);
  }
  S.defer_end();
}

void lf_YnWt_all(State &S) {  // bcc_lf_YnWt (bcc_lf.c:223-290)
  double *aj = S.A_ajdk.data();
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->Z_rbother)
        wrap_AnZt_vv__run(TARGS, T_pm, SP_b, SP_b, E1->M_An->p(), E2->M_Zn->p(), aj, E1->lf_An_ajdk, E2->lf_Zn_ajdk, &F->lf_AnZt);
      if (S.A_cbother && E1->A_rbother && E2->A_rbother) {
        if (nb1 == nb2)
          wrap_AnAt_vv__run(TARGS, T_pm, SP_b, SP_b, E1->M_An->p(), E2->M_An->p(), aj, E1->lf_An_ajdk, E2->lf_An_ajdk, &F->lf_AnAt);
        if (nb1 < nb2)
          wrap_AnZt_vv__run(TARGS, T_pm, SP_b, SP_b, E1->M_An->p(), E2->M_An->p(), aj, E1->lf_An_ajdk, E2->lf_An_ajdk, &F->lf_AnAt);
      }
    }
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->A_rbother && nb1 > nb2)
        S.transpose(S.f(nb1, nb2)->lf_AnAt, S.f(nb2, nb1)->lf_AnAt);
    }
}

// bcc_M_YnWt_excerpt (bcc_lf.c:300-316)
void xcalc_excerpt(State &S, int trm, MH *M_in1, MH *M_in2, L_handle *L_in, MH *M_out) {
  M_handle *out = M_out->p();
  int b_mlt = S.P.B_MLT;
  if (trm == 0)
    wrap_xcalc(TARGS, M_in1->h.mr_j, M_in1->h.mr_b, M_in2->h.mr_j, M_in2->h.mr_b, L_in, L_in->lf,
               &M_in1->h.nrows, &M_in2->h.nrows, &out, &b_mlt, 0);
  else
    wrap_xcalc(TARGS, M_in2->h.mr_j, M_in2->h.mr_b, M_in1->h.mr_j, M_in1->h.mr_b, L_in, L_in->lf,
               &M_in2->h.nrows, &M_in1->h.nrows, &out, &b_mlt, 1);
}

void M_YnWt_all(State &S) {  // bcc_M_YnWt (bcc_lf.c:318-356)
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->Z_rbother) xcalc_excerpt(S, F->M_AnZt_trm, E1->M_An, E2->M_Zn, F->lf_AnZt, F->M_AnZt);
      if (S.A_cbother && E1->A_rbother && E2->A_rbother) xcalc_excerpt(S, F->M_AnAt_trm, E1->M_An, E2->M_An, F->lf_AnAt, F->M_AnAt);
    }
}

// bcc_lf_At_T_YnWt_S_Zn_excerpt (bcc_lf.c:636-647)
void bitplane_excerpt(State &S, int trm, MH *At, MH *Tt, MH *Yn, MH *Wn, MH *St, MH *Zt, MH *YnWt, L_handle **out) {
  if (trm == 0)
    wrap_At_T_YnWt_S_Zn_ww__run(TARGS, SP_a, SP_a, At->p(), Tt->p(), Yn->p(), Wn->p(), St->p(), Zt->p(), S.A_ajdk.data(), YnWt->p(), out);
  else
    wrap_At_T_YnWt_S_Zn_ww__run(TARGS, SP_a, SP_a, Zt->p(), St->p(), Wn->p(), Yn->p(), Tt->p(), At->p(), S.A_ajdk.data(), YnWt->p(), out);
}

void lf_At_T_YnWt_S_Zn_all(State &S) {  // bcc_lf_At_T_YnWt_S_Zn (bcc_lf.c:649-709)
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->Z_rbother)
        bitplane_excerpt(S, F->M_AnZt_trm, E1->M_At, E1->M_Tt, E1->M_An, E2->M_Zn, E2->M_St, E2->M_Zt, F->M_AnZt, &F->lf_At_T_AnZt_S_Zn);
      if (S.A_cbother && E1->A_rbother && E2->A_rbother && nb1 <= nb2)
        bitplane_excerpt(S, F->M_AnAt_trm, E1->M_At, E1->M_Tt, E1->M_An, E2->M_An, E2->M_Tt, E2->M_At, F->M_AnAt, &F->lf_At_T_AnAt_T_An);
    }
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->A_rbother && nb1 > nb2)
        lh_duplicate(S.f(nb1, nb2)->lf_At_T_AnAt_T_An, S.f(nb2, nb1)->lf_At_T_AnAt_T_An);
    }
}

// The column strategies in use (GLOBAL_QC_strategy): YnWt (the bit-plane loop
// product of the quantised Grams) and / or ZtSWn (SNP x SNP products); when
// both are named the column scores come from ZtSWn (bcc_flattenloop.c:1458-1463).
bool qc_ynwt(const State &S) { return S.P.QC_strategy.find("YnWt") != std::string::npos; }
bool qc_ztswn(const State &S) { return S.P.QC_strategy.find("ZtSWn") != std::string::npos; }

void lf_ZtSWn_all(State &S) {  // bcc_lf_ZtSWn (bcc_lf.c:105-153), the terms without Y/W blocks
  if (!qc_ztswn(S)) return;
  double *aj = S.A_ajdk.data();
  for (auto &E : S.E) {
    if (E->Z_rbother && S.A_cbother)
      wrap_AtTAn_vv__run(TARGS, SP_b, SP_b, SP_b, E->M_Zt->p(), E->M_St->p(), E->M_Zt->p(), aj, aj, E->lf_ZtSn,
                         E->lf_ZtSn, &E->lf_ZtSZn);
    if (E->A_rbother && S.A_cbother)
      wrap_AtTAn_vv__run(TARGS, SP_b, SP_b, SP_b, E->M_At->p(), E->M_Tt->p(), E->M_At->p(), aj, aj, E->lf_AtTn,
                         E->lf_AtTn, &E->lf_AtTAn);
  }
}

void lf_AtTYn____WtSZn_all(State &S) {  // bcc_lf_AtTYn____WtSZn (bcc_lf.c:566-632)
  if (!qc_ztswn(S)) return;
  double *aj = S.A_ajdk.data();
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->Z_rbother)
        wrap_AtTYn____WtSZn_vv__run(TARGS, SP_a, SP_a, E1->M_At->p(), E1->M_Tt->p(), E1->M_At->p(), E2->M_Zt->p(),
                                    E2->M_St->p(), E2->M_Zt->p(), aj, E1->lf_AtTAn, E2->lf_ZtSZn,
                                    &F->lf_AtTAn____ZtSZn);
      if (S.A_cbother && E1->A_rbother && E2->A_rbother && nb1 <= nb2)
        wrap_AtTYn____WtSZn_vv__run(TARGS, SP_a, SP_a, E1->M_At->p(), E1->M_Tt->p(), E1->M_At->p(), E2->M_At->p(),
                                    E2->M_Tt->p(), E2->M_At->p(), aj, E1->lf_AtTAn, E2->lf_AtTAn,
                                    &F->lf_AtTAn____AtTAn);
    }
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->A_rbother && nb1 > nb2)
        lh_duplicate(S.f(nb1, nb2)->lf_AtTAn____AtTAn, S.f(nb2, nb1)->lf_AtTAn____AtTAn);
    }
}

// bcc_lrup_QC_ZtSWn_stage_0/1/2 (bcc_lrup.c:896-1006): the case rows just
// removed leave lf_AtTAn through a low-rank product of theirs, subtracted
// element by element (the control products never change: controls are not
// eliminated).
void lrup_QC_ZtSWn(State &S) {
  if (!qc_ztswn(S)) return;
  double *aj = S.A_ajdk.data();
  for (auto &E : S.E)
    if (E->A_rbother && S.A_cbother)
      wrap_AnZt_vv__run(TARGS, T_pm, SP_a, SP_a, E->M_kt->p(), E->M_rt->p(), nullptr, nullptr, nullptr, &E->lf_ktrn);
  for (auto &E : S.E)
    if (E->A_rbother && S.A_cbother)
      wrap_AtTAn_vv__run(TARGS, SP_b, SP_b, SP_b, E->M_kt->p(), E->M_rt->p(), E->M_kt->p(), aj, aj, E->lf_ktrn,
                         E->lf_ktrn, &E->lf_ktrkn);
  for (auto &E : S.E)
    if (E->A_rbother && S.A_cbother)
      for (unsigned long long i = 0; i < E->lf_AtTAn->length; ++i) E->lf_AtTAn->lf[i] -= E->lf_ktrkn->lf[i];
}

void lf_AnZt_S_WnYt_all(State &S) {  // bcc_lf_AnZt_S_WnYt (bcc_lf.c:360-410)
  // the bin pairs' products are independent: one joined group
  S.defer_begin();
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->Z_rbother)
        wrap_AnZt_S_WnYt_vv__run(TARGS, SP_a, SP_a, E1->M_An->p(), E2->M_St->p(), E2->M_Zn->p(), F->lf_AnZt, F->lf_AnZt, &F->lf_AnZt_S_ZnAt);
      if (S.A_cbother && E1->A_rbother && E2->A_rbother)
        wrap_AnZt_S_WnYt_vv__run(TARGS, SP_a, SP_a, E1->M_An->p(), E2->M_Tt->p(), E2->M_An->p(), F->lf_AnAt, F->lf_AnAt, &F->lf_AnAt_T_AnAt);
    }
  S.defer_end();
}

void set_l1(L_handle *L, unsigned long long length) {
  L->row_stride = length; L->spacing_row = SP_a; lh_zero(L);
}

unsigned popcount_masked_row(const unsigned char *row, const unsigned char *mask, long nbytes) {
  unsigned c = 0;
  long i = 0;
  for (; i + 8 <= nbytes; i += 8) {
    uint64_t a, m;
    memcpy(&a, row + i, 8);
    memcpy(&m, mask + i, 8);
    c += (unsigned)__builtin_popcountll(a & m);
  }
  for (; i < nbytes; ++i) c += (unsigned)__builtin_popcount((unsigned)(row[i] & mask[i]));
  return c;
}

// get_singlestudy_vv (bcc_flattenloop.c:359-731) for one bin, without the Y terms.
void singlestudy_vv(State &S, Single *E) {
  M_handle *An = E->M_An->p(), *At = E->M_At->p(), *Tt = E->M_Tt->p(), *St = E->M_St->p(), *Zt = E->M_Zt->p();
  L_handle *lfA = E->lf_An_ajdk, *lfZ = E->lf_Zn_ajdk;
  double *aj = S.A_ajdk.data();
  const int P = (int)psize(At->nrows);
  const int T = Tt->nrows, A_ncols = At->nrows, A_nrows = At->ncols;
  set_l1(E->lf_a1d2_Zt_Sn, T); set_l1(E->lf_a2d2_Zt_Sn, T); set_l1(E->lf_a3d2_Zt_Sn, T);
  set_l1(E->lf_a1d2_At_Tn, T); set_l1(E->lf_a2d2_At_Tn, T); set_l1(E->lf_a3d2_At_Tn, T);
  set_l1(E->lf_et_Tn, T); set_l1(E->lf_et_Sn, T);
  set_l1(E->lf_et_An, A_ncols); set_l1(E->lf_a1d1_At_en, A_ncols);
  set_l1(E->lf_a1d2_At_en, A_ncols); set_l1(E->lf_a3d2_At_en, A_ncols);
  set_l1(E->lf_et_An_a1d1, 1); set_l1(E->lf_Tt_An_a1d1, T);
  L_handle *TAA = E->lf_T_AnAt_AnAt;
  TAA->row_stride = T; TAA->spacing_row = SP_a; TAA->col_stride = A_nrows; TAA->spacing_col = SP_a; lh_zero(TAA);
  const int QR_AnZtSZnAt = E->A_rbother && S.A_cbother && E->Z_rbother;
  const int QR_AnAtTAnAt = E->A_rbother && S.A_cbother;
  const int QC_AtTAnZtSZn = QR_AnZtSZnAt;
  const int QC_AtTAnAtTAn = QR_AnAtTAnAt;
  unsigned *ma_a_ = An->m_a_, *ma_b_ = An->m_b_;
  unsigned *na_a_ = An->n_a_, *na_b_ = An->n_b_;
  unsigned *mz_a_ = Zt->n_a_, *mz_b_ = Zt->n_b_;
  unsigned *ns_a_ = St->m_a_, *ns_b_ = St->m_b_;
  if (QC_AtTAnAtTAn) {
    for (int ns_j = 0; ns_j < Tt->rpop_j; ++ns_j) {
      const unsigned ns_a = ns_a_[ns_j], ns_b = ns_b_[ns_j];
      const unsigned char *Tt_tag = Tt->wX + (long)ns_b * Tt->mc_length;
      for (int ma_j = 0; ma_j < At->cpop_j; ++ma_j) {
        const unsigned ma_a = ma_a_[ma_j], ma_b = ma_b_[ma_j];
        const int vT = bget_pm(Tt_tag, ma_a);
        *L1_get(E->lf_Tt_An_a1d1, ns_j, ns_b, ns_a) += vT * (*L2_get(lfA, ma_j, ma_b, ma_a, 0, 0, AJDK_1_1));
      }
    }
  }
  if (QR_AnZtSZnAt || QR_AnAtTAnAt) {
    for (int ns_j = 0; ns_j < Tt->rpop_j; ++ns_j) {
      const unsigned ns_a = ns_a_[ns_j], ns_b = ns_b_[ns_j];
      const unsigned char *Tt_tag = Tt->wX + (long)ns_b * Tt->mc_length;
      if (QR_AnAtTAnAt) {
        for (int ma_j = 0; ma_j < At->cpop_j; ++ma_j) {
          const unsigned ma_a = ma_a_[ma_j], ma_b = ma_b_[ma_j];
          const int vT = bget_pm(Tt_tag, ma_a);
          *L1_get(E->lf_a1d2_At_Tn, ns_j, ns_b, ns_a) += vT * (*L2_get(lfA, ma_j, ma_b, ma_a, 0, 0, AJDK_1_2));
          *L1_get(E->lf_a2d2_At_Tn, ns_j, ns_b, ns_a) += vT * (*L2_get(lfA, ma_j, ma_b, ma_a, 0, 0, AJDK_2_2));
          *L1_get(E->lf_a3d2_At_Tn, ns_j, ns_b, ns_a) += vT * (*L2_get(lfA, ma_j, ma_b, ma_a, 0, 0, AJDK_3_2));
        }
      }
      const unsigned char *St_tag = St->wX + (long)ns_b * St->mc_length;
      if (QR_AnZtSZnAt) {
        for (int mz_j = 0; mz_j < Zt->cpop_j; ++mz_j) {
          const unsigned mz_a = mz_a_[mz_j], mz_b = mz_b_[mz_j];
          const int vS = bget_pm(St_tag, mz_a);
          *L1_get(E->lf_a1d2_Zt_Sn, ns_j, ns_b, ns_a) += vS * (*L2_get(lfZ, mz_j, mz_b, mz_a, 0, 0, AJDK_1_2));
          *L1_get(E->lf_a2d2_Zt_Sn, ns_j, ns_b, ns_a) += vS * (*L2_get(lfZ, mz_j, mz_b, mz_a, 0, 0, AJDK_2_2));
          *L1_get(E->lf_a3d2_Zt_Sn, ns_j, ns_b, ns_a) += vS * (*L2_get(lfZ, mz_j, mz_b, mz_a, 0, 0, AJDK_3_2));
        }
      }
    }
  }
  if (QC_AtTAnAtTAn || QR_AnAtTAnAt) {
    for (int na_j = 0; na_j < At->rpop_j; ++na_j) {
      const unsigned na_a = na_a_[na_j], na_b = na_b_[na_j];
      const unsigned char *row = At->wX + (long)na_b * At->mc_length;
      if (QC_AtTAnAtTAn)
        *L1_get(E->lf_et_An, na_j, na_b, na_a) += (double)(-At->cpop_j + 2 * (long long)popcount_masked_row(row, At->mc_j, (long)At->mc_length));
      if (QR_AnAtTAnAt) {
        *L1_get(E->lf_a1d1_At_en, na_j, na_b, na_a) += aj[na_a / POPLENGTH + AJDK_1_1 * P] * (*L1_get(E->lf_et_An, na_j, na_b, na_a));
        *L1_get(E->lf_a1d2_At_en, na_j, na_b, na_a) += aj[na_a / POPLENGTH + AJDK_1_2 * P] * (*L1_get(E->lf_et_An, na_j, na_b, na_a));
        *L1_get(E->lf_a3d2_At_en, na_j, na_b, na_a) += aj[na_a / POPLENGTH + AJDK_3_2 * P] * (*L1_get(E->lf_et_An, na_j, na_b, na_a));
      }
    }
  }
  if (QC_AtTAnZtSZn || QC_AtTAnAtTAn || QR_AnZtSZnAt || QR_AnAtTAnAt) {
    for (int ns_j = 0; ns_j < Tt->rpop_j; ++ns_j) {
      const unsigned ns_a = ns_a_[ns_j], ns_b = ns_b_[ns_j];
      if (QC_AtTAnZtSZn || QC_AtTAnAtTAn || QR_AnAtTAnAt) {
        const unsigned char *row = Tt->wX + (long)ns_b * Tt->mc_length;
        *L1_get(E->lf_et_Tn, ns_j, ns_b, ns_a) = (double)(-Tt->cpop_j + 2 * (long long)popcount_masked_row(row, Tt->mc_j, (long)Tt->mc_length));
      }
      if (QC_AtTAnZtSZn || QR_AnZtSZnAt) {
        const unsigned char *row = St->wX + (long)ns_b * St->mc_length;
        *L1_get(E->lf_et_Sn, ns_j, ns_b, ns_a) = (double)(-St->cpop_j + 2 * (long long)popcount_masked_row(row, St->mc_j, (long)St->mc_length));
      }
    }
  }
  if (QC_AtTAnAtTAn) {
    for (int ma_j = 0; ma_j < At->cpop_j; ++ma_j) {
      const unsigned ma_a = ma_a_[ma_j], ma_b = ma_b_[ma_j];
      *L1_get(E->lf_et_An_a1d1, 0, 0, 0) += (*L2_get(lfA, ma_j, ma_b, ma_a, 0, 0, AJDK_1_1));
    }
  }
  if (QR_AnAtTAnAt) {
    double A_dtmp_a0d1 = 0, A_dtmp_a2d1 = 0;
    const int AP = (int)psize(An->ncols);
    for (int nc = 0; nc < AP; ++nc)
      A_dtmp_a0d1 += (double)aj[nc + AJDK_0_1 * AP] * (double)popcount_bytes(An->mc_j + (long)nc * (POPLENGTH / BIT8), POPLENGTH / BIT8);
    for (int nc = 0; nc < AP; ++nc)
      A_dtmp_a2d1 += (double)aj[nc + AJDK_2_1 * AP] * (double)popcount_bytes(An->mc_j + (long)nc * (POPLENGTH / BIT8), POPLENGTH / BIT8);
    for (int ma_j = 0; ma_j < At->cpop_j; ++ma_j) {
      const unsigned ma_a = ma_a_[ma_j], ma_b = ma_b_[ma_j];
      double A_dtmp = A_dtmp_a0d1;
      // The reference subtracts 2*popcount_xor_lf(row, row), a weighted
      // popcount of a row XORed with itself, which is exactly zero.
      A_dtmp -= (*L2_get(lfA, ma_j, ma_b, ma_a, 0, 0, AJDK_1_1)) + (*L2_get(lfA, ma_j, ma_b, ma_a, 0, 0, AJDK_1_1)) - A_dtmp_a2d1;
      for (int ns_j = 0; ns_j < Tt->rpop_j; ++ns_j) {
        const unsigned ns_a = ns_a_[ns_j], ns_b = ns_b_[ns_j];
        const unsigned char *Tt_tag = Tt->wX + (long)ns_b * Tt->mc_length;
        const int vT = bget_pm(Tt_tag, ma_a);
        *L2_get(TAA, ns_j, ns_b, ns_a, ma_j, ma_b, ma_a) = vT * A_dtmp * A_dtmp;
      }
    }
  }
}

void singlestudy_ww(State &S) {  // bcc_singlestudy_ww (bcc_flattenloop.c:773-831)
  for (auto &Ep : S.E) {
    Single *E = Ep.get();
    if (E->A_rbother && S.A_cbother) {  // At_Yn_a1d1_excerpt (:753-771)
      L_handle *L = E->lf_An_a1d1;
      L->spacing_row = SP_b; L->spacing_col = SP_b; L->row_stride = E->M_An->h.rpop_b; L->col_stride = 1;
      lh_zero(L);
      M_handle *An = E->M_An->p();
      for (int my_j = 0; my_j < An->rpop_j; ++my_j) {
        const unsigned my_a = An->m_a_[my_j], my_b = An->m_b_[my_j];
        *L1_get(L, my_j, my_b, my_a) = *L2_get(E->lf_An_ajdk, my_j, my_b, my_a, 0, 0, AJDK_1_1);
      }
    }
  }
  S.defer_begin();
  for (auto &Ep : S.E) {
    Single *E = Ep.get();
    if (E->A_rbother && S.A_cbother) {
      M_handle *out = E->M_An_a1d1->p();
      int one = 1, b_mlt = S.P.B_MLT;
      wrap_xcalc(TARGS, E->M_An->h.mr_j, E->M_An->h.mr_b, E->M_1->h.mr_j, E->M_1->h.mr_b, E->lf_An_a1d1,
                 E->lf_An_a1d1->lf, &E->M_An->h.nrows, &one, &out, &b_mlt, 0);
    }
  }
  S.defer_end();
  S.defer_begin();
  for (auto &Ep : S.E) {
    Single *E = Ep.get();
    if (E->A_rbother && S.A_cbother)
      wrap_An_ZtSn_ww__run(TARGS, SP_a, SP_a, E->M_At->p(), E->lf_An_a1d1, E->M_An_a1d1->p(), E->M_1->p(), &E->lf_At_An_a1d1);
  }
  S.defer_end();
  for (auto &Ep : S.E) singlestudy_vv(S, Ep.get());
}

// An_a2d2_ZtSn_excerpt (An_ZtSn_ww.c:267-289)
void a2d2_excerpt(State &S, M_handle *Zt, M_handle *St, L_handle *lf_ZtSn, L_handle *out) {
  out->spacing_row = SP_b; out->spacing_col = SP_b;
  out->row_stride = Zt->rpop_b; out->col_stride = St->rpop_b;
  lh_zero(out);
  const int P = (int)psize(Zt->nrows);
  for (int nz_j = 0; nz_j < Zt->rpop_j; ++nz_j) {
    const unsigned nz_a = Zt->m_a_[nz_j], nz_b = Zt->m_b_[nz_j];
    for (int ns_j = 0; ns_j < St->rpop_j; ++ns_j) {
      const unsigned ns_a = St->m_a_[ns_j], ns_b = St->m_b_[ns_j];
      *L2_get(out, nz_j, nz_b, nz_a, ns_j, ns_b, ns_a) =
          S.A_ajdk[nz_a / POPLENGTH + AJDK_2_2 * P] * (*L2_get(lf_ZtSn, nz_j, nz_b, nz_a, ns_j, ns_b, ns_a));
    }
  }
}

void doublestudy_ww(State &S) {  // bcc_doublestudy_ww (bcc_flattenloop.c:977-1029)
  for (auto &E : S.E) {
    if (E->Z_rbother && S.A_cbother) a2d2_excerpt(S, E->M_Zt->p(), E->M_St->p(), E->lf_ZtSn, E->lf_a2d2_ZtSn);
    if (E->A_rbother && S.A_cbother) a2d2_excerpt(S, E->M_At->p(), E->M_Tt->p(), E->lf_AtTn, E->lf_a2d2_AtTn);
  }
  int b_mlt = S.P.B_MLT;
  S.defer_begin();
  for (auto &E : S.E) {
    if (E->Z_rbother && S.A_cbother) {
      M_handle *out = E->M_a2d2_ZtSn->p();
      wrap_xcalc(TARGS, E->M_Zt->h.mr_j, E->M_Zt->h.mr_b, E->M_St->h.mr_j, E->M_St->h.mr_b, E->lf_a2d2_ZtSn,
                 E->lf_a2d2_ZtSn->lf, &E->M_Zt->h.nrows, &E->M_St->h.nrows, &out, &b_mlt, 0);
    }
    if (E->A_rbother && S.A_cbother) {
      M_handle *out = E->M_a2d2_AtTn->p();
      wrap_xcalc(TARGS, E->M_At->h.mr_j, E->M_At->h.mr_b, E->M_Tt->h.mr_j, E->M_Tt->h.mr_b, E->lf_a2d2_AtTn,
                 E->lf_a2d2_AtTn->lf, &E->M_At->h.nrows, &E->M_Tt->h.nrows, &out, &b_mlt, 0);
    }
  }
  S.defer_end();
  S.defer_begin();  // the bin pairs' products, read from flattenloop on
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      for (L_handle *L : {F->lf_An_a2d2_Zt_Sn, F->lf_An_a2d2_At_Tn}) {
        L->row_stride = E1->A_nrows; L->spacing_row = SP_a; L->col_stride = S.T_ncols; L->spacing_col = SP_a; lh_zero(L);
      }
      if (E1->A_rbother && S.A_cbother && E2->Z_rbother)
        wrap_An_ZtSn_ww__run(TARGS, SP_a, SP_a, E1->M_An->p(), E2->lf_a2d2_ZtSn, E2->M_a2d2_ZtSn->p(), E2->M_St->p(), &F->lf_An_a2d2_Zt_Sn);
      if (E1->A_rbother && S.A_cbother && E2->A_rbother)
        wrap_An_ZtSn_ww__run(TARGS, SP_a, SP_a, E1->M_An->p(), E2->lf_a2d2_AtTn, E2->M_a2d2_AtTn->p(), E2->M_Tt->p(), &F->lf_An_a2d2_At_Tn);
    }
  S.defer_end();
}

double mask_sum(State &S, M_handle *An, int k) {
  const int P = (int)psize(An->ncols);
  double s = 0;
  for (int nc = 0; nc < P; ++nc)
    s += (double)S.A_ajdk[nc + k * P] * (double)popcount_bytes(An->mc_j + (long)nc * (POPLENGTH / BIT8), POPLENGTH / BIT8);
  return s;
}

// get_flattenloop (bcc_flattenloop.c:1431-1889) for one bin pair, without Y terms.
void flattenloop_pair(State &S, Double *F) {
  Single *E1 = S.E[F->nb1].get(), *E2 = S.E[F->nb2].get();
  M_handle *An1 = E1->M_An->p(), *At1 = E1->M_At->p(), *Tt2 = E2->M_Tt->p();
  double *aj = S.A_ajdk.data();
  const int P = (int)psize(At1->nrows);
  const int A_ncols = At1->nrows, T = E1->M_Tt->h.nrows, A_nrows1 = At1->ncols;
  const int QR_AnZtSZnAt = E1->A_rbother && S.A_cbother && E2->Z_rbother;
  const int QR_AnAtTAnAt = E1->A_rbother && S.A_cbother && E2->A_rbother;
  const int QC_AtTAnZtSZn = QR_AnZtSZnAt, QC_AtTAnAtTAn = QR_AnAtTAnAt;
  // the column loop products: ZtSWn's when that strategy is named
  // (use_AtTXn____XtXXn_flag, bcc_flattenloop.c:1463), else the bit-plane ones
  L_handle *qc_zs = qc_ztswn(S) ? F->lf_AtTAn____ZtSZn : F->lf_At_T_AnZt_S_Zn;
  L_handle *qc_at = qc_ztswn(S) ? F->lf_AtTAn____AtTAn : F->lf_At_T_AnAt_T_An;
  for (L_handle *L : {F->QR_AnZtSZnAt, F->QR_AnAtTAnAt}) {
    L->row_stride = A_nrows1; L->spacing_row = SP_a; L->col_stride = T; L->spacing_col = SP_b; lh_zero(L);
  }
  for (L_handle *L : {F->QC_AtTAnZtSZn, F->QC_AtTAnAtTAn}) {
    L->row_stride = A_ncols; L->spacing_row = SP_a; L->col_stride = T; L->spacing_col = SP_b; lh_zero(L);
  }
  double lf_A_a0d2 = 0, lf_A_a2d2 = 0, lf_A_a4d2 = 0, lf_A_a0d1 = 0, lf_A_a2d1 = 0;
  if (QR_AnZtSZnAt || QR_AnAtTAnAt) {
    lf_A_a0d2 = mask_sum(S, An1, AJDK_0_2);
    lf_A_a2d2 = mask_sum(S, An1, AJDK_2_2);
    lf_A_a4d2 = mask_sum(S, An1, AJDK_4_2);
    lf_A_a0d1 = mask_sum(S, An1, AJDK_0_1);
    lf_A_a2d1 = mask_sum(S, An1, AJDK_2_1);
  }
  if (QR_AnZtSZnAt || QR_AnAtTAnAt) {
    for (int ns_j = 0; ns_j < Tt2->rpop_j; ++ns_j) {
      const unsigned ns_a = Tt2->m_a_[ns_j], ns_b = Tt2->m_b_[ns_j];
      for (int ma_j = 0; ma_j < An1->rpop_j; ++ma_j) {
        const unsigned ma_a = An1->m_a_[ma_j], ma_b = An1->m_b_[ma_j];
        if (QR_AnZtSZnAt) *L2_get(F->QR_AnZtSZnAt, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a) = *L2_get(F->lf_AnZt_S_ZnAt, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a);
        if (QR_AnAtTAnAt) *L2_get(F->QR_AnAtTAnAt, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a) = *L2_get(F->lf_AnAt_T_AnAt, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a);
      }
    }
    for (int ns_j = 0; ns_j < Tt2->rpop_j; ++ns_j) {
      const unsigned ns_a = Tt2->m_a_[ns_j], ns_b = Tt2->m_b_[ns_j];
      for (int ma_j = 0; ma_j < An1->rpop_j; ++ma_j) {
        const unsigned ma_a = An1->m_a_[ma_j], ma_b = An1->m_b_[ma_j];
        L_handle *lfA = E1->lf_An_ajdk;
        if (QR_AnZtSZnAt) {
          const double et = *L1_get(E2->lf_et_Sn, ns_j, ns_b, ns_a);
          const double dtmp =
              +1 * lf_A_a0d2 * et
              - 2 * (*L1_get(E2->lf_a1d2_Zt_Sn, ns_j, ns_b, ns_a))
              + 1 * lf_A_a2d2 * et
              - 2 * (*L2_get(lfA, ma_j, ma_b, ma_a, 0, 0, AJDK_1_2)) * et
              + 4 * (*L2_get(F->lf_An_a2d2_Zt_Sn, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a))
              - 2 * (*L2_get(lfA, ma_j, ma_b, ma_a, 0, 0, AJDK_3_2)) * et
              + 1 * lf_A_a2d2 * et
              - 2 * (*L1_get(E2->lf_a3d2_Zt_Sn, ns_j, ns_b, ns_a))
              + 1 * lf_A_a4d2 * et;
          *L2_get(F->QR_AnZtSZnAt, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a) += -dtmp;
        }
        if (QR_AnAtTAnAt) {
          const double et = *L1_get(E2->lf_et_Tn, ns_j, ns_b, ns_a);
          const double dtmp =
              +1 * lf_A_a0d2 * et
              - 2 * (*L1_get(E2->lf_a1d2_At_Tn, ns_j, ns_b, ns_a))
              + 1 * lf_A_a2d2 * et
              - 2 * (*L2_get(lfA, ma_j, ma_b, ma_a, 0, 0, AJDK_1_2)) * et
              + 4 * (*L2_get(F->lf_An_a2d2_At_Tn, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a))
              - 2 * (*L2_get(lfA, ma_j, ma_b, ma_a, 0, 0, AJDK_3_2)) * et
              + 1 * lf_A_a2d2 * et
              - 2 * (*L1_get(E2->lf_a3d2_At_Tn, ns_j, ns_b, ns_a))
              + 1 * lf_A_a4d2 * et;
          *L2_get(F->QR_AnAtTAnAt, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a) += -dtmp;
        }
      }
    }
  }
  if (QR_AnAtTAnAt && F->nb1 == F->nb2) {
    for (int ns_j = 0; ns_j < Tt2->rpop_j; ++ns_j) {
      const unsigned ns_a = Tt2->m_a_[ns_j], ns_b = Tt2->m_b_[ns_j];
      for (int ma_j = 0; ma_j < An1->rpop_j; ++ma_j) {
        const unsigned ma_a = An1->m_a_[ma_j], ma_b = An1->m_b_[ma_j];
        const double dtmp = *L2_get(E1->lf_T_AnAt_AnAt, ns_j, ns_b, ns_a, ma_j, ma_b, ma_a);
        *L2_get(F->QR_AnAtTAnAt, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a) += -dtmp;
      }
    }
    for (int ns_j = 0; ns_j < Tt2->rpop_j; ++ns_j) {
      const unsigned ns_a = Tt2->m_a_[ns_j], ns_b = Tt2->m_b_[ns_j];
      const unsigned char *Tt_tag = Tt2->wX + (long)ns_b * Tt2->mc_length;
      for (int ma_j = 0; ma_j < An1->rpop_j; ++ma_j) {
        const unsigned ma_a = An1->m_a_[ma_j], ma_b = An1->m_b_[ma_j];
        const int vT = bget_pm(Tt_tag, ma_a);
        L_handle *lfA = E1->lf_An_ajdk;
        const double dtmp = vT * (+1 * lf_A_a0d2
                                  - 4 * (*L2_get(lfA, ma_j, ma_b, ma_a, 0, 0, AJDK_1_2))
                                  + 6 * lf_A_a2d2
                                  - 4 * (*L2_get(lfA, ma_j, ma_b, ma_a, 0, 0, AJDK_3_2))
                                  + 1 * lf_A_a4d2);
        *L2_get(F->QR_AnAtTAnAt, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a) += +dtmp;
      }
    }
  }
  if (QC_AtTAnZtSZn || QC_AtTAnAtTAn) {
    for (int ns_j = 0; ns_j < Tt2->rpop_j; ++ns_j) {
      const unsigned ns_a = Tt2->m_a_[ns_j], ns_b = Tt2->m_b_[ns_j];
      for (int na_j = 0; na_j < At1->rpop_j; ++na_j) {
        const unsigned na_a = At1->m_a_[na_j], na_b = At1->m_b_[na_j];
        const double D = aj[na_a / POPLENGTH + AJDK_0_1 * P];
        if (QC_AtTAnZtSZn) *L2_get(F->QC_AtTAnZtSZn, na_j, na_b, na_a, ns_j, ns_b, ns_a) = D * (*L2_get(qc_zs, na_j, na_b, na_a, ns_j, ns_b, ns_a));
        if (QC_AtTAnAtTAn) *L2_get(F->QC_AtTAnAtTAn, na_j, na_b, na_a, ns_j, ns_b, ns_a) = D * (*L2_get(qc_at, na_j, na_b, na_a, ns_j, ns_b, ns_a));
      }
    }
    for (int ns_j = 0; ns_j < Tt2->rpop_j; ++ns_j) {
      const unsigned ns_a = Tt2->m_a_[ns_j], ns_b = Tt2->m_b_[ns_j];
      for (int na_j = 0; na_j < At1->rpop_j; ++na_j) {
        const unsigned na_a = At1->m_a_[na_j], na_b = At1->m_b_[na_j];
        const double D01 = aj[na_a / POPLENGTH + AJDK_0_1 * P];
        const double A10 = aj[na_a / POPLENGTH + AJDK_1_0 * P];
        const double A20 = aj[na_a / POPLENGTH + AJDK_2_0 * P];
        const double etT1 = *L1_get(E1->lf_et_Tn, ns_j, ns_b, ns_a);
        const double AtTn1 = *L2_get(E1->lf_AtTn, na_j, na_b, na_a, ns_j, ns_b, ns_a);
        if (QC_AtTAnZtSZn) {
          const double etS2 = *L1_get(E2->lf_et_Sn, ns_j, ns_b, ns_a);
          const double ZtSn2 = *L2_get(E2->lf_ZtSn, na_j, na_b, na_a, ns_j, ns_b, ns_a);
          const double dtmp = D01 * (+(1 * etT1) - (2 * A10 * AtTn1) + (A20 * etT1)) * D01 *
                              (+(1 * etS2) - (2 * A10 * ZtSn2) + (A20 * etS2));
          *L2_get(F->QC_AtTAnZtSZn, na_j, na_b, na_a, ns_j, ns_b, ns_a) += -dtmp;
        }
        if (QC_AtTAnAtTAn) {
          const double etT2 = *L1_get(E2->lf_et_Tn, ns_j, ns_b, ns_a);
          const double AtTn2 = *L2_get(E2->lf_AtTn, na_j, na_b, na_a, ns_j, ns_b, ns_a);
          const double dtmp = D01 * (+(1 * etT1) - (2 * A10 * AtTn1) + (A20 * etT1)) * D01 *
                              (+(1 * etT2) - (2 * A10 * AtTn2) + (A20 * etT2));
          *L2_get(F->QC_AtTAnAtTAn, na_j, na_b, na_a, ns_j, ns_b, ns_a) += -dtmp;
        }
      }
    }
  }
  if (QC_AtTAnAtTAn && F->nb1 == F->nb2) {
    const double rpop = (double)An1->rpop_j;
    for (int ns_j = 0; ns_j < Tt2->rpop_j; ++ns_j) {
      const unsigned ns_a = Tt2->m_a_[ns_j], ns_b = Tt2->m_b_[ns_j];
      for (int na_j = 0; na_j < At1->rpop_j; ++na_j) {
        const unsigned na_a = At1->m_a_[na_j], na_b = At1->m_b_[na_j];
        const double A01 = aj[na_a / POPLENGTH + AJDK_0_1 * P], A11 = aj[na_a / POPLENGTH + AJDK_1_1 * P];
        const double A21 = aj[na_a / POPLENGTH + AJDK_2_1 * P];
        const double etAn = *L1_get(E1->lf_et_An, na_j, na_b, na_a);
        const double etAa = *L1_get(E1->lf_et_An_a1d1, 0, 0, 0);
        const double AtAa = *L1_get(E1->lf_At_An_a1d1, na_j, na_b, na_a);
        const double dtmp = (+(1 * A01 * rpop * lf_A_a0d1)
                             - (2 * A11 * etAn * lf_A_a0d1)
                             + (1 * A21 * rpop * lf_A_a0d1)
                             - (2 * A01 * etAa)
                             + (4 * A11 * AtAa)
                             - (2 * A21 * etAa)
                             + (1 * A01 * rpop * lf_A_a2d1)
                             - (2 * A11 * etAn * lf_A_a2d1)
                             + (1 * A21 * rpop * lf_A_a2d1));
        *L2_get(F->QC_AtTAnAtTAn, na_j, na_b, na_a, ns_j, ns_b, ns_a) += -dtmp;
      }
    }
    for (int ns_j = 0; ns_j < Tt2->rpop_j; ++ns_j) {
      const unsigned ns_a = Tt2->m_a_[ns_j], ns_b = Tt2->m_b_[ns_j];
      for (int na_j = 0; na_j < At1->rpop_j; ++na_j) {
        const unsigned na_a = At1->m_a_[na_j], na_b = At1->m_b_[na_j];
        const double etAn = *L1_get(E1->lf_et_An, na_j, na_b, na_a);
        const double dtmp = (+(1 * aj[na_a / POPLENGTH + AJDK_0_2 * P] * rpop)
                             - (4 * aj[na_a / POPLENGTH + AJDK_1_2 * P] * etAn)
                             + (6 * aj[na_a / POPLENGTH + AJDK_2_2 * P] * rpop)
                             - (4 * aj[na_a / POPLENGTH + AJDK_3_2 * P] * etAn)
                             + (1 * aj[na_a / POPLENGTH + AJDK_4_2 * P] * rpop));
        *L2_get(F->QC_AtTAnAtTAn, na_j, na_b, na_a, ns_j, ns_b, ns_a) += +dtmp;
      }
    }
  }
}

void flattenloop(State &S) {
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) flattenloop_pair(S, S.f(nb1, nb2));
}

// f(r) for every r < n whose bit is on in m1 (and in m2 when given), in
// ascending order, a mask byte at a time.
template <typename F>
inline void for_each_on(const unsigned char *m1, const unsigned char *m2, unsigned long long n, F f) {
  const unsigned long long nbytes = (n + 7) / 8;
  for (unsigned long long i = 0; i < nbytes; ++i) {
    const unsigned v = m2 ? (unsigned)(m1[i] & m2[i]) : (unsigned)m1[i];
    if (!v) continue;
    const unsigned long long r0 = i * 8;
    if (v == 0xFFu && r0 + 8 <= n) {
      for (unsigned long long r = r0; r < r0 + 8; ++r) f(r);
    } else {
      for (unsigned k = 0; k < 8 && r0 + k < n; ++k)
        if ((v >> (7 - k)) & 1u) f(r0 + k);
    }
  }
}

// dra_plusdivequals_s___m_m (ra_stats.c:69-76).  Every element here and in
// plustimes is updated on its own, so the order of the visits does not
// change the results.
void plusdiv(const State &S, double *d1, unsigned long long nrows, unsigned long long ncols, const double *d2,
             double denominator, const unsigned char *bmr, const unsigned char *bmc) {
  double d_use = denominator;
  if (fabs(d_use) < S.P.tolerance) d_use = 1;
  for (unsigned long long c = 0; c < ncols; ++c)
    if (bget_on(bmc, (long)c)) {
      double *o = d1 + c * nrows;
      const double *in = d2 + c * nrows;
      for_each_on(bmr, nullptr, nrows, [&](unsigned long long r) { o[r] += in[r] / d_use; });
    }
}

// dra_plustimesequals_s___m_m (ra_stats.c:63-68)
void plustimes(double *d1, unsigned long long nrows, unsigned long long ncols, const double *d2, double m,
               const unsigned char *bmr, const unsigned char *bmc) {
  for (unsigned long long c = 0; c < ncols; ++c)
    if (bget_on(bmc, (long)c)) {
      double *o = d1 + c * nrows;
      const double *in = d2 + c * nrows;
      for_each_on(bmr, nullptr, nrows, [&](unsigned long long r) { o[r] += m * in[r]; });
    }
}

void dra_sumx0(double *d, unsigned long long stride, unsigned long long length) {
  for (unsigned long long r = 1; r < length; ++r) d[0] += d[r * stride];
}

// bcc_sumscores_nrm with GLOBAL_Ireq > 0 (bcc_sumscores.c:583-628): each bin
// pair normalised by its own number of summands, nothing summed over bins.
void sumscores_nrm_per_bin(State &S) {
  const int nb = S.nbins, T = S.T_ncols;
  const bool dcc = dcc_mode(S.P);  // dcc_sumscores_nrm (dcc_sumscores.c:478-532): one fewer column factor
  for (int nb1 = 0; nb1 < nb; ++nb1)
    for (int nb2 = 0; nb2 < nb; ++nb2) {
      const int nbx = nb1 + nb2 * nb, same = nb1 == nb2 ? 1 : 0;
      Single *E = S.E[nb1].get(), *E2 = S.E[nb2].get();
      Double *F = S.f(nb1, nb2);
      const unsigned long long AN = (unsigned long long)E->A_nrows;
      if (E->A_rbother && S.A_cbother && E2->Z_rbother) {
        double *d = &E->QR_AnZtSZnAt_nrm[nb2 * AN * T];
        memset(d, 0, AN * T * sizeof(double));
        const long long lld = dcc ? (long long)(E2->M_Zn->h.rpop_j - 0) * (long long)(E2->M_Zn->h.cpop_j)
                                  : (long long)(E2->M_Zn->h.rpop_j - 0) * (long long)(E2->M_Zn->h.cpop_j) * (long long)(E2->M_Zn->h.cpop_j - 1);
        plusdiv(S, d, AN, T, F->QR_AnZtSZnAt->lf, (double)lld, E->A_bmr_j.data(), S.T_bmc_j.data());
      }
      if (E->A_rbother && S.A_cbother && E2->A_rbother) {
        double *d = &E->QR_AnAtTAnAt_nrm[nb2 * AN * T];
        memset(d, 0, AN * T * sizeof(double));
        const long long lld = dcc ? (long long)(E2->M_An->h.rpop_j - same) * (long long)(E2->M_An->h.cpop_j)
                                  : (long long)(E2->M_An->h.rpop_j - same) * (long long)(E2->M_An->h.cpop_j) * (long long)(E2->M_An->h.cpop_j - 1);
        plusdiv(S, d, AN, T, F->QR_AnAtTAnAt->lf, (double)lld, E->A_bmr_j.data(), S.T_bmc_j.data());
      }
      const unsigned long long AC = (unsigned long long)S.A_ncols;
      if (E->A_rbother && S.A_cbother && E2->Z_rbother) {
        double *d = &S.QC_AtTAnZtSZn_nrm[nbx * AC * T];
        memset(d, 0, AC * T * sizeof(double));
        const long long lld = dcc ? (long long)(E->M_An->h.rpop_j) * (long long)(E2->M_Zn->h.rpop_j)
                                  : (long long)(E->M_An->h.rpop_j) * (long long)(E->M_An->h.cpop_j - 1) * (long long)(E2->M_Zn->h.rpop_j);
        plusdiv(S, d, AC, T, F->QC_AtTAnZtSZn->lf, (double)lld, S.A_bmc_j.data(), S.T_bmc_j.data());
      }
      if (E->A_rbother && S.A_cbother && E2->A_rbother) {
        double *d = &S.QC_AtTAnAtTAn_nrm[nbx * AC * T];
        memset(d, 0, AC * T * sizeof(double));
        const long long lld = dcc ? (long long)(E->M_An->h.rpop_j) * (long long)(E2->M_An->h.rpop_j - same)
                                  : (long long)(E->M_An->h.rpop_j) * (long long)(E->M_An->h.cpop_j - 1) * (long long)(E2->M_An->h.rpop_j - same);
        plusdiv(S, d, AC, T, F->QC_AtTAnAtTAn->lf, (double)lld, S.A_bmc_j.data(), S.T_bmc_j.data());
      }
    }
}

// dra_mds_nrm_s___m_m (dir_c/ra_stats.c:77-85): column 0 of an nrows x
// ncols column-major array loses sum_{c >= 1} d[:, c] / den, in column order.
void dra_mds_nrm(double *d, unsigned long long nrows, unsigned long long ncols, double den,
                 const unsigned char *bmr, const unsigned char *bmc) {
  if (!(den > 0)) return;
  for (unsigned long long r = 0; r < nrows; ++r) {
    if (!bget_on(bmr, (long)r)) continue;
    for (unsigned long long c = 1; c < ncols; ++c)
      if (bget_on(bmc, (long)c)) d[r] -= d[r + c * nrows] / den;
  }
}

// dra_mds_pow_s___m_m (dir_c/ra_stats.c:86-100): for rows whose column-0
// value x >= 0, x becomes x^2 - sum_{c >= 1} d[:, c]^2 / den, then the signed
// square root of that.
void dra_mds_pow(double *d, unsigned long long nrows, unsigned long long ncols, double den,
                 const unsigned char *bmr, const unsigned char *bmc) {
  if (!(den > 0)) return;
  for (unsigned long long r = 0; r < nrows; ++r) {
    if (!bget_on(bmr, (long)r) || !(d[r] >= 0)) continue;
    d[r] *= d[r];
    for (unsigned long long c = 1; c < ncols; ++c)
      if (bget_on(bmc, (long)c)) d[r] -= d[r + c * nrows] * d[r + c * nrows] / den;
    d[r] = d[r] >= 0 ? sqrt(d[r]) : -sqrt(-d[r]);
  }
}

// bcc_sumscores_ifT (bcc_sumscores.c:483-548): the MDS correction of the
// row and column scores for covariate columns 2 and up, with n_mds =
// min(6, T_cpop_j - 1).  The reference sets the scale factor with
//   if (GLOBAL_kappa_squared>0);{ mds_scale_factor = GLOBAL_kappa_squared;}
// -- the statement after the empty `if` always runs -- so the denominator
// is n_mds * GLOBAL_kappa_squared, and the correction does nothing unless
// GLOBAL_kappa_squared is positive.  Kept as is: the outputs must match.
// Only bin pair nb2 = 0 of each nb1 is corrected when GLOBAL_Ireq <= 0.
void sumscores_ifT(State &S) {
  int n_mds = std::max(0, (int)S.T_cpop_j - 1);
  if (n_mds > 6) n_mds = 6;
  if (n_mds <= 0) return;
  const double den = n_mds * S.P.kappa_squared;
  const int nb = S.nbins, T = S.T_ncols;
  const unsigned long long AC = (unsigned long long)S.A_ncols;
  for (int nb1 = 0; nb1 < nb; ++nb1) {
    Single *E = S.E[nb1].get();
    const unsigned long long AN = (unsigned long long)E->A_nrows;
    for (int nb2 = 0; nb2 < (S.P.Ireq > 0 ? nb : 1); ++nb2) {
      const int nbx = nb1 + nb2 * nb;
      if (E->A_rbother && S.A_cbother && E->Z_rbother)
        dra_mds_pow(&E->QR_AnZtSZnAt_nrm[nb2 * AN * T], AN, T, den, E->A_bmr_j.data(), S.T_bmc_j.data());
      if (E->A_rbother && S.A_cbother)
        dra_mds_pow(&E->QR_AnAtTAnAt_nrm[nb2 * AN * T], AN, T, den, E->A_bmr_j.data(), S.T_bmc_j.data());
      if (S.A_rpop_b_total && S.A_cbother && S.Z_rpop_b_total)
        dra_mds_nrm(&S.QC_AtTAnZtSZn_nrm[nbx * AC * T], AC, T, den, S.A_bmc_j.data(), S.T_bmc_j.data());
      if (S.A_cbother && S.A_rpop_b_total)
        dra_mds_nrm(&S.QC_AtTAnAtTAn_nrm[nbx * AC * T], AC, T, den, S.A_bmc_j.data(), S.T_bmc_j.data());
    }
  }
}

// bcc_sumscores_srt (bcc_sumscores.c:358-482), GLOBAL_Ireq > 0: every
// retained row's scores sorted across its bins, every retained column's
// across the bin pairs, each ascending (dQuickSort on the strided values).
void sumscores_srt(State &S) {
  const int nb = S.nbins, T = S.T_ncols;
  const unsigned lim = S.P.recursion_limit;
  for (int nb1 = 0; nb1 < nb; ++nb1) {
    Single *E = S.E[nb1].get();
    const long stride = (long)E->A_nrows * T;
    for (int which = 0; which < 2; ++which) {
      if (!(E->A_rbother && S.A_cbother && (which == 0 ? E->Z_rbother : E->A_rbother))) continue;
      double *v = which == 0 ? E->QR_AnZtSZnAt_nrm.data() : E->QR_AnAtTAnAt_nrm.data();
      for (int ma_a = 0; ma_a < E->A_nrows; ++ma_a)
        if (bget_on(E->A_bmr_b.data(), ma_a) && bget_on(E->A_bmr_j.data(), ma_a))
          dquicksort_strided(lim, &v[ma_a], stride, 0, nb - 1);
    }
  }
  const long stride = (long)S.A_ncols * T;
  for (int which = 0; which < 2; ++which) {
    if (which == 0 ? !(S.A_rpop_b_total && S.A_cbother && S.Z_rpop_b_total) : !(S.A_cbother && S.A_rpop_b_total))
      continue;
    double *v = which == 0 ? S.QC_AtTAnZtSZn_nrm.data() : S.QC_AtTAnAtTAn_nrm.data();
    for (int na_a = 0; na_a < S.A_ncols; ++na_a)
      if (bget_on(S.A_bmc_b.data(), na_a) && bget_on(S.A_bmc_j.data(), na_a))
        dquicksort_strided(lim, &v[na_a], stride, 0, nb * nb - 1);
  }
}

void sumscores_nrm(State &S) {  // bcc_sumscores_nrm (bcc_sumscores.c:550-779)
  if (S.P.Ireq > 0) {
    sumscores_nrm_per_bin(S);
    return;
  }
  const int nb = S.nbins, T = S.T_ncols;
  const bool dcc = dcc_mode(S.P);  // dcc_sumscores_nrm (dcc_sumscores.c:533-573): one fewer column factor
  for (int nb1 = 0; nb1 < nb; ++nb1)
    for (int nb2 = 0; nb2 < nb; ++nb2) {
      const int nbx = nb1 + nb2 * nb;
      Single *E = S.E[nb1].get(), *E2 = S.E[nb2].get();
      Double *F = S.f(nb1, nb2);
      const unsigned long long AN = (unsigned long long)E->A_nrows;
      if (E->A_rbother && S.A_cbother && E2->Z_rbother) {
        double *d = &E->QR_AnZtSZnAt_nrm[nb2 * AN * T];
        memset(d, 0, AN * T * sizeof(double));
        const long long lld = dcc ? (long long)(S.Z_rpop_j_total - 0) * (long long)(E2->M_Zn->h.cpop_j)
                                  : (long long)(S.Z_rpop_j_total - 0) * (long long)(E2->M_Zn->h.cpop_j) * (long long)(E2->M_Zn->h.cpop_j - 1);
        plusdiv(S, d, AN, T, F->QR_AnZtSZnAt->lf, (double)lld, E->A_bmr_j.data(), S.T_bmc_j.data());
      }
      if (E->A_rbother && S.A_cbother && E2->A_rbother) {
        double *d = &E->QR_AnAtTAnAt_nrm[nb2 * AN * T];
        memset(d, 0, AN * T * sizeof(double));
        const long long lld = dcc ? (long long)(S.A_rpop_j_total - 1) * (long long)(E2->M_An->h.cpop_j)
                                  : (long long)(S.A_rpop_j_total - 1) * (long long)(E2->M_An->h.cpop_j) * (long long)(E2->M_An->h.cpop_j - 1);
        plusdiv(S, d, AN, T, F->QR_AnAtTAnAt->lf, (double)lld, E->A_bmr_j.data(), S.T_bmc_j.data());
      }
      const unsigned long long AC = (unsigned long long)S.A_ncols;
      if (E->A_rbother && S.A_cbother && E2->Z_rbother) {
        double *d = &S.QC_AtTAnZtSZn_nrm[nbx * AC * T];
        memset(d, 0, AC * T * sizeof(double));
        const long long lld = dcc ? (long long)(S.A_rpop_j_total) * (long long)(S.Z_rpop_j_total)
                                  : (long long)(S.A_rpop_j_total) * (long long)(E->M_An->h.cpop_j - 1) * (long long)(S.Z_rpop_j_total);
        plusdiv(S, d, AC, T, F->QC_AtTAnZtSZn->lf, (double)lld, S.A_bmc_j.data(), S.T_bmc_j.data());
      }
      if (E->A_rbother && S.A_cbother && E2->A_rbother) {
        double *d = &S.QC_AtTAnAtTAn_nrm[nbx * AC * T];
        memset(d, 0, AC * T * sizeof(double));
        const long long lld = dcc ? (long long)(S.A_rpop_j_total) * (long long)(S.A_rpop_j_total - 1)
                                  : (long long)(S.A_rpop_j_total) * (long long)(E->M_An->h.cpop_j - 1) * (long long)(S.A_rpop_j_total - 1);
        plusdiv(S, d, AC, T, F->QC_AtTAnAtTAn->lf, (double)lld, S.A_bmc_j.data(), S.T_bmc_j.data());
      }
    }
  for (int ns_a = 0; ns_a < T; ++ns_a) {
    if (!bget_on(S.T_bmc_j.data(), ns_a)) continue;
    for (int nb1 = 0; nb1 < nb; ++nb1) {
      Single *E = S.E[nb1].get();
      const unsigned long long AN = (unsigned long long)E->A_nrows;
      if (E->A_rbother && S.A_cbother && E->Z_rbother)
        for_each_on(E->A_bmr_b.data(), E->A_bmr_j.data(), AN, [&](unsigned long long ma) {
          dra_sumx0(&E->QR_AnZtSZnAt_nrm[ma + ns_a * AN], AN * T, nb);
        });
      if (E->A_rbother && S.A_cbother)
        for_each_on(E->A_bmr_b.data(), E->A_bmr_j.data(), AN, [&](unsigned long long ma) {
          dra_sumx0(&E->QR_AnAtTAnAt_nrm[ma + ns_a * AN], AN * T, nb);
        });
    }
    const unsigned long long AC = (unsigned long long)S.A_ncols;
    if (S.A_rpop_b_total && S.A_cbother && S.Z_rpop_b_total)
      for_each_on(S.A_bmc_b.data(), S.A_bmc_j.data(), AC, [&](unsigned long long na) {
        dra_sumx0(&S.QC_AtTAnZtSZn_nrm[na + ns_a * AC], AC * T, (unsigned long long)nb * nb);
      });
    if (S.A_cbother && S.A_rpop_b_total)
      for_each_on(S.A_bmc_b.data(), S.A_bmc_j.data(), AC, [&](unsigned long long na) {
        dra_sumx0(&S.QC_AtTAnAtTAn_nrm[na + ns_a * AC], AC * T, (unsigned long long)nb * nb);
      });
  }
}

void sumscores_cmb(State &S) {  // bcc_sumscores_cmb (bcc_sumscores.c:324-356)
  const unsigned char bmc1 = 255;
  if (S.A_cbother && S.A_rpop_b_total) {
    if (S.A_rpop_b_total && S.A_cbother && S.Z_rpop_b_total)
      for (int nbx = 0; nbx < S.nbins * S.nbins; ++nbx) {
        const size_t o = (size_t)nbx * S.A_ncols * S.T_ncols;
        plustimes(&S.QC_AtTAnAtTAn_nrm[o], S.A_ncols, 1, &S.QC_AtTAnZtSZn_nrm[o], -1.0, S.A_bmc_j.data(), &bmc1);
      }
  }
  for (auto &E : S.E) {
    if (E->A_rbother && S.A_cbother && E->Z_rbother)
      for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
        const size_t o = (size_t)nb2 * E->A_nrows * S.T_ncols;
        plustimes(&E->QR_AnAtTAnAt_nrm[o], E->A_nrows, 1, &E->QR_AnZtSZnAt_nrm[o], -1.0, E->A_bmr_j.data(), &bmc1);
      }
  }
}

// The bins still holding rows (Irem) and xcc_get_Ireq("empty low")
// (bcc_sumscores.c:207-223): the Ireq-th highest of the per-bin (per-bin-pair)
// scores sorted by sumscores_srt, as row / column-pair offsets.
void get_Ireq(State &S, int &Irow, int &Icol) {
  S.Irem = 0;
  for (auto &E : S.E) S.Irem += (E->A_rpop_j > 0 ? 1 : 0);
  S.Ireq = std::max(0, std::min(S.nbins, S.P.Ireq));
  Irow = S.Ireq > 0 ? S.nbins - S.Ireq : 0;
  Icol = S.Ireq > 0 ? S.nbins * S.nbins - S.Ireq * S.Ireq : 0;
}

void sumscores_xij(State &S) {  // bcc_sumscores_xij (bcc_sumscores.c:225-322)
  int Irow = 0, Icol = 0;
  get_Ireq(S, Irow, Icol);
  if (S.A_cbother && S.A_rpop_b_total) {
    int na_b = 0, na_j = 0;
    for (int na_a = 0; na_a < S.A_ncols; ++na_a) {
      if (bget_on(S.A_bmc_b.data(), na_a)) {
        if (bget_on(S.A_bmc_j.data(), na_a)) {
          S.QC_svalue[na_j] = S.QC_AtTAnAtTAn_nrm[na_a + 0 * S.A_ncols + (size_t)Icol * S.A_ncols * S.T_ncols];
          S.QC_index_local_mc_a[na_j] = na_a; S.QC_index_local_mc_b[na_j] = na_b; S.QC_index_local_mc_j[na_j] = na_j;
          na_j++;
        }
        na_b++;
      }
    }
    quicksort_xij(S.P.recursion_limit, S.QC_svalue.data(), S.QC_index_local_mc_a.data(), S.QC_index_local_mc_b.data(),
                  S.QC_index_local_mc_j.data(), nullptr, nullptr, nullptr, 0, (int)S.A_cpop_j - 1);
  }
  if (S.A_rpop_b_total && S.A_cbother) {
    S.A_nrows_total = 0; S.A_rpop_b_total = 0; S.A_rpop_j_total = 0;
    for (int nb1 = 0; nb1 < S.nbins; ++nb1) {
      Single *E = S.E[nb1].get();
      int ma_b = 0, ma_j = 0;
      for (int ma_a = 0; ma_a < E->A_nrows; ++ma_a) {
        if (bget_on(E->A_bmr_b.data(), ma_a)) {
          if (bget_on(E->A_bmr_j.data(), ma_a)) {
            const unsigned t = S.A_rpop_j_total;
            S.QR_svalue[t] = E->QR_AnAtTAnAt_nrm[ma_a + 0 * E->A_nrows + (size_t)Irow * E->A_nrows * S.T_ncols];
            S.QR_index_local_mr_a[t] = ma_a; S.QR_index_local_mr_b[t] = ma_b; S.QR_index_local_mr_j[t] = ma_j;
            S.QR_index_local_nb[t] = nb1;
            S.QR_index_global_mr_a[t] = E->QR_index_global_mr_a[ma_a];
            S.QR_index_global_mr_b[t] = E->QR_index_global_mr_b[ma_a];
            ma_j++; S.A_rpop_j_total++;
          }
          ma_b++; S.A_rpop_b_total++;
        }
        S.A_nrows_total++;
      }
    }
    quicksort_xij(S.P.recursion_limit, S.QR_svalue.data(), S.QR_index_local_mr_a.data(), S.QR_index_local_mr_b.data(),
                  S.QR_index_local_mr_j.data(), S.QR_index_local_nb.data(), S.QR_index_global_mr_a.data(),
                  S.QR_index_global_mr_b.data(), 0, (int)S.A_rpop_j_total - 1);
  }
}

double ra_mean(const double *v, unsigned long long n) {  // ra_stats "double" mean (ra_stats.c:24-25)
  double mean = 0;
  for (unsigned long long i = 0; i < n; ++i) mean += v[i];
  mean /= (double)n;
  return mean;
}

// The elimination choice shared by bcc_sumscores_mxA (bcc_sumscores.c:115-160)
// and bcc_scorebox_mxA (bcc_scorebox.c:5-20): the first cdrop columns of
// QC_index_local_mc_a and the first rdrop rows of QR_index_local_mr_a /
// QR_index_local_nb move from the retained to the removed masks.
void mx_select(State &S, int rdrop, int cdrop) {
  for (int nc = 0; nc < S.A_ncols; ++nc) S.A_umc_j[nc] = (unsigned char)bget_on(S.A_bmc_j.data(), nc);
  for (int nc = 0; nc < S.A_ncols; ++nc) { S.A_umc_j_rtn[nc] = S.A_umc_j[nc]; S.A_umc_j_rmv[nc] = 0; }
  for (int nc = 0; nc < std::min(cdrop, (int)S.A_cpop_j); ++nc) {
    S.A_umc_j_rmv[S.QC_index_local_mc_a[nc]] = 1; S.A_umc_j_rtn[S.QC_index_local_mc_a[nc]] = 0;
  }
  for (auto &E : S.E) {
    for (int nr = 0; nr < E->A_nrows; ++nr) E->A_umr_j[nr] = (unsigned char)bget_on(E->A_bmr_j.data(), nr);
    for (int nr = 0; nr < E->A_nrows; ++nr) { E->A_umr_j_rtn[nr] = E->A_umr_j[nr]; E->A_umr_j_rmv[nr] = 0; }
  }
  for (int nr = 0; nr < std::min(rdrop, (int)S.A_rpop_j_total); ++nr) {
    Single *E = S.E[S.QR_index_local_nb[nr]].get();
    E->A_umr_j_rmv[S.QR_index_local_mr_a[nr]] = 1; E->A_umr_j_rtn[S.QR_index_local_mr_a[nr]] = 0;
  }
}

void sumscores_mxB(State &S) {  // bcc_sumscores_mxB (bcc_sumscores.c:37-91)
  bits_from_ura(S.A_bmc_j, S.A_umc_j, S.A_ncols);
  bits_from_ura(S.A_bmc_j_rmv, S.A_umc_j_rmv, S.A_ncols);
  bits_from_ura(S.A_bmc_j_rtn, S.A_umc_j_rtn, S.A_ncols);
  for (auto &E : S.E) {
    bits_from_ura(E->A_bmr_j, E->A_umr_j, E->A_nrows);
    bits_from_ura(E->A_bmr_j_rmv, E->A_umr_j_rmv, E->A_nrows);
    bits_from_ura(E->A_bmr_j_rtn, E->A_umr_j_rtn, E->A_nrows);
  }
  S.A_cpop_j = popcount_bytes(S.A_bmc_j.data(), S.A_mc_length);
  S.A_cpop_j_rmv = popcount_bytes(S.A_bmc_j_rmv.data(), S.A_mc_length);
  S.A_cpop_j_rtn = popcount_bytes(S.A_bmc_j_rtn.data(), S.A_mc_length);
  for (auto &E : S.E) {
    E->A_rpop_j = popcount_bytes(E->A_bmr_j.data(), E->A_mr_length);
    E->A_rpop_j_rmv = popcount_bytes(E->A_bmr_j_rmv.data(), E->A_mr_length);
    E->A_rpop_j_rtn = popcount_bytes(E->A_bmr_j_rtn.data(), E->A_mr_length);
  }
  lrup_mxset(S);
}

void sumscores_mxA(State &S) {  // bcc_sumscores_mxA / mxB / mxC (bcc_sumscores.c:37-205)
  int rdrop = 0, cdrop = 0;
  get_xdrop(S.P, (double)S.A_rpop_j_total, (double)S.A_cpop_j, &rdrop, &cdrop);
  mx_select(S, rdrop, cdrop);
  sumscores_mxB(S);
  // mxC: trace
  Output &O = *S.out;
  double m = ra_mean(S.QR_svalue.data(), S.A_rpop_j_total);
  const double trace_QR = std::isfinite(m) ? m : 1.0;
  m = ra_mean(S.QC_svalue.data(), S.A_cpop_j);
  const double trace_QC = std::isfinite(m) ? m : 1.0;
  O.trace.push_back((double)O.iterations);
  O.trace.push_back((double)S.A_rpop_j_total);
  O.trace.push_back((double)S.A_cpop_j);
  O.trace.push_back(trace_QR);
  O.trace.push_back(trace_QC);
  O.trace.push_back((double)S.Irem);
  O.iterations++;
  for (int nr = 0; nr < std::min(rdrop, (int)S.A_rpop_j_total); ++nr) {
    O.xdrop_a.push_back(S.QR_index_global_mr_a[nr]); O.xdrop_a.push_back(-1);
    O.xdrop_b.push_back(S.QR_index_global_mr_b[nr]); O.xdrop_b.push_back(-1);
  }
  for (int nc = 0; nc < std::min(cdrop, (int)S.A_cpop_j); ++nc) {
    O.xdrop_a.push_back(-1); O.xdrop_a.push_back(S.QC_index_local_mc_a[nc]);
    O.xdrop_b.push_back(-1); O.xdrop_b.push_back(S.QC_index_local_mc_b[nc]);
  }
}

// --- low-rank update ------------------------------------------------------------

// bcc_lrup_QR_YnWt_stage_2 (bcc_lrup.c:772-861), the condense form of
// stages 0 and 1: the removed columns of every bin as dense centred FP64
// matrices (SNPs x rows), then their FP64 products.
void lrup_QR_condense(State &S) {
  double *aj = S.A_ajdk.data();
  for (auto &E : S.E) {
    if (S.A_cbother && E->A_rbother) wrap_M_At_to_L2_run(TARGS, T_pm, SP_j, SP_b, E->M_jt->p(), aj, &E->lf_jn);
    if (S.A_cbother && E->Z_rbother) wrap_M_At_to_L2_run(TARGS, T_pm, SP_j, SP_b, E->M_vt->p(), aj, &E->lf_vn);
  }
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->Z_rbother) wrap_AnZt_mm__run(TARGS, E1->lf_jn, E2->lf_vn, &F->lf_jnvt);
      if (S.A_cbother && E1->A_rbother && E2->A_rbother && nb1 <= nb2)
        wrap_AnZt_mm__run(TARGS, E1->lf_jn, E2->lf_jn, &F->lf_jnjt);
    }
}

void lrup_QR(State &S) {  // bcc_lrup_QR_YnWt_stage_0/1/3 (bcc_lrup.c:659-892)
  double *aj = S.A_ajdk.data();
  if (qr_condense(S.P)) {
    lrup_QR_condense(S);
  } else {
  S.defer_begin();
  for (auto &E : S.E) {
    if (E->A_rbother && S.A_cbother) wrap_An_ajdk_v(TARGS, T_pm, SP_a, E->M_jn->p(), aj, &E->lf_jn_ajdk);
    if (E->Z_rbother && S.A_cbother) wrap_An_ajdk_v(TARGS, T_pm, SP_a, E->M_vn->p(), aj, &E->lf_vn_ajdk);
  }
  S.defer_end();
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->Z_rbother)
        wrap_AnZt_vv__run(TARGS, T_pm, SP_b, SP_b, E1->M_jn->p(), E2->M_vn->p(), aj, E1->lf_jn_ajdk, E2->lf_vn_ajdk, &F->lf_jnvt);
      if (S.A_cbother && E1->A_rbother && E2->A_rbother) {
        if (nb1 == nb2)
          wrap_AnAt_vv__run(TARGS, T_pm, SP_b, SP_b, E1->M_jn->p(), E2->M_jn->p(), aj, E1->lf_jn_ajdk, E2->lf_jn_ajdk, &F->lf_jnjt);
        if (nb1 < nb2)
          wrap_AnZt_vv__run(TARGS, T_pm, SP_b, SP_b, E1->M_jn->p(), E2->M_jn->p(), aj, E1->lf_jn_ajdk, E2->lf_jn_ajdk, &F->lf_jnjt);
      }
    }
  }
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->A_rbother && nb1 > nb2)
        S.transpose(S.f(nb1, nb2)->lf_jnjt, S.f(nb2, nb1)->lf_jnjt);
    }
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->Z_rbother) S.sub(F->lf_AnZt, F->lf_jnvt);
      if (S.A_cbother && E1->A_rbother && E2->A_rbother) S.sub(F->lf_AnAt, F->lf_jnjt);
    }
}

void lrup_QC(State &S) {  // bcc_lrup_QC_YnWt_stage_a0..a3, b0..b2 (bcc_lrup.c:5-481)
  double *aj = S.A_ajdk.data();
  // a0 (its outputs are read from a1 on: one joined group)
  S.defer_begin();
  for (auto &E : S.E) {
    if (E->A_rbother && S.A_cbother) {
      wrap_An_ajdk_v(TARGS, T_pm, SP_a, E->M_kn->p(), aj, &E->lf_kn_ajdk);
      wrap_An_ajdk_v(TARGS, T_pm, SP_a, E->M_hn->p(), aj, &E->lf_hn_ajdk);
      wrap_An_ajdk_v(TARGS, T_pm, SP_a, E->M_an->p(), aj, &E->lf_an_ajdk);
    }
    if (E->Z_rbother && S.A_cbother) {
      wrap_An_ajdk_v(TARGS, T_pm, SP_a, E->M_zn->p(), aj, &E->lf_zn_ajdk);
      wrap_An_ajdk_v(TARGS, T_pm, SP_a, E->M_vn->p(), aj, &E->lf_vn_ajdk);
    }
  }
  S.defer_end();
  g_clock.tick("lrup_QC_a0");
  // a1
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->Z_rbother) {
        wrap_AnZt_vv__run(TARGS, T_pm, SP_j, SP_j, E1->M_kn->p(), E2->M_zn->p(), aj, E1->lf_kn_ajdk, E2->lf_zn_ajdk, &F->lf_knzt);
        wrap_AnZt_vv__run(TARGS, T_pm, SP_j, SP_j, E1->M_hn->p(), E2->M_vn->p(), aj, E1->lf_hn_ajdk, E2->lf_vn_ajdk, &F->lf_hnvt);
      }
      if (S.A_cbother && E1->A_rbother && E2->A_rbother) {
        wrap_AnZt_vv__run(TARGS, T_pm, SP_j, SP_j, E1->M_an->p(), E2->M_kn->p(), aj, E1->lf_an_ajdk, E2->lf_kn_ajdk, &F->lf_ankt);
        if (nb1 == nb2)
          wrap_AnAt_vv__run(TARGS, T_pm, SP_j, SP_j, E1->M_kn->p(), E2->M_kn->p(), aj, E1->lf_kn_ajdk, E2->lf_kn_ajdk, &F->lf_knkt);
        if (nb1 < nb2)
          wrap_AnZt_vv__run(TARGS, T_pm, SP_j, SP_j, E1->M_kn->p(), E2->M_kn->p(), aj, E1->lf_kn_ajdk, E2->lf_kn_ajdk, &F->lf_knkt);
      }
    }
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2), *Ft = S.f(nb2, nb1);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->A_rbother) {
        S.transpose(F->lf_knat, Ft->lf_ankt);
        if (nb1 > nb2) S.transpose(F->lf_knkt, Ft->lf_knkt);
      }
    }
  g_clock.tick("lrup_QC_a1");
  // a2: the quantisations of every bin pair, one joined group (their planes
  // and scalars are read from a3 on)
  S.defer_begin();
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->Z_rbother) {
        xcalc_excerpt(S, F->M_knzt_trm, E1->M_kn, E2->M_zn, F->lf_knzt, F->M_knzt);
        xcalc_excerpt(S, F->M_hnvt_trm, E1->M_hn, E2->M_vn, F->lf_hnvt, F->M_hnvt);
      }
      if (S.A_cbother && E1->A_rbother && E2->A_rbother) {
        xcalc_excerpt(S, F->M_ankt_trm, E1->M_an, E2->M_kn, F->lf_ankt, F->M_ankt);
        if (nb1 <= nb2) xcalc_excerpt(S, F->M_knkt_trm, E1->M_kn, E2->M_kn, F->lf_knkt, F->M_knkt);
      }
    }
  S.defer_end();
  g_clock.tick("lrup_QC_a2");
  // a3: independent bit-plane products of every bin pair, one joined group
  S.defer_begin();
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->Z_rbother) {
        bitplane_excerpt(S, F->M_knzt_trm, E1->M_kt, E1->M_rt, E1->M_kn, E2->M_zn, E2->M_St, E2->M_zt, F->M_knzt, &F->lf_kt_r_knzt_s_zn);
        bitplane_excerpt(S, F->M_hnvt_trm, E1->M_kt, E1->M_rt, E1->M_hn, E2->M_vn, E2->M_St, E2->M_zt, F->M_hnvt, &F->lf_kt_r_hnvt_s_zn);
      }
      if (S.A_cbother && E1->A_rbother && E2->A_rbother) {
        bitplane_excerpt(S, F->M_ankt_trm, E1->M_at, E1->M_tt, E1->M_an, E2->M_kn, E2->M_rt, E2->M_kt, F->M_ankt, &F->lf_at_t_ankt_r_kn);
        if (nb1 <= nb2)
          bitplane_excerpt(S, F->M_knkt_trm, E1->M_kt, E1->M_rt, E1->M_kn, E2->M_kn, E2->M_rt, E2->M_kt, F->M_knkt, &F->lf_kt_r_knkt_r_kn);
      }
    }
  S.defer_end();
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2), *Ft = S.f(nb2, nb1);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->A_rbother) {
        lh_duplicate(F->lf_kt_r_knat_t_an, Ft->lf_at_t_ankt_r_kn);
        if (nb1 > nb2) lh_duplicate(F->lf_kt_r_knkt_r_kn, Ft->lf_kt_r_knkt_r_kn);
      }
    }
  g_clock.tick("lrup_QC_a3");
  // b0 (its outputs are read from b1 on: one joined group)
  S.defer_begin();
  for (auto &E : S.E) {
    if (E->A_rbother && S.A_cbother) {
      wrap_AnZt_vv__run(TARGS, T_pm, SP_a, SP_a, E->M_at->p(), E->M_tt->p(), nullptr, nullptr, nullptr, &E->lf_attn);
      wrap_AnZt_vv__run(TARGS, T_pm, SP_a, SP_a, E->M_jt->p(), E->M_tt->p(), nullptr, nullptr, nullptr, &E->lf_jttn);
      wrap_AnZt_vv__run(TARGS, T_pm, SP_a, SP_a, E->M_kt->p(), E->M_rt->p(), nullptr, nullptr, nullptr, &E->lf_ktrn);
      wrap_AnZt_vv__run(TARGS, T_pm, SP_a, SP_a, E->M_ht->p(), E->M_rt->p(), nullptr, nullptr, nullptr, &E->lf_htrn);
    }
    if (E->Z_rbother && S.A_cbother) {
      wrap_AnZt_vv__run(TARGS, T_pm, SP_a, SP_a, E->M_zt->p(), E->M_St->p(), nullptr, nullptr, nullptr, &E->lf_ztsn);
      wrap_AnZt_vv__run(TARGS, T_pm, SP_a, SP_a, E->M_vt->p(), E->M_St->p(), nullptr, nullptr, nullptr, &E->lf_vtsn);
    }
  }
  S.defer_end();
  g_clock.tick("lrup_QC_b0");
  // b1
  for (auto &E : S.E) {
    if (E->Z_rbother && S.A_cbother)
      wrap_AtTYn_vv__run(TARGS, SP_j, SP_j, SP_j, E->M_zt->p(), E->M_St->p(), E->M_vt->p(), aj, aj, E->lf_ztsn, E->lf_vtsn, &E->lf_ztsvn);
    if (E->A_rbother && S.A_cbother) {
      wrap_AtTYn_vv__run(TARGS, SP_j, SP_j, SP_j, E->M_at->p(), E->M_tt->p(), E->M_jt->p(), aj, aj, E->lf_attn, E->lf_jttn, &E->lf_attjn);
      wrap_AtTYn_vv__run(TARGS, SP_j, SP_j, SP_j, E->M_kt->p(), E->M_rt->p(), E->M_ht->p(), aj, aj, E->lf_ktrn, E->lf_htrn, &E->lf_ktrhn);
    }
    // The SNP x SNP products are read only by the next stage's kernels: keep
    // them on the device from their first (allocating) call on.
    S.mirror(E->lf_ztsvn); S.mirror(E->lf_attjn); S.mirror(E->lf_ktrhn);
  }
  g_clock.tick("lrup_QC_b1");
  // b2: independent products of every bin pair, one joined group
  S.defer_begin();
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->Z_rbother)
        wrap_AtTYn____WtSZn_vv__run(TARGS, SP_a, SP_a, E1->M_at->p(), E1->M_tt->p(), E1->M_jt->p(), E2->M_vt->p(), E2->M_St->p(), E2->M_zt->p(), aj, E1->lf_attjn, E2->lf_ztsvn, &F->lf_attjn____vtszn);
      if (S.A_cbother && E1->A_rbother && E2->A_rbother) {
        if (nb1 <= nb2)
          wrap_AtTYn____WtSZn_vv__run(TARGS, SP_a, SP_a, E1->M_at->p(), E1->M_tt->p(), E1->M_jt->p(), E2->M_jt->p(), E2->M_tt->p(), E2->M_at->p(), aj, E1->lf_attjn, E2->lf_attjn, &F->lf_attjn____jttan);
        wrap_AtTYn____WtSZn_vv__run(TARGS, SP_a, SP_a, E1->M_at->p(), E1->M_tt->p(), E1->M_jt->p(), E2->M_ht->p(), E2->M_rt->p(), E2->M_kt->p(), aj, E1->lf_attjn, E2->lf_ktrhn, &F->lf_attjn____htrkn);
        if (nb1 <= nb2)
          wrap_AtTYn____WtSZn_vv__run(TARGS, SP_a, SP_a, E1->M_kt->p(), E1->M_rt->p(), E1->M_ht->p(), E2->M_ht->p(), E2->M_rt->p(), E2->M_kt->p(), aj, E1->lf_ktrhn, E2->lf_ktrhn, &F->lf_ktrhn____htrkn);
      }
    }
  S.defer_end();
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2), *Ft = S.f(nb2, nb1);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->A_rbother) {
        if (nb1 > nb2) lh_duplicate(F->lf_attjn____jttan, Ft->lf_attjn____jttan);
        lh_duplicate(F->lf_ktrhn____jttan, Ft->lf_attjn____htrkn);
        if (nb1 > nb2) lh_duplicate(F->lf_ktrhn____htrkn, Ft->lf_ktrhn____htrkn);
      }
    }
}

void lrup_mxdup(State &S) {  // bcc_lrup_mxdup (bcc_lrup.c:1128-1138)
  S.A_bmc_j = S.A_bmc_j_rtn;
  for (int i = 0; i < S.A_ncols; ++i) S.A_umc_j[i] = S.A_umc_j_rtn[i];
  for (auto &E : S.E) {
    E->A_bmr_j = E->A_bmr_j_rtn;
    for (int i = 0; i < E->A_nrows; ++i) E->A_umr_j[i] = E->A_umr_j_rtn[i];
  }
}

// The indices of a mask pair as L2_clean / LL2_plustimes walk them: for each
// index a in [0, n), in order, its j / b / a positions, split into those in
// both masks (kept), in mc_b only (b_not_j) and outside mc_b (not_b).
struct MaskWalk {
  std::vector<unsigned long long> kj, kb, ka, bj, bb, ba, nj, nb_, na;
  MaskWalk(unsigned long long n, const unsigned char *mb, const unsigned char *mj) {
    unsigned long long j = 0, b = 0;
    for (unsigned long long a = 0; a < n; ++a) {
      if (bget_on(mb, (long)a)) {
        if (bget_on(mj, (long)a)) { kj.push_back(j); kb.push_back(b); ka.push_back(a); ++j; }
        else { bj.push_back(j); bb.push_back(b); ba.push_back(a); }
        ++b;
      } else {
        nj.push_back(j); nb_.push_back(b); na.push_back(a);
      }
    }
  }
  // the kept indices in the given spacing
  const unsigned long long *kept(int spacing) const {
    return spacing == SP_j ? kj.data() : spacing == SP_b ? kb.data() : ka.data();
  }
};

// bcc_lrup_QC_YnWt_stage_c (bcc_lrup.c:592-655): L2_clean and the
// LL2_plustimes subtractions of each column product, on index lists built
// once per call from the masks.  Each element sees the same operations in
// the same order as the element-by-element walk (its clearing, then the
// subtractions in list order), so the results are identical.
void stage_c_update(L_handle *LA, std::initializer_list<L_handle *> LBs, const MaskWalk &R, const MaskWalk &Cw) {
  const unsigned long long rs = LA->row_stride;
  // L2_clean (L_init.c:287-326)
  const int sr = LA->spacing_row, sc = LA->spacing_col;
  for (size_t c = 0; c < Cw.ka.size(); ++c) {
    const unsigned long long tc = pick(sc, Cw.kj[c], Cw.kb[c], Cw.ka[c]) * rs;
    if (sr == SP_b || sr == SP_a)
      for (size_t r = 0; r < R.ba.size(); ++r) LA->lf[pick(sr, R.bj[r], R.bb[r], R.ba[r]) + tc] = 0;
    if (sr == SP_a)
      for (size_t r = 0; r < R.na.size(); ++r) LA->lf[R.na[r] + tc] = 0;
  }
  if (sc == SP_b || sc == SP_a)
    for (size_t c = 0; c < Cw.ba.size(); ++c) {
      const unsigned long long tc = pick(sc, Cw.bj[c], Cw.bb[c], Cw.ba[c]) * rs;
      for (unsigned long long r = 0; r < rs; ++r) LA->lf[r + tc] = 0;
    }
  if (sc == SP_a)
    for (size_t c = 0; c < Cw.na.size(); ++c)
      for (unsigned long long r = 0; r < rs; ++r) LA->lf[r + Cw.na[c] * rs] = 0;
  // LL2_plustimesequals with multiplier -1 (L_init.c:328-358), all sources
  // of one element in turn
  const size_t nlb = LBs.size();
  std::vector<const double *> base(nlb);
  std::vector<const unsigned long long *> rsel(nlb);
  std::vector<unsigned long long> lrs(nlb);
  const unsigned long long *rA = R.kept(sr);
  for (size_t c = 0; c < Cw.ka.size(); ++c) {
    double *colA = LA->lf + pick(sc, Cw.kj[c], Cw.kb[c], Cw.ka[c]) * rs;
    size_t k = 0;
    for (L_handle *LB : LBs) {
      base[k] = LB->lf + pick(LB->spacing_col, Cw.kj[c], Cw.kb[c], Cw.ka[c]) * LB->row_stride;
      rsel[k] = R.kept(LB->spacing_row);
      ++k;
    }
    for (size_t r = 0; r < R.ka.size(); ++r) {
      double v = colA[rA[r]];
      for (size_t q = 0; q < nlb; ++q) v += -1.0 * base[q][rsel[q][r]];
      colA[rA[r]] = v;
    }
  }
}

void lrup_QC_stage_c(State &S) {  // bcc_lrup_QC_YnWt_stage_c (bcc_lrup.c:592-655)
  const MaskWalk R(S.A_ncols, S.A_bmc_b.data(), S.A_bmc_j_rtn.data()), Cw(S.T_ncols, S.T_bmc_b.data(), S.T_bmc_j.data());
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (S.A_cbother && E1->A_rbother && E2->Z_rbother)
        stage_c_update(F->lf_At_T_AnZt_S_Zn, {F->lf_attjn____vtszn, F->lf_kt_r_knzt_s_zn, F->lf_kt_r_hnvt_s_zn}, R, Cw);
      if (S.A_cbother && E1->A_rbother && E2->A_rbother)
        stage_c_update(F->lf_At_T_AnAt_T_An,
                       {F->lf_attjn____jttan, F->lf_attjn____htrkn, F->lf_ktrhn____jttan, F->lf_ktrhn____htrkn,
                        F->lf_at_t_ankt_r_kn, F->lf_kt_r_knat_t_an, F->lf_kt_r_knkt_r_kn},
                       R, Cw);
    }
}

// Optional stage trace (LAKBCC_TRACE=<file>): after every stage, one line
// per live intermediate with an FNV-1a hash of its values.  Two builds whose
// kernels agree bit for bit write identical traces, so the first differing
// line names the stage and the product that diverged.
unsigned long long fnv(const void *p, size_t n, unsigned long long h = 1469598103934665603ull) {
  const unsigned char *b = (const unsigned char *)p;
  for (size_t i = 0; i < n; ++i) { h ^= b[i]; h *= 1099511628211ull; }
  return h;
}

thread_local const Hooks *g_trace_hooks = nullptr;

void trace_L(FILE *f, const char *stage, int it, const char *name, int a, int b, const L_handle *L) {
  if (!L) return;
  if (g_trace_hooks && g_trace_hooks->L_to_host) g_trace_hooks->L_to_host(const_cast<L_handle *>(L));
  unsigned long long n = L->row_stride * L->col_stride * (L->lyr_stride ? L->lyr_stride : 1);
  if (n > L->length) n = L->length;
  fprintf(f, "%s %d %s %d %d n=%llu h=%016llx\n", stage, it, name, a, b, n, fnv(L->lf, n * sizeof(double)));
}

void trace_M(FILE *f, const char *stage, int it, const char *name, int a, int b, const MH *M) {
  if (!M) return;
  const M_handle &h = M->h;
  unsigned long long x = fnv(h.wX, (size_t)h.nrows * h.mc_length);
  x = fnv(&h.min_d, sizeof(double), x);
  x = fnv(&h.mlt_d, sizeof(double), x);
  fprintf(f, "%s %d %s %d %d rows=%d h=%016llx\n", stage, it, name, a, b, h.nrows, x);
}


void trace_stage(State &S, const char *stage) {
  g_clock.tick(stage);
  thread_local FILE *f = nullptr;
  thread_local bool checked = false;
  if (!checked) {
    checked = true;
    const char *path = getenv("LAKBCC_TRACE");
    if (path && *path) f = fopen(path, "w");
  }
  if (!f) return;
  g_trace_hooks = S.hooks;
  const int it = S.out ? S.out->iterations : -1;
#define TL(name, a, b, L) trace_L(f, stage, it, name, a, b, L)
  for (auto &E : S.E) {
    const int nb = E->nb;
    TL("An_ajdk", nb, 0, E->lf_An_ajdk); TL("Zn_ajdk", nb, 0, E->lf_Zn_ajdk);
    TL("AtTn", nb, 0, E->lf_AtTn); TL("ZtSn", nb, 0, E->lf_ZtSn); TL("At_An_a1d1", nb, 0, E->lf_At_An_a1d1);
    TL("jn_ajdk", nb, 0, E->lf_jn_ajdk); TL("vn_ajdk", nb, 0, E->lf_vn_ajdk); TL("kn_ajdk", nb, 0, E->lf_kn_ajdk);
    TL("zn_ajdk", nb, 0, E->lf_zn_ajdk); TL("hn_ajdk", nb, 0, E->lf_hn_ajdk); TL("an_ajdk", nb, 0, E->lf_an_ajdk);
    TL("attn", nb, 0, E->lf_attn); TL("jttn", nb, 0, E->lf_jttn); TL("ktrn", nb, 0, E->lf_ktrn);
    TL("htrn", nb, 0, E->lf_htrn); TL("ztsn", nb, 0, E->lf_ztsn); TL("vtsn", nb, 0, E->lf_vtsn);
    TL("ztsvn", nb, 0, E->lf_ztsvn); TL("attjn", nb, 0, E->lf_attjn); TL("ktrhn", nb, 0, E->lf_ktrhn);
    TL("At_rsum", nb, 0, E->lf_At_rsum); TL("Zt_rsum", nb, 0, E->lf_Zt_rsum);
    trace_M(f, stage, it, "M_An_a1d1", nb, 0, E->M_An_a1d1);
    trace_M(f, stage, it, "M_a2d2_ZtSn", nb, 0, E->M_a2d2_ZtSn);
    trace_M(f, stage, it, "M_a2d2_AtTn", nb, 0, E->M_a2d2_AtTn);
  }
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      TL("AnZt", nb1, nb2, F->lf_AnZt); TL("AnAt", nb1, nb2, F->lf_AnAt);
      TL("jnvt", nb1, nb2, F->lf_jnvt); TL("jnjt", nb1, nb2, F->lf_jnjt);
      TL("knzt", nb1, nb2, F->lf_knzt); TL("hnvt", nb1, nb2, F->lf_hnvt); TL("ankt", nb1, nb2, F->lf_ankt);
      TL("knat", nb1, nb2, F->lf_knat); TL("knkt", nb1, nb2, F->lf_knkt);
      TL("kt_r_knzt_s_zn", nb1, nb2, F->lf_kt_r_knzt_s_zn); TL("kt_r_hnvt_s_zn", nb1, nb2, F->lf_kt_r_hnvt_s_zn);
      TL("at_t_ankt_r_kn", nb1, nb2, F->lf_at_t_ankt_r_kn); TL("kt_r_knkt_r_kn", nb1, nb2, F->lf_kt_r_knkt_r_kn);
      TL("attjn____vtszn", nb1, nb2, F->lf_attjn____vtszn); TL("attjn____jttan", nb1, nb2, F->lf_attjn____jttan);
      TL("attjn____htrkn", nb1, nb2, F->lf_attjn____htrkn); TL("ktrhn____htrkn", nb1, nb2, F->lf_ktrhn____htrkn);
      TL("AnZt_S_ZnAt", nb1, nb2, F->lf_AnZt_S_ZnAt); TL("AnAt_T_AnAt", nb1, nb2, F->lf_AnAt_T_AnAt);
      TL("At_T_AnZt_S_Zn", nb1, nb2, F->lf_At_T_AnZt_S_Zn); TL("At_T_AnAt_T_An", nb1, nb2, F->lf_At_T_AnAt_T_An);
      TL("An_a2d2_Zt_Sn", nb1, nb2, F->lf_An_a2d2_Zt_Sn); TL("An_a2d2_At_Tn", nb1, nb2, F->lf_An_a2d2_At_Tn);
      TL("QR_AnZtSZnAt", nb1, nb2, F->QR_AnZtSZnAt); TL("QR_AnAtTAnAt", nb1, nb2, F->QR_AnAtTAnAt);
      TL("QC_AtTAnZtSZn", nb1, nb2, F->QC_AtTAnZtSZn); TL("QC_AtTAnAtTAn", nb1, nb2, F->QC_AtTAnAtTAn);
      trace_M(f, stage, it, "M_AnZt", nb1, nb2, F->M_AnZt); trace_M(f, stage, it, "M_AnAt", nb1, nb2, F->M_AnAt);
      trace_M(f, stage, it, "M_knzt", nb1, nb2, F->M_knzt); trace_M(f, stage, it, "M_hnvt", nb1, nb2, F->M_hnvt);
      trace_M(f, stage, it, "M_ankt", nb1, nb2, F->M_ankt); trace_M(f, stage, it, "M_knkt", nb1, nb2, F->M_knkt);
    }
#undef TL
  fflush(f);
}

void initial_subscores(State &S) {  // lakcluster_driver.c:70-100
  An_ajdk_all(S); trace_stage(S, "An_ajdk");
  lf_ZtSn_all(S); trace_stage(S, "lf_ZtSn");
  lf_ZtSWn_all(S); trace_stage(S, "lf_ZtSWn");
  lf_YnWt_all(S); trace_stage(S, "lf_YnWt");
  if (qc_ynwt(S)) { M_YnWt_all(S); trace_stage(S, "M_YnWt"); }
  lf_AtTYn____WtSZn_all(S); trace_stage(S, "lf_AtTYn____WtSZn");
  if (qc_ynwt(S)) { lf_At_T_YnWt_S_Zn_all(S); trace_stage(S, "lf_At_T_YnWt_S_Zn"); }
  lf_AnZt_S_WnYt_all(S); trace_stage(S, "lf_AnZt_S_WnYt");
  singlestudy_ww(S); trace_stage(S, "singlestudy");
  doublestudy_ww(S); trace_stage(S, "doublestudy");
  flattenloop(S); trace_stage(S, "flattenloop");
}

// ---------------------------------------------------------------------------
// out_xdrop lists (dir_c/bcc_scorebox.c:125-180, dir_c/R_init.c:216-262)

// xcc_out_xdrop_sort: the row indices (first entries >= 0) and the column
// indices (second entries >= 0) of out_xdrop lines, in line order.
void xdrop_lists(const std::vector<int> &pairs, std::vector<int> &rows, std::vector<int> &cols) {
  rows.clear(); cols.clear();
  for (size_t l = 0; l + 1 < pairs.size(); l += 2) {
    if (pairs[l] >= 0) rows.push_back(pairs[l]);
    if (pairs[l + 1] >= 0) cols.push_back(pairs[l + 1]);
  }
}

// bcc_out_xdrop_lkp: global row indices (bins concatenated) to (bin, row).
int xdrop_lookup(const State &S, const std::vector<int> &rows, std::vector<int> &lnb, std::vector<int> &lmr,
                 std::string &err) {
  lnb.assign(rows.size(), 0); lmr.assign(rows.size(), 0);
  for (size_t l = 0; l < rows.size(); ++l) {
    int r = rows[l], nb = 0;
    while (nb < S.nbins && r >= S.E[nb]->A_nrows) { r -= S.E[nb]->A_nrows; ++nb; }
    if (nb >= S.nbins || r < 0) { err = "out_xdrop row index " + std::to_string(rows[l]) + " out of range"; return 2; }
    lnb[l] = nb; lmr[l] = r;
  }
  return 0;
}

// R01GET (dir_c/boxmuller.c:57-65): seed <- seed*35 mod (2^31-1), drawn as
// (double)((long double)seed / (long double)(2^31-1)).  The reference runs on
// x86-64, whose long double has a 64-bit significand, so the quotient is
// rounded to 64 significant bits and then to 53.  The same two roundings are
// done here in integer arithmetic, so that every host draws the same doubles.
// The quotient s/M never terminates in binary (M is an odd prime, 0 < s < M),
// so the first rounding meets no ties.
double r01_next(unsigned long long *seed) {
  const unsigned long long M = 2147483647ULL;
  *seed = (*seed * 35ULL) % M;
  const unsigned long long s = *seed;
  if (s == 0) return 0.0;
  int k = 0;  // 2^-k <= s/M < 2^(1-k)
  while (((unsigned __int128)s << k) < M) ++k;
  const unsigned __int128 q = ((unsigned __int128)s << (k + 64)) / M;  // in [2^64, 2^65)
  unsigned __int128 m64 = (q + 1) >> 1;                                 // 64-bit significand
  if (m64 >> 64) { m64 >>= 1; --k; }
  unsigned long long m = (unsigned long long)m64;
  const unsigned long long low = m & 0x7FFULL;
  unsigned long long m53 = m >> 11;
  if (low > 0x400ULL || (low == 0x400ULL && (m53 & 1ULL))) ++m53;
  if (m53 >> 53) { m53 >>= 1; --k; }
  return ldexp((double)m53, -k - 52);
}

// bcc_scramble (dir_c/R_init.c:165-207) after bcc_out_xdrop_prune /
// bcc_out_xdrop_lkp (R_init.c:216-262, bcc_scorebox.c:100-123): every case
// entry in a row and a column listed by out_xdrop (rows and columns each in
// ascending order, those outside the row / column masks dropped) is redrawn,
// set when an R01GET draw falls below that column's frequency among the
// controls (Zt row sums over the control count), in row-major order.  Both
// the case rows (An) and their transpose (At) are changed.  Where a listed
// row or column is outside the retained masks the reference's index walk
// runs past its arrays; here that row / the remaining columns are skipped.
int scramble(State &S, const Input::Scramble &sc, std::string &err) {
  for (auto &E : S.E) {
    memset(E->lf_Zt_rsum->lf, 0, sizeof(double) * E->lf_Zt_rsum->length);
    wrap_An_v__run(TARGS, LAKGB_TYPE_00, SP_a, E->M_Zt->p(), &E->lf_Zt_rsum);
  }
  std::vector<int> rows, cols;
  xdrop_lists(sc.xdrop, rows, cols);
  std::sort(rows.begin(), rows.end());
  std::sort(cols.begin(), cols.end());
  std::vector<int> keep_c, keep_r;
  for (int c : cols)
    if (c >= 0 && c < S.A_ncols && bget_on(S.A_bmc_b.data(), c)) keep_c.push_back(c);
  for (int r : rows) {
    if (r < 0 || r >= S.A_nrows_total) continue;
    int x = r, nb = 0;
    while (x >= S.E[nb]->A_nrows) { x -= S.E[nb]->A_nrows; ++nb; }
    if (bget_on(S.E[nb]->A_bmr_b.data(), x)) keep_r.push_back(r);
  }
  std::vector<int> lnb, lmr;
  int rc = xdrop_lookup(S, keep_r, lnb, lmr, err);
  if (rc) return rc;
  unsigned long long seed = sc.rseed;
  std::vector<int> ma_j(S.nbins, 0);
  int nb = 0;
  for (size_t mx = 0; mx < keep_r.size(); ++mx) {
    while (nb < lnb[mx]) ++nb;
    Single *E = S.E[nb].get();
    M_handle &An = E->M_An->h, &At = E->M_At->h;
    while (ma_j[nb] < (int)An.rpop_j && (int)An.m_a_[ma_j[nb]] < lmr[mx]) ++ma_j[nb];
    if (ma_j[nb] >= (int)An.rpop_j) continue;
    const unsigned ma_a = An.m_a_[ma_j[nb]], ma_b = An.m_b_[ma_j[nb]];
    unsigned char *An_tag = An.wX + (size_t)ma_b * An.mc_length;
    int na_j = 0;
    const double zr = (double)E->M_Zn->h.rpop_b;
    for (size_t nx = 0; nx < keep_c.size(); ++nx) {
      while (na_j < (int)An.cpop_j && (int)An.n_a_[na_j] < keep_c[nx]) ++na_j;
      if (na_j >= (int)An.cpop_j) break;
      const unsigned na_a = An.n_a_[na_j], na_b = An.n_b_[na_j];
      unsigned char *At_tag = At.wX + (size_t)na_b * At.mc_length;
      const bool on = r01_next(&seed) < E->lf_Zt_rsum->lf[na_a] / zr;
      if (on) { bset_on(An_tag, na_a); bset_on(At_tag, ma_a); }
      else { bset_off(An_tag, na_a); bset_off(At_tag, ma_a); }
    }
  }
  // the device copies of the case rows are stale now
  for (auto &E : S.E) { S.forget(E->An_w); S.forget(E->At_w); }
  return 0;
}

// The packed case rows as wrap_bcc_scramble writes them around the scrambles
// (R_init.c:268-289 with binary_write, binary_read.c:57-81): a header of
// three ints (16, bits per record, records) and each record's bits rounded
// up to 16; At_<bin>_scramble_* holds the rows of An, An_<bin>_* those of At.
void scramble_snapshot(State &S, const char *when) {
  auto b16 = [](const M_handle &M) {
    const int bitj = BITJ, nrows = M.ncols, ncols = (int)M.rpop_b;
    const long wp = (long)(nrows + (bitj - nrows % bitj) % bitj) / 8;
    std::vector<unsigned char> f(12 + (size_t)wp * ncols);
    memcpy(&f[0], &bitj, 4); memcpy(&f[4], &nrows, 4); memcpy(&f[8], &ncols, 4);
    for (int c = 0; c < ncols; ++c) memcpy(&f[12 + (size_t)c * wp], M.wX + (size_t)c * bsize(nrows), wp);
    return f;
  };
  for (auto &E : S.E) {
    char name[64];
    snprintf(name, sizeof name, "At_%.2d_scramble_%s.b16", E->nb, when);
    S.out->files.emplace_back(name, b16(E->M_An->h));
    snprintf(name, sizeof name, "An_%.2d_scramble_%s.b16", E->nb, when);
    S.out->files.emplace_back(name, b16(E->M_At->h));
  }
}

// ---------------------------------------------------------------------------
// scorebox (dir_c/lakcluster_scorebox.c, dir_c/bcc_scorebox.c)

// xcc_scorebox_xdrop_array (bcc_scorebox.c:283-308): x_num values from x_max
// down to 0 and the number of indices removed to reach each.
void scorebox_xdrop_array(int nxols, int x_max, int x_num, std::vector<int> &xval, std::vector<int> &xdrop) {
  xval.assign(std::max(0, x_num), 0);
  xdrop.assign(std::max(0, x_num), 0);
  if (x_num <= 0) return;
  const double d = (double)(x_max - 0) / (double)std::max(1, x_num - 1);
  for (int nx = 0; nx < x_num; ++nx) xval[nx] = (int)round(x_max - nx * d);
  xdrop[0] = std::max(0, nxols - (x_max + 1));
  for (int nx = 1; nx < x_num; ++nx) xdrop[nx] = xval[nx - 1] - xval[nx];
}

struct ScoreboxLists {
  std::vector<int> rows, cols, lnb, lmr;
};

// bcc_scorebox_srt (bcc_scorebox.c:82-98): the elimination order of the rows
// and columns still retained is the tail of the out_xdrop lists.
void scorebox_srt(State &S, const ScoreboxLists &L) {
  const int ncols = (int)L.cols.size(), nrows = (int)L.rows.size();
  if (ncols >= (int)S.A_cpop_j)
    for (int j = 0; j < (int)S.A_cpop_j; ++j) S.QC_index_local_mc_a[j] = L.cols[ncols - S.A_cpop_j + j];
  if (nrows >= (int)S.A_rpop_j_total)
    for (int r = 0; r < (int)S.A_rpop_j_total; ++r) {
      S.QR_index_local_mr_a[r] = L.lmr[nrows - S.A_rpop_j_total + r];
      S.QR_index_local_nb[r] = L.lnb[nrows - S.A_rpop_j_total + r];
    }
}

void scorebox_mxA(State &S, int rdrop, int cdrop) {  // bcc_scorebox_mxA (bcc_scorebox.c:5-49)
  mx_select(S, rdrop, cdrop);
  sumscores_mxB(S);
}

// bcc_scorebox_svalue (bcc_scorebox.c:51-80): the selection scores of
// sumscores_xij without the sort.
void scorebox_svalue(State &S) {
  int Irow = 0, Icol = 0;
  get_Ireq(S, Irow, Icol);
  if (S.A_cbother && S.A_rpop_b_total) {
    int na_j = 0;
    for (int na_a = 0; na_a < S.A_ncols; ++na_a)
      if (bget_on(S.A_bmc_b.data(), na_a) && bget_on(S.A_bmc_j.data(), na_a))
        S.QC_svalue[na_j++] = S.QC_AtTAnAtTAn_nrm[na_a + 0 * S.A_ncols + (size_t)Icol * S.A_ncols * S.T_ncols];
  }
  if (S.A_rpop_b_total && S.A_cbother) {
    S.A_nrows_total = 0; S.A_rpop_b_total = 0; S.A_rpop_j_total = 0;
    for (auto &E : S.E) {
      for (int ma_a = 0; ma_a < E->A_nrows; ++ma_a) {
        if (bget_on(E->A_bmr_b.data(), ma_a)) {
          if (bget_on(E->A_bmr_j.data(), ma_a))
            S.QR_svalue[S.A_rpop_j_total++] = E->QR_AnAtTAnAt_nrm[ma_a + 0 * E->A_nrows + (size_t)Irow * E->A_nrows * S.T_ncols];
          S.A_rpop_b_total++;
        }
        S.A_nrows_total++;
      }
    }
  }
}

void scorebox_scores(State &S) {  // the scoring tail of lakcluster_scorebox_excerpt_1/2
  sumscores_nrm(S);
  sumscores_ifT(S);
  if (S.P.Ireq > 0) sumscores_srt(S);
  sumscores_cmb(S);
  scorebox_svalue(S);
}

void dcc_subscores(State &S);

// lakcluster_scorebox_excerpt_1 (lakcluster_scorebox.c:22-52): the loop
// subscores computed directly; for dexcluster its sub-scores
// (dexcluster_scorebox_excerpt_1, dir_c/dexcluster_scorebox.c:21-43).
void scorebox_full(State &S) {
  if (dcc_mode(S.P)) dcc_subscores(S);
  else initial_subscores(S);
  scorebox_scores(S);
}

// lakcluster_scorebox_excerpt_2 (lakcluster_scorebox.c:54-101): the loop
// subscores after a removal, by the low-rank update of the elimination loop.
void scorebox_update(State &S) {
  if (dcc_mode(S.P)) {  // dexcluster_scorebox_excerpt_2 (dir_c/dexcluster_scorebox.c:45-65): recomputed
    lrup_mxdup(S);
    M_mxset_all(S);
    dcc_subscores(S);
    scorebox_scores(S);
    return;
  }
  lrup_QR(S);
  lrup_QC_ZtSWn(S);
  if (qc_ynwt(S)) lrup_QC(S);
  lrup_mxdup(S);
  M_mxset_all(S);
  lf_AtTYn____WtSZn_all(S);
  if (qc_ynwt(S)) lrup_QC_stage_c(S);
  lf_AnZt_S_WnYt_all(S);
  An_ajdk_all(S);
  lf_ZtSn_all(S);
  singlestudy_ww(S);
  doublestudy_ww(S);
  flattenloop(S);
  scorebox_scores(S);
}

// ---------------------------------------------------------------------------
// dexcluster (dcc): the half-loop method of dir_c/dexcluster_driver.c on the
// same state -- one pass of row and column sub-scores per elimination step,
// recomputed each step (no low-rank update).  The dcc score arrays reuse the
// bcc ones of the same shape and role: QR_AnZtSZnAt(_nrm) holds QR_TAnZtS,
// QR_AnAtTAnAt QR_TAnAtT, QC_AtTAnZtSZn QC_TAnZtS, QC_AtTAnAtTAn QC_TAnAtT.

// get_D_AtTn_ZtSn_vv / get_D_AtTn_AtTn_vv (dir_c/D_AtTn_ZtSn.c:5-110,
// :152-270), output spacing a x a: for every retained covariate ns and row
// na of At, ((AtTn - etT a) D (ZtSn - a etS)), less the repeated-index term
// D (cpop - 2 etA a + cpop a^2) when repeated (At == Zt).
void D_AtTn_ZtSn(State &S, MH *At_, MH *Tt_, MH *Zt_, MH *St_, L_handle *lf_AtTn, L_handle *lf_ZtSn,
                 L_handle *out, bool repeated) {
  M_handle *At = At_->p(), *Tt = Tt_->p(), *St = St_->p();
  (void)Zt_;
  const int P = (int)psize(At->nrows);
  const double *D_An = &S.A_ajdk[AJDK_0_1 * P], *a_An = &S.A_ajdk[AJDK_1_0 * P];
  out->spacing_row = SP_a; out->row_stride = At->nrows;
  out->spacing_col = SP_a; out->col_stride = Tt->nrows;
  lh_zero(out);
  for (int ns_j = 0; ns_j < (int)St->rpop_j; ++ns_j) {
    const unsigned ns_a = St->m_a_[ns_j], ns_b = St->m_b_[ns_j];
    const double etS = -(double)St->cpop_j + 2.0 * popcount_masked_row(St->wX + (long)ns_b * St->mc_length, St->mc_j, (long)St->mc_length);
    const double etT = -(double)Tt->cpop_j + 2.0 * popcount_masked_row(Tt->wX + (long)ns_b * Tt->mc_length, Tt->mc_j, (long)Tt->mc_length);
    for (int na_j = 0; na_j < (int)At->rpop_j; ++na_j) {
      const unsigned na_a = At->m_a_[na_j], na_b = At->m_b_[na_j];
      const double a = a_An[na_a / POPLENGTH], D = D_An[na_a / POPLENGTH];
      double v = (*L2_get(lf_AtTn, na_j, na_b, na_a, ns_j, ns_b, ns_a) - etT * a) * D *
                 (*L2_get(lf_ZtSn, na_j, na_b, na_a, ns_j, ns_b, ns_a) - a * etS);
      if (repeated) {
        const double etA = -(double)At->cpop_j +
                           2.0 * popcount_masked_row(At->wX + (long)na_b * At->mc_length, At->mc_j, (long)At->mc_length);
        v -= D * (At->cpop_j - 2 * etA * a + At->cpop_j * a * a);
      }
      out->lf[na_a + (size_t)ns_a * out->row_stride] = v;
    }
  }
}

void dcc_D_AtTn_ZtSn_all(State &S) {  // dcc_lf_D_AtTn_ZtSn_vv (dir_c/dcc_lf.c:102-163), no Y blocks
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      if (E1->A_rbother && S.A_cbother && E2->Z_rbother)
        D_AtTn_ZtSn(S, E1->M_At, E1->M_Tt, E2->M_Zt, E2->M_St, E1->lf_AtTn, E2->lf_ZtSn, F->lf_D_AtTn_ZtSn_vv, false);
      if (E1->A_rbother && S.A_cbother && E2->A_rbother)
        D_AtTn_ZtSn(S, E1->M_At, E1->M_Tt, E2->M_At, E2->M_Tt, E1->lf_AtTn, E2->lf_AtTn, F->lf_D_AtTn_AtTn_vv,
                    nb1 == nb2);
    }
}

// get_dcc_TAnZtS_ww_stage_0 (dir_c/TAnZtS.c:5-209): per bin, the masked
// column weight sums, the covariate-weighted a1d1 row sums and et_Tn / et_Sn.
void dcc_stage_0(State &S) {
  for (auto &Ep : S.E) {
    Single *E = Ep.get();
    M_handle *An = E->M_An->p(), *At = E->M_At->p(), *Tt = E->M_Tt->p(), *St = E->M_St->p(), *Zt = E->M_Zt->p();
    const int T = Tt->nrows;
    set_l1(E->lf_A_a0d1, 1); set_l1(E->lf_A_a2d1, 1);
    set_l1(E->lf_a1d1_ZtSn, T); set_l1(E->lf_a1d1_AtTn, T);
    set_l1(E->lf_et_Tn, T); set_l1(E->lf_et_Sn, T);
    E->lf_A_a0d1->lf[0] = mask_sum(S, An, AJDK_0_1);
    E->lf_A_a2d1->lf[0] = mask_sum(S, An, AJDK_2_1);
    const int QR_TAnZtS = E->A_rbother && S.A_cbother && E->Z_rbother;
    const int QR_TAnAtT = E->A_rbother && S.A_cbother;
    if (QR_TAnZtS || QR_TAnAtT) {
      for (int ns_j = 0; ns_j < (int)Tt->rpop_j; ++ns_j) {
        const unsigned ns_a = St->m_a_[ns_j], ns_b = St->m_b_[ns_j];
        const unsigned char *Tt_tag = Tt->wX + (long)ns_b * Tt->mc_length;
        if (QR_TAnAtT)
          for (int ma_j = 0; ma_j < (int)At->cpop_j; ++ma_j) {
            const unsigned ma_a = An->m_a_[ma_j], ma_b = An->m_b_[ma_j];
            *L1_get(E->lf_a1d1_AtTn, ns_j, ns_b, ns_a) += bget_pm(Tt_tag, ma_a) * (*L2_get(E->lf_An_ajdk, ma_j, ma_b, ma_a, 0, 0, AJDK_1_1));
          }
        const unsigned char *St_tag = St->wX + (long)ns_b * St->mc_length;
        if (QR_TAnZtS)
          for (int mz_j = 0; mz_j < (int)Zt->cpop_j; ++mz_j) {
            const unsigned mz_a = Zt->n_a_[mz_j], mz_b = Zt->n_b_[mz_j];
            *L1_get(E->lf_a1d1_ZtSn, ns_j, ns_b, ns_a) += bget_pm(St_tag, mz_a) * (*L2_get(E->lf_Zn_ajdk, mz_j, mz_b, mz_a, 0, 0, AJDK_1_1));
          }
      }
      for (int ns_j = 0; ns_j < (int)Tt->rpop_j; ++ns_j) {
        const unsigned ns_a = St->m_a_[ns_j], ns_b = St->m_b_[ns_j];
        if (QR_TAnAtT)
          *L1_get(E->lf_et_Tn, ns_j, ns_b, ns_a) = (double)(-(long long)Tt->cpop_j + 2 * (long long)popcount_masked_row(Tt->wX + (long)ns_b * Tt->mc_length, Tt->mc_j, (long)Tt->mc_length));
        if (QR_TAnZtS)
          *L1_get(E->lf_et_Sn, ns_j, ns_b, ns_a) = (double)(-(long long)St->cpop_j + 2 * (long long)popcount_masked_row(St->wX + (long)ns_b * St->mc_length, St->mc_j, (long)St->mc_length));
      }
    }
  }
}

// An_a0d1_ZtSn_excerpt (dir_c/An_ZtSn_ww.c:243-265): lf_ZtSn scaled by the
// column weights D (AJDK_0_1), spacing b x b.
void a0d1_excerpt(State &S, M_handle *Zt, M_handle *St, L_handle *lf_ZtSn, L_handle *out) {
  out->spacing_row = SP_b; out->spacing_col = SP_b;
  out->row_stride = Zt->rpop_b; out->col_stride = St->rpop_b;
  lh_zero(out);
  const int P = (int)psize(Zt->nrows);
  for (int nz_j = 0; nz_j < (int)Zt->rpop_j; ++nz_j) {
    const unsigned nz_a = Zt->m_a_[nz_j], nz_b = Zt->m_b_[nz_j];
    for (int ns_j = 0; ns_j < (int)St->rpop_j; ++ns_j) {
      const unsigned ns_a = St->m_a_[ns_j], ns_b = St->m_b_[ns_j];
      *L2_get(out, nz_j, nz_b, nz_a, ns_j, ns_b, ns_a) =
          S.A_ajdk[nz_a / POPLENGTH + AJDK_0_1 * P] * (*L2_get(lf_ZtSn, nz_j, nz_b, nz_a, ns_j, ns_b, ns_a));
    }
  }
}

void dcc_stage_1(State &S) {  // dcc_TAnZtS_ww_stage_1 (dir_c/TAnZtS.c:254-326)
  for (auto &E : S.E) {
    if (E->Z_rbother && S.A_cbother) a0d1_excerpt(S, E->M_Zt->p(), E->M_St->p(), E->lf_ZtSn, E->lf_a0d1_ZtSn);
    if (E->A_rbother && S.A_cbother) a0d1_excerpt(S, E->M_At->p(), E->M_Tt->p(), E->lf_AtTn, E->lf_a0d1_AtTn);
  }
  int b_mlt = S.P.B_MLT;
  for (auto &E : S.E) {
    if (E->Z_rbother && S.A_cbother) {
      M_handle *out = E->M_a0d1_ZtSn->p();
      wrap_xcalc(TARGS, E->M_Zt->h.mr_j, E->M_Zt->h.mr_b, E->M_St->h.mr_j, E->M_St->h.mr_b, E->lf_a0d1_ZtSn,
                 E->lf_a0d1_ZtSn->lf, &E->M_Zt->h.nrows, &E->M_St->h.nrows, &out, &b_mlt, 0);
    }
    if (E->A_rbother && S.A_cbother) {
      M_handle *out = E->M_a0d1_AtTn->p();
      wrap_xcalc(TARGS, E->M_At->h.mr_j, E->M_At->h.mr_b, E->M_Tt->h.mr_j, E->M_Tt->h.mr_b, E->lf_a0d1_AtTn,
                 E->lf_a0d1_AtTn->lf, &E->M_At->h.nrows, &E->M_Tt->h.nrows, &out, &b_mlt, 0);
    }
  }
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      for (L_handle *L : {F->lf_An_a0d1_ZtSn, F->lf_An_a0d1_AtTn}) {
        L->row_stride = E1->A_nrows; L->spacing_row = SP_a; L->col_stride = S.T_ncols; L->spacing_col = SP_a; lh_zero(L);
      }
      if (E1->A_rbother && S.A_cbother && E2->Z_rbother)
        wrap_An_ZtSn_ww__run(TARGS, SP_a, SP_a, E1->M_An->p(), E2->lf_a0d1_ZtSn, E2->M_a0d1_ZtSn->p(), E2->M_St->p(), &F->lf_An_a0d1_ZtSn);
      if (E1->A_rbother && S.A_cbother && E2->A_rbother)
        wrap_An_ZtSn_ww__run(TARGS, SP_a, SP_a, E1->M_An->p(), E2->lf_a0d1_AtTn, E2->M_a0d1_AtTn->p(), E2->M_Tt->p(), &F->lf_An_a0d1_AtTn);
    }
}

void dcc_stage_2(State &S) {  // get_dcc_TAnZtS_ww_stage_2 (dir_c/TAnZtS.c:380-495), no Y blocks
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      for (L_handle *L : {F->lf_TAnZtS_ww, F->lf_TAnAtT_ww}) {
        L->row_stride = E1->A_nrows; L->spacing_row = SP_a; L->col_stride = S.T_ncols; L->spacing_col = SP_a; lh_zero(L);
      }
      M_handle *An = E1->M_An->p(), *Tt = E1->M_Tt->p();
      const int QR_TAnZtS = E1->A_rbother && S.A_cbother && E2->Z_rbother;
      const int QR_TAnAtT = E1->A_rbother && S.A_cbother && E2->A_rbother;
      const double A_a2d1 = E1->lf_A_a2d1->lf[0], A_a0d1 = E1->lf_A_a0d1->lf[0];
      if (QR_TAnZtS || QR_TAnAtT)
        for (int ns_j = 0; ns_j < (int)Tt->rpop_j; ++ns_j) {
          const unsigned ns_a = Tt->m_a_[ns_j], ns_b = Tt->m_b_[ns_j];
          if (QR_TAnZtS)
            for (int ma_j = 0; ma_j < (int)An->rpop_j; ++ma_j) {
              const unsigned ma_a = An->m_a_[ma_j], ma_b = An->m_b_[ma_j];
              const double et = *L1_get(E2->lf_et_Sn, ns_j, ns_b, ns_a);
              const double v = (*L2_get(F->lf_An_a0d1_ZtSn, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a)) -
                               (*L1_get(E2->lf_a1d1_ZtSn, ns_j, ns_b, ns_a)) -
                               (*L2_get(E1->lf_An_ajdk, ma_j, ma_b, ma_a, 0, 0, AJDK_1_1)) * et + A_a2d1 * et;
              *L2_get(F->lf_TAnZtS_ww, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a) += +v;
            }
          if (QR_TAnAtT)
            for (int ma_j = 0; ma_j < (int)An->rpop_j; ++ma_j) {
              const unsigned ma_a = An->m_a_[ma_j], ma_b = An->m_b_[ma_j];
              const double et = *L1_get(E2->lf_et_Tn, ns_j, ns_b, ns_a);
              const double v = (*L2_get(F->lf_An_a0d1_AtTn, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a)) -
                               (*L1_get(E2->lf_a1d1_AtTn, ns_j, ns_b, ns_a)) -
                               (*L2_get(E1->lf_An_ajdk, ma_j, ma_b, ma_a, 0, 0, AJDK_1_1)) * et + A_a2d1 * et;
              *L2_get(F->lf_TAnAtT_ww, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a) += +v;
            }
        }
      if (QR_TAnAtT && nb1 == nb2)
        for (int ns_j = 0; ns_j < (int)Tt->rpop_j; ++ns_j) {
          const unsigned ns_a = Tt->m_a_[ns_j], ns_b = Tt->m_b_[ns_j];
          const unsigned char *Tt_tag = Tt->wX + (long)ns_b * Tt->mc_length;
          for (int ma_j = 0; ma_j < (int)An->rpop_j; ++ma_j) {
            const unsigned ma_a = An->m_a_[ma_j], ma_b = An->m_b_[ma_j];
            const double v = bget_pm(Tt_tag, ma_a) *
                             (A_a0d1 - 2 * (*L2_get(E1->lf_An_ajdk, ma_j, ma_b, ma_a, 0, 0, AJDK_1_1)) + A_a2d1);
            *L2_get(F->lf_TAnAtT_ww, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a) += -v;
          }
        }
    }
}

// get_dcc_halfloop (dir_c/dcc_lf.c:379-488): the row and column loop scores,
// covariates turned from spacing a to spacing b.
void dcc_halfloop(State &S) {
  for (int nb1 = 0; nb1 < S.nbins; ++nb1)
    for (int nb2 = 0; nb2 < S.nbins; ++nb2) {
      Double *F = S.f(nb1, nb2);
      Single *E1 = S.E[nb1].get(), *E2 = S.E[nb2].get();
      M_handle *An = E1->M_An->p(), *At = E1->M_At->p(), *Tt2 = E2->M_Tt->p();
      for (L_handle *L : {F->QR_AnZtSZnAt, F->QR_AnAtTAnAt}) {
        L->row_stride = At->ncols; L->spacing_row = SP_a; L->col_stride = S.T_ncols; L->spacing_col = SP_b; lh_zero(L);
      }
      for (L_handle *L : {F->QC_AtTAnZtSZn, F->QC_AtTAnAtTAn}) {
        L->row_stride = At->nrows; L->spacing_row = SP_a; L->col_stride = S.T_ncols; L->spacing_col = SP_b; lh_zero(L);
      }
      const int ZS = E1->A_rbother && S.A_cbother && E2->Z_rbother;
      const int AT = E1->A_rbother && S.A_cbother && E2->A_rbother;
      if (ZS || AT)
        for (int ns_j = 0; ns_j < (int)Tt2->rpop_j; ++ns_j) {
          const unsigned ns_a = Tt2->m_a_[ns_j], ns_b = Tt2->m_b_[ns_j];
          for (int ma_j = 0; ma_j < (int)An->rpop_j; ++ma_j) {
            const unsigned ma_a = An->m_a_[ma_j], ma_b = An->m_b_[ma_j];
            if (ZS) *L2_get(F->QR_AnZtSZnAt, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a) = *L2_get(F->lf_TAnZtS_ww, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a);
            if (AT) *L2_get(F->QR_AnAtTAnAt, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a) = *L2_get(F->lf_TAnAtT_ww, ma_j, ma_b, ma_a, ns_j, ns_b, ns_a);
          }
          for (int na_j = 0; na_j < (int)At->rpop_j; ++na_j) {
            const unsigned na_a = At->m_a_[na_j], na_b = At->m_b_[na_j];
            if (ZS) *L2_get(F->QC_AtTAnZtSZn, na_j, na_b, na_a, ns_j, ns_b, ns_a) = *L2_get(F->lf_D_AtTn_ZtSn_vv, na_j, na_b, na_a, ns_j, ns_b, ns_a);
            if (AT) *L2_get(F->QC_AtTAnAtTAn, na_j, na_b, na_a, ns_j, ns_b, ns_a) = *L2_get(F->lf_D_AtTn_AtTn_vv, na_j, na_b, na_a, ns_j, ns_b, ns_a);
          }
        }
    }
}

// dexcluster_driver.c:22-28 / :43-47: every step's sub-scores.
void dcc_subscores(State &S) {
  An_ajdk_all(S); trace_stage(S, "An_ajdk");
  lf_ZtSn_all(S); trace_stage(S, "lf_ZtSn");
  dcc_D_AtTn_ZtSn_all(S); trace_stage(S, "D_AtTn_ZtSn");
  dcc_stage_0(S); dcc_stage_1(S); dcc_stage_2(S); trace_stage(S, "TAnZtS");
  dcc_halfloop(S); trace_stage(S, "halfloop");
}

}  // namespace

namespace {
thread_local StopCheck t_stop = nullptr;
thread_local void *t_stop_ctx = nullptr;

int stop_requested(std::string &err) {
  if (!t_stop) return 0;
  const char *why = nullptr;
  const int rc = t_stop(t_stop_ctx, &why);
  if (rc) err = why ? why : "solve stopped";
  return rc;
}
}  // namespace

void set_stop_check(StopCheck fn, void *ctx) {
  t_stop = fn;
  t_stop_ctx = ctx;
}

int solve(const Params &P, const Input &I, Output &O, std::string &err, const Hooks *hooks) {
  if (!strategies_supported(P)) {
    err = kStrategyError;
    return 4;
  }
  if (P.B_MLT < 1 || P.B_MLT > 62) { err = "B_MLT out of range"; return 4; }
  State S;
  S.P = P;
  S.hooks = hooks;
  S.out = &O;
  const char *prof = getenv("LAKBCC_PROFILE");
  // LAKBCC_PROGRESS=N: a line on stderr every N iterations (long solves)
  const char *prog = getenv("LAKBCC_PROGRESS");
  const int progress = prog ? atoi(prog) : 0;
  const auto t_start = std::chrono::steady_clock::now();
  g_clock = StageClock();
  g_clock.on = prof && *prof && *prof != '0';
  g_clock.last = std::chrono::steady_clock::now();
  O = Output();
  int rc = load(S, I, err);
  if (rc) return rc;
  if ((rc = stop_requested(err))) return rc;
  M_mxset_all(S);
  if (!I.scramble.empty()) {  // wrap_bcc_scramble (R_init.c:264-290), lakcluster_driver.c:58-62
    scramble_snapshot(S, "pre");
    for (const auto &sc : I.scramble)
      if ((rc = scramble(S, sc, err))) return rc;
    scramble_snapshot(S, "pos");
  }
  trace_stage(S, "load");
  initial_subscores(S);
  while (S.A_rpop_j_total > 0 || S.A_cpop_j > 0) {
    if ((rc = stop_requested(err))) return rc;
    sumscores_nrm(S);
    sumscores_ifT(S);
    if (S.P.Ireq > 0) sumscores_srt(S);
    sumscores_cmb(S);
    g_clock.tick("sumscores (nrm, ifT, srt, cmb)");  // LAKBCC_PROFILE only
    sumscores_xij(S);
    g_clock.tick("sumscores (xij)");
    sumscores_mxA(S);
    trace_stage(S, "sumscores");
    lrup_QR(S); trace_stage(S, "lrup_QR");
    lrup_QC_ZtSWn(S); trace_stage(S, "lrup_QC_ZtSWn");
    if (qc_ynwt(S)) { lrup_QC(S); trace_stage(S, "lrup_QC"); }
    lrup_mxdup(S);
    M_mxset_all(S);
    g_clock.tick("lrup_mxdup, M_mxset");
    // bcc_M_YnWt here requantises the updated Grams, but nothing on the
    // YnWt path reads those planes before they are rebuilt, so it is skipped.
    lf_AtTYn____WtSZn_all(S); trace_stage(S, "lf_AtTYn____WtSZn");
    if (qc_ynwt(S)) { lrup_QC_stage_c(S); trace_stage(S, "lrup_QC_stage_c"); }
    lf_AnZt_S_WnYt_all(S); trace_stage(S, "lf_AnZt_S_WnYt");
    An_ajdk_all(S); trace_stage(S, "An_ajdk");
    lf_ZtSn_all(S); trace_stage(S, "lf_ZtSn");
    singlestudy_ww(S); trace_stage(S, "singlestudy");
    doublestudy_ww(S); trace_stage(S, "doublestudy");
    flattenloop(S); trace_stage(S, "flattenloop");
    if (O.iterations > 10000000) { err = "iteration limit"; return 5; }
    if (progress > 0 && O.iterations % progress == 0)
      fprintf(stderr, " %% iteration %d: %u rows and %u columns left, %.1f s\n", O.iterations,
              (unsigned)S.A_rpop_j_total, (unsigned)S.A_cpop_j,
              std::chrono::duration<double>(std::chrono::steady_clock::now() - t_start).count());
  }
  if (g_clock.on) {
    double tot = 0;
    for (auto &kv : g_clock.acc) tot += kv.second;
    fprintf(stderr, " %% stage profile (%d iterations, %.3f s):\n", O.iterations, tot);
    for (auto &kv : g_clock.acc) fprintf(stderr, " %%   %-20s %9.3f s\n", kv.first.c_str(), kv.second);
  }
  return 0;
}

// lakcluster_scorebox (lakcluster_scorebox.c:103-271): rows and columns are
// removed in the order of a previous run's out_xdrop, and the mean row and
// column scores are recorded on a row_num x col_num grid of retained counts
// (row_max ... 0 rows and col_max ... 0 columns past the initial removal).
// The first grid point is computed directly, every other one by one
// low-rank update from its neighbour: the longer dimension is stepped in the
// inner loop from a copy of the state reached by the outer one.  The copy
// (bcc_copy, bcc.c:1440-1480) is made here by replaying the outer steps on
// a second state loaded from the same inputs, which reaches the same values
// bit for bit.
int scorebox(const Params &P, const Input &I, ScoreboxOutput &SO, std::string &err, const Hooks *hooks) {
  if (!dcc_mode(P) && !strategies_supported(P)) {
    err = kStrategyError;
    return 4;
  }
  const int row_num = std::max(0, P.scorebox_row_num), col_num = std::max(0, P.scorebox_col_num);
  SO = ScoreboxOutput();
  SO.row_max = P.scorebox_row_max; SO.row_num = row_num;
  SO.col_max = P.scorebox_col_max; SO.col_num = col_num;
  const size_t cells = (size_t)row_num * col_num;
  SO.A_rpop_j_total.assign(cells, 0); SO.A_cpop_j.assign(cells, 0); SO.Irem.assign(cells, 0);
  SO.QR_avg.assign(cells, 0.0); SO.QC_avg.assign(cells, 0.0);
  g_clock = StageClock();
  Output O_ori, O_sub;
  auto prepare = [&](State &S, Output &O) -> int {
    S.P = P; S.hooks = hooks; S.out = &O;
    const int rc = load(S, I, err);
    if (rc) return rc;
    M_mxset_all(S);
    return 0;
  };
  std::unique_ptr<State> D(new State);
  int rc = prepare(*D, O_ori);
  if (rc) return rc;
  ScoreboxLists L;
  xdrop_lists(I.scorebox_xdrop, L.rows, L.cols);
  if ((rc = xdrop_lookup(*D, L.rows, L.lnb, L.lmr, err))) return rc;
  std::vector<int> ckeep, cdrop, rkeep, rdrop;
  scorebox_xdrop_array((int)D->A_cpop_j, P.scorebox_col_max, col_num, ckeep, cdrop);
  scorebox_xdrop_array((int)D->A_rpop_j_total, P.scorebox_row_max, row_num, rkeep, rdrop);
  auto record = [&](State &S, int nr, int nc) {  // lakcluster_scorebox_excerpt_0 (:5-20)
    const size_t t = (size_t)nr + (size_t)nc * row_num;
    SO.A_rpop_j_total[t] = (int)S.A_rpop_j_total;
    SO.A_cpop_j[t] = (int)S.A_cpop_j;
    SO.Irem[t] = S.Irem;
    double m = ra_mean(S.QR_svalue.data(), S.A_rpop_j_total);
    SO.QR_avg[t] = std::isfinite(m) ? m : 1.0;
    m = ra_mean(S.QC_svalue.data(), S.A_cpop_j);
    SO.QC_avg[t] = std::isfinite(m) ? m : 1.0;
  };
  // rows outer when row_max > col_max is false (lakcluster_scorebox:
  // _rc steps columns outside, rows inside; _cr the reverse)
  const bool rows_inner = P.scorebox_row_max > P.scorebox_col_max;
  const int outer_num = rows_inner ? col_num : row_num, inner_num = rows_inner ? row_num : col_num;
  auto outer_step = [&](State &S, int k) {
    scorebox_srt(S, L);
    if (k == 0) {
      scorebox_mxA(S, rdrop.empty() ? 0 : rdrop[0], cdrop.empty() ? 0 : cdrop[0]);
      lrup_mxdup(S);
      M_mxset_all(S);
      scorebox_full(S);
    } else {
      scorebox_mxA(S, rows_inner ? 0 : rdrop[k], rows_inner ? cdrop[k] : 0);
      scorebox_update(S);
    }
  };
  if (row_num > 0 && col_num > 0) {
    for (int k = 0; k < outer_num; ++k) {
      if ((rc = stop_requested(err))) return rc;
      outer_step(*D, k);
      record(*D, rows_inner ? 0 : k, rows_inner ? k : 0);
      if (inner_num <= 1) continue;
      std::unique_ptr<State> Sub(new State);
      if ((rc = prepare(*Sub, O_sub))) return rc;
      for (int r = 0; r <= k; ++r) outer_step(*Sub, r);
      for (int j = 1; j < inner_num; ++j) {
        if ((rc = stop_requested(err))) return rc;
        scorebox_srt(*Sub, L);
        scorebox_mxA(*Sub, rows_inner ? rdrop[j] : 0, rows_inner ? 0 : cdrop[j]);
        scorebox_update(*Sub);
        record(*Sub, rows_inner ? j : k, rows_inner ? k : j);
      }
    }
  }
  return 0;
}

// dexcluster_driver (dir_c/dexcluster_driver.c:5-57): the dcc method on the
// same inputs and outputs as the bcc solve.
int dcc_solve(const Params &P, const Input &I, Output &O, std::string &err, const Hooks *hooks) {
  if (P.B_MLT < 1 || P.B_MLT > 62) { err = "B_MLT out of range"; return 4; }
  State S;
  S.P = P;
  S.hooks = hooks;
  S.out = &O;
  g_clock = StageClock();
  O = Output();
  int rc = load(S, I, err);
  if (rc) return rc;
  if ((rc = stop_requested(err))) return rc;
  M_mxset_all(S);
  // wrap_dcc_scramble (dir_c/R_init.c:134-160): bcc_scramble on the dcc
  // state; its .b16 snapshots are written only when its (fixed-off) verbose
  // flag is set, so none are written here
  for (const auto &sc : I.scramble)
    if ((rc = scramble(S, sc, err))) return rc;
  trace_stage(S, "load");
  dcc_subscores(S);
  while (S.A_rpop_j_total > 0 || S.A_cpop_j > 0) {
    if ((rc = stop_requested(err))) return rc;
    sumscores_nrm(S);
    sumscores_ifT(S);
    if (S.P.Ireq > 0) sumscores_srt(S);
    sumscores_cmb(S);
    g_clock.tick("sumscores (nrm, ifT, srt, cmb)");  // LAKBCC_PROFILE only
    sumscores_xij(S);
    g_clock.tick("sumscores (xij)");
    sumscores_mxA(S);
    trace_stage(S, "sumscores");
    lrup_mxdup(S);
    M_mxset_all(S);
    g_clock.tick("lrup_mxdup, M_mxset");
    dcc_subscores(S);
    if (O.iterations > 10000000) { err = "iteration limit"; return 5; }
  }
  return 0;
}

namespace {
int write_mda_i4(const std::string &path, int nrows, int ncols, const std::vector<int> &v) {
  FILE *fp = fopen(path.c_str(), "wb");
  if (!fp) return 1;
  const int hdr[3] = {2, nrows, ncols};
  fwrite(hdr, sizeof(int), 3, fp);
  if (!v.empty()) fwrite(v.data(), sizeof(int), v.size(), fp);
  return fclose(fp) != 0;
}
int write_mda_r8(const std::string &path, int nrows, int ncols, const std::vector<double> &v) {
  FILE *fp = fopen(path.c_str(), "wb");
  if (!fp) return 1;
  const int hdr[3] = {2, nrows, ncols};
  fwrite(hdr, sizeof(int), 3, fp);
  if (!v.empty()) fwrite(v.data(), sizeof(double), v.size(), fp);
  return fclose(fp) != 0;
}
}  // namespace

// S_handle_dmp (dir_c/S_init.c:79-89): five row_num x col_num arrays in the
// mda format of mda_write_d2_i4 / mda_write_d2_r8 (dir_c/mda_io.c:5-31).
int write_scorebox(const std::string &dir, const ScoreboxOutput &SO) {
  char prefix[160];
  snprintf(prefix, sizeof prefix, "%s/scorebox_r%dn%d_c%dn%d", dir.c_str(), SO.row_max, SO.row_num, SO.col_max,
           SO.col_num);
  const std::string p = prefix;
  int rc = write_mda_i4(p + "_A_rpop_j_total.mda", SO.row_num, SO.col_num, SO.A_rpop_j_total);
  rc |= write_mda_i4(p + "_A_cpop_j.mda", SO.row_num, SO.col_num, SO.A_cpop_j);
  rc |= write_mda_i4(p + "_Irem.mda", SO.row_num, SO.col_num, SO.Irem);
  rc |= write_mda_r8(p + "_QR_avg.mda", SO.row_num, SO.col_num, SO.QR_avg);
  rc |= write_mda_r8(p + "_QC_avg.mda", SO.row_num, SO.col_num, SO.QC_avg);
  return rc;
}

int write_outputs(const std::string &dir, const Output &O) {
  std::string p = dir + "/out_trace.txt";
  FILE *fp = fopen(p.c_str(), "w");
  if (!fp) return 2;
  for (int nl = 0; nl < O.iterations; ++nl) {
    const double *t = &O.trace[(size_t)nl * 6];
    fprintf(fp, "%d %d %d %0.16f %0.16f %d\n", (int)t[0], (int)t[1], (int)t[2], t[3], t[4], (int)t[5]);
  }
  fclose(fp);
  FILE *fa = fopen((dir + "/out_xdrop_a.txt").c_str(), "w");
  FILE *fb = fopen((dir + "/out_xdrop_b.txt").c_str(), "w");
  if (!fa || !fb) { if (fa) fclose(fa); if (fb) fclose(fb); return 2; }
  for (size_t i = 0; i + 1 < O.xdrop_a.size(); i += 2) {
    fprintf(fa, "%d %d\n", O.xdrop_a[i], O.xdrop_a[i + 1]);
    fprintf(fb, "%d %d\n", O.xdrop_b[i], O.xdrop_b[i + 1]);
  }
  fclose(fa);
  fclose(fb);
  for (const auto &f : O.files) {
    FILE *fo = fopen((dir + "/" + f.first).c_str(), "wb");
    if (!fo) return 2;
    const size_t n = f.second.size();
    const bool ok = (n == 0 || fwrite(f.second.data(), 1, n, fo) == n);
    if (fclose(fo) != 0 || !ok) return 2;
  }
  return 0;
}

}  // namespace lakbcc
