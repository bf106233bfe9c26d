/* lak_oracle.c -- TEST INFRASTRUCTURE ONLY: plain-C restatement of the
 * reference's bcc kernels (see lak_oracle.h).  Portable C11 + OpenMP, no SIMD
 * intrinsics; popcounts use __builtin_popcountll on 64-bit words of each
 * 1920-bit block, which gives the same exact integer counts as the reference's
 * SSE2 Lauradoux/Walisch routine (dir_c/popcount.c:31-621).  FP64 expressions
 * are written in the reference's evaluation order and compiled with FP
 * contraction off, so results are bit-identical on x86-64 and aarch64. */
#include "lak_oracle.h"

#include <math.h>
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define BLK_BYTES 240
#define BLK_WORDS 30 /* 64-bit words per 1920-bit block */
#define AJDK_0_1 5
#define AJDK_1_1 6
#define AJDK_2_1 7

static int g_threads = 0;
void lako_set_threads(int n) { g_threads = n; }
static int nthreads(void) { return g_threads > 0 ? g_threads : omp_get_max_threads(); }

static unsigned long long spacing_len(int spacing, const struct M_handle *M)
{
  switch (spacing) {
    case LAKGB_SPACING_j: return (unsigned long long)M->rpop_j;
    case LAKGB_SPACING_b: return (unsigned long long)M->rpop_b;
    case LAKGB_SPACING_a: return (unsigned long long)M->nrows;
    default: return 0;
  }
}

static unsigned long long tab(int spacing, const struct M_handle *M, long long j)
{
  switch (spacing) {
    case LAKGB_SPACING_j: return (unsigned long long)j;
    case LAKGB_SPACING_b: return M->m_b_[j];
    case LAKGB_SPACING_a: return M->m_a_[j];
    default: return 0;
  }
}

static struct L_handle *ensure(struct L_handle **pp, unsigned long long length)
{
  if (*pp == NULL) {
    struct L_handle *L = (struct L_handle *)calloc(1, sizeof(struct L_handle));
    L->length = length;
    L->lf = (double *)calloc(length ? length : 1, sizeof(double));
    *pp = L;
  }
  if ((*pp)->length < length) return NULL;
  memset((*pp)->lf, 0, length * sizeof(double));
  return *pp;
}

static int popc_bytes(const unsigned char *p, int n)
{
  int c = 0;
  for (int i = 0; i < n; i++) c += __builtin_popcount((unsigned)p[i]);
  return c;
}

static inline uint64_t ld64(const unsigned char *p)
{
  uint64_t x;
  memcpy(&x, p, 8);
  return x;
}

/* masked popcount of one 1920-bit block: op 0 = x, 1 = x^y, 2 = x&y */
static inline int blk_count(const unsigned char *x, const unsigned char *y, const unsigned char *m, int op)
{
  int c = 0;
  for (int w = 0; w < BLK_WORDS; w++) {
    uint64_t a = ld64(x + 8 * w), mm = ld64(m + 8 * w);
    uint64_t v = (op == 0) ? a : (op == 1 ? (a ^ ld64(y + 8 * w)) : (a & ld64(y + 8 * w)));
    c += __builtin_popcountll(v & mm);
  }
  return c;
}

static int gram(int symmetric, int type_flag, int spacing_r, int spacing_c, struct M_handle *M_An,
                struct M_handle *M_Zn, double *A_ajdk, struct L_handle *lfA, struct L_handle *lfZ,
                struct L_handle **out_p)
{
  unsigned long long len_r = spacing_len(spacing_r, M_An), len_c = spacing_len(spacing_c, M_Zn);
  unsigned long long length = len_r * len_c;
  struct L_handle *out = ensure(out_p, length);
  if (!out) return (int)length;
  out->spacing_row = spacing_r; out->row_stride = len_r;
  out->spacing_col = spacing_c; out->col_stride = len_c;
  if (type_flag == LAKGB_TYPE_p0) return (int)length;
  const int P = (int)(M_An->mc_length / BLK_BYTES);
  double a0d1 = 0, a2d1 = 0;
  for (int nc = 0; nc < P; nc++) {
    double c = (double)popc_bytes(M_An->mc_j + (long)nc * BLK_BYTES, BLK_BYTES);
    a0d1 += (A_ajdk ? A_ajdk[nc + AJDK_0_1 * P] : 1) * c;
    a2d1 += (A_ajdk ? A_ajdk[nc + AJDK_2_1 * P] : 0) * c;
  }
  const long long nA = M_An->rpop_j, nZ = M_Zn->rpop_j;
  const int op = (type_flag == LAKGB_TYPE_pm) ? 1 : 2;
  const double *D = A_ajdk ? A_ajdk + AJDK_0_1 * P : NULL;
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads())
  for (long long ma = 0; ma < nA; ma++) {
    const unsigned char *wa = M_An->wX + (long long)M_An->m_b_[ma] * M_An->mc_length;
    for (long long mz = symmetric ? ma : 0; mz < nZ; mz++) {
      const unsigned char *wz = M_Zn->wX + (long long)M_Zn->m_b_[mz] * M_Zn->mc_length;
      double o = (op == 1) ? a0d1 : 0.0;
      double dtmp = 0;
      if (D) {
        for (int b = 0; b < P; b++)
          dtmp += D[b] * (double)blk_count(wa + b * BLK_BYTES, wz + b * BLK_BYTES, M_An->mc_j + b * BLK_BYTES, op);
      } else {
        long long t = 0;
        for (int b = 0; b < P; b++)
          t += blk_count(wa + b * BLK_BYTES, wz + b * BLK_BYTES, M_An->mc_j + b * BLK_BYTES, op);
        dtmp = (double)t;
      }
      if (op == 1) o -= 2 * dtmp; else o += dtmp;
      if (lfA && lfZ)
        o -= lfA->lf[tab(lfA->spacing_row, M_An, ma) + AJDK_1_1 * lfA->row_stride] +
             lfZ->lf[tab(lfZ->spacing_row, M_Zn, mz) + AJDK_1_1 * lfZ->row_stride] - a2d1;
      out->lf[tab(spacing_r, M_An, ma) + tab(spacing_c, M_Zn, mz) * len_r] = o;
      if (symmetric) out->lf[tab(spacing_r, M_Zn, mz) + tab(spacing_c, M_An, ma) * len_r] = o;
    }
  }
  return (int)length;
}

int lako_AnZt_vv(int type_flag, int spacing_r, int spacing_c, struct M_handle *M_An,
                 struct M_handle *M_Zn, double *A_ajdk, struct L_handle *lf_An_ajdk,
                 struct L_handle *lf_Zn_ajdk, struct L_handle **out_p)
{
  return gram(0, type_flag, spacing_r, spacing_c, M_An, M_Zn, A_ajdk, lf_An_ajdk, lf_Zn_ajdk, out_p);
}

int lako_AnAt_vv(int type_flag, int spacing_r, int spacing_c, struct M_handle *M_An,
                 struct M_handle *M_Zn, double *A_ajdk, struct L_handle *lf_An_ajdk,
                 struct L_handle *lf_Zn_ajdk, struct L_handle **out_p)
{
  return gram(1, type_flag, spacing_r, spacing_c, M_An, M_Zn, A_ajdk, lf_An_ajdk, lf_Zn_ajdk, out_p);
}

int lako_An_v(int type_flag, int spacing_r, struct M_handle *M_An, struct L_handle **out_p)
{
  unsigned long long length = spacing_len(spacing_r, M_An);
  struct L_handle *out = ensure(out_p, length);
  if (!out) return (int)length;
  out->spacing_row = spacing_r; out->row_stride = length;
  if (type_flag == LAKGB_TYPE_p0) return (int)length;
  const int P = (int)(M_An->mc_length / BLK_BYTES);
  for (long long ma = 0; ma < M_An->rpop_j; ma++) {
    const unsigned char *wa = M_An->wX + (long long)M_An->m_b_[ma] * M_An->mc_length;
    long long t = 0;
    for (int b = 0; b < P; b++) t += blk_count(wa + b * BLK_BYTES, NULL, M_An->mc_j + b * BLK_BYTES, 0);
    double o = (type_flag == LAKGB_TYPE_pm) ? -(double)M_An->cpop_j : 0.0;
    if (type_flag == LAKGB_TYPE_pm) o += 2 * (double)t; else o += (double)t;
    out->lf[tab(spacing_r, M_An, ma)] = o;
  }
  return (int)length;
}

int lako_An_ajdk_v(int type_flag, int spacing_r, struct M_handle *M_An, double *A_ajdk,
                   struct L_handle **out_p)
{
  unsigned long long len_r = spacing_len(spacing_r, M_An);
  unsigned long long length = len_r * LAKGB_AJDK_TOT;
  struct L_handle *out = ensure(out_p, length);
  if (!out) return (int)length;
  out->spacing_row = spacing_r; out->row_stride = len_r;
  out->spacing_col = LAKGB_SPACING_a; out->col_stride = LAKGB_AJDK_TOT;
  if (type_flag == LAKGB_TYPE_p0) return (int)length;
  const int P = (int)(M_An->mc_length / BLK_BYTES);
  for (int k = 0; k < LAKGB_AJDK_TOT; k++) {
    double base = 0;
    for (int nc = 0; nc < P; nc++)
      base += A_ajdk[nc + k * P] * (double)popc_bytes(M_An->mc_j + (long)nc * BLK_BYTES, BLK_BYTES);
    for (long long ma = 0; ma < M_An->rpop_j; ma++) {
      const unsigned char *wa = M_An->wX + (long long)M_An->m_b_[ma] * M_An->mc_length;
      double s = 0;
      for (int b = 0; b < P; b++)
        s += A_ajdk[b + k * P] * (double)blk_count(wa + b * BLK_BYTES, NULL, M_An->mc_j + b * BLK_BYTES, 0);
      unsigned long long o = tab(spacing_r, M_An, ma) + (unsigned long long)k * len_r;
      if (type_flag == LAKGB_TYPE_pm) { out->lf[o] = -base; out->lf[o] += 2 * s; }
      else { out->lf[o] = 0; out->lf[o] += s; }
    }
  }
  return (int)length;
}

void lako_calc_A_ajdk(const double *A_p, int A_pcols, double *A_ajdk)
{
  for (int k = 0; k < 3; k++)
    for (int j = 0; j < 5; j++)
      for (int nc = 0; nc < A_pcols; nc++)
        A_ajdk[nc + (j + 5 * k) * A_pcols] =
            pow(A_p[nc] - (1 - A_p[nc]), j) *
            pow(1.0 / fmax(0.01, (4.0 * A_p[nc] * (1 - A_p[nc]))), k);
}

/* ------------------------------------------------------------------------
 * Loop-product kernels of the YnWt solve path.
 * ------------------------------------------------------------------------ */

static inline int bit_on(const unsigned char *b, long n) { return (b[n / 8] >> (7 - n % 8)) & 1; }
static inline int bit_pm(const unsigned char *b, long n) { return 2 * bit_on(b, n) - 1; }
static inline void bit_set(unsigned char *b, long n) { b[n / 8] |= (unsigned char)(1 << (7 - n % 8)); }
static long bsize_c(long n) { long m = n + (16 - n % 16) % 16; return (m + (1920 - m % 1920) % 1920) / 8; }
static long psize_c(long n) { long m = n + (16 - n % 16) % 16; return (m + (1920 - m % 1920) % 1920) / 1920; }
static unsigned long long pick(int s, unsigned long long j, unsigned long long b, unsigned long long a)
{
  return s == LAKGB_SPACING_j ? j : (s == LAKGB_SPACING_b ? b : a);
}
static double *L2(struct L_handle *L, unsigned long long rj, unsigned long long rb, unsigned long long ra,
                  unsigned long long cj, unsigned long long cb, unsigned long long ca)
{
  return &L->lf[pick(L->spacing_row, rj, rb, ra) + pick(L->spacing_col, cj, cb, ca) * L->row_stride];
}
static double *L3(struct L_handle *L, unsigned long long rj, unsigned long long rb, unsigned long long ra,
                  unsigned long long cj, unsigned long long cb, unsigned long long ca, unsigned long long lj,
                  unsigned long long lb, unsigned long long la)
{
  return &L->lf[pick(L->spacing_row, rj, rb, ra) + pick(L->spacing_col, cj, cb, ca) * L->row_stride +
                pick(L->spacing_lyr, lj, lb, la) * L->row_stride * L->col_stride];
}

/* masked signed popcounts over whole rows (popcount.c:425-540):
 *   pm0(a,y)     = #(a=1,y=1) - #(a=0,y=1)
 *   pmpm0(a,t,y) = #(a==t,y=1) - #(a!=t,y=1)
 *   notxorxor    = #(~(a^t^y)) ; all under mask m, nbytes a multiple of 240 */
static long long row_pm0(const unsigned char *a, const unsigned char *y, const unsigned char *m, long nbytes)
{
  long long c = 0;
  for (long w = 0; w < nbytes / 8; w++) {
    uint64_t ym = ld64(y + 8 * w) & ld64(m + 8 * w), aa = ld64(a + 8 * w);
    c += __builtin_popcountll(aa & ym) - __builtin_popcountll(~aa & ym);
  }
  return c;
}
static long long row_pmpm0(const unsigned char *a, const unsigned char *t, const unsigned char *y,
                           const unsigned char *m, long nbytes)
{
  long long c = 0;
  for (long w = 0; w < nbytes / 8; w++) {
    uint64_t ym = ld64(y + 8 * w) & ld64(m + 8 * w), x = ld64(a + 8 * w) ^ ld64(t + 8 * w);
    c += __builtin_popcountll(~x & ym) - __builtin_popcountll(x & ym);
  }
  return c;
}
static long long row_notxorxor(const unsigned char *a, const unsigned char *t, const unsigned char *y,
                               const unsigned char *m, long nbytes)
{
  long long c = 0;
  for (long w = 0; w < nbytes / 8; w++)
    c += __builtin_popcountll(~(ld64(a + 8 * w) ^ ld64(t + 8 * w) ^ ld64(y + 8 * w)) & ld64(m + 8 * w));
  return c;
}
static long long row_and(const unsigned char *a, const unsigned char *m, long nbytes)
{
  long long c = 0;
  for (long w = 0; w < nbytes / 8; w++) c += __builtin_popcountll(ld64(a + 8 * w) & ld64(m + 8 * w));
  return c;
}

/* M_mxget (M_init.c:268-295) */
static void mxget_part(int n, const unsigned char *mb, const unsigned char *mj, long long *pb, long long *pj,
                       unsigned int *a_, unsigned int *b_, long length)
{
  *pb = popc_bytes(mb, (int)length);
  *pj = popc_bytes(mj, (int)length);
  int a = 0, b = 0, j = 0;
  while (a < n) {
    while (a < n && !bit_on(mb, a)) a++;
    if (a < n && bit_on(mb, a) && bit_on(mj, a)) { b_[j] = b; a_[j] = a; j++; b++; a++; }
    else if (a < n && bit_on(mb, a)) { b++; a++; }
  }
}
static void mxget(struct M_handle *M)
{
  mxget_part(M->nrows, M->mr_b, M->mr_j, &M->rpop_b, &M->rpop_j, M->m_a_, M->m_b_, (long)M->mr_length);
  mxget_part(M->ncols, M->mc_b, M->mc_j, &M->cpop_b, &M->cpop_j, M->n_a_, M->n_b_, (long)M->mc_length);
}

static long long g_d_mlt = 4294967296LL;
void lako_set_d_mlt(long long d) { g_d_mlt = d; }

/* dir_c/xcalc.c:5-246 (xcalc_setmaxmin + get_xcalc), into a pre-allocated M_X */
void lako_xcalc(unsigned char *mr_j, unsigned char *mr_b, unsigned char *mc_j, unsigned char *mc_b,
                struct L_handle *lf, double *YnWt, int Yn_nrows, int Wn_nrows, struct M_handle *M_X,
                int b_mlt, int trm_flag)
{
  const int rpop_j = popc_bytes(mr_j, (int)bsize_c(Yn_nrows)), rpop_b = popc_bytes(mr_b, (int)bsize_c(Yn_nrows));
  const int cpop_j = popc_bytes(mc_j, (int)bsize_c(Wn_nrows));
  double min_d = 0, max_d = 0;
  int set = 0;
#define XGET(nrj, nrb, nra, ncj, ncb, nca) \
  (trm_flag ? YnWt[pick(lf->spacing_row, ncj, ncb, nca) + pick(lf->spacing_col, nrj, nrb, nra) * lf->row_stride] \
            : YnWt[pick(lf->spacing_row, nrj, nrb, nra) + pick(lf->spacing_col, ncj, ncb, nca) * lf->row_stride])
  {
    long nc_j = 0, nc_b = 0;
    for (long nc_a = 0; nc_a < Wn_nrows; nc_a++) {
      if (!bit_on(mc_b, nc_a)) continue;
      if (bit_on(mc_j, nc_a)) {
        long nr_j = 0, nr_b = 0;
        for (long nr_a = 0; nr_a < Yn_nrows; nr_a++) {
          if (!bit_on(mr_b, nr_a)) continue;
          if (bit_on(mr_j, nr_a)) {
            double x = XGET(nr_j, nr_b, nr_a, nc_j, nc_b, nc_a);
            if (!set) { min_d = x; max_d = x; set = 1; }
            else { min_d = x < min_d ? x : min_d; max_d = x > max_d ? x : max_d; }
            nr_j++;
          }
          nr_b++;
        }
        nc_j++;
      }
      nc_b++;
    }
  }
  if (min_d >= max_d) max_d = min_d + 1;
  const double mn = min_d - 0.0625 * (max_d - min_d), mx = max_d + 0.0625 * (max_d - min_d);
  const double mlt = (double)g_d_mlt / (mx - mn);
  const int ncols_per = b_mlt + 1;
  int ncols_bZ = 0, nrows_bZ = 0;
  if ((long long)Yn_nrows * Wn_nrows > 0 && lf) {
    ncols_bZ = ncols_per * cpop_j;
    nrows_bZ = Yn_nrows;
    const long brows = bsize_c(nrows_bZ);
    if (!M_X->Ara) M_X->Ara = (unsigned char *)calloc((size_t)ncols_bZ * brows + 240, 1);
    unsigned char *bZ = M_X->Ara;
    memset(bZ, 0, (size_t)ncols_bZ * brows);
    for (long nr_a = 0; nr_a < Yn_nrows; nr_a++)
      if (bit_on(mr_j, nr_a)) bit_set(bZ, nr_a);
    long nc_j = 0, nc_b = 0;
    for (long nc_a = 0; nc_a < Wn_nrows; nc_a++) {
      if (!bit_on(mc_b, nc_a)) continue;
      if (bit_on(mc_j, nc_a)) {
        long nr_j = 0, nr_b = 0;
        for (long nr_a = 0; nr_a < Yn_nrows; nr_a++) {
          if (!bit_on(mr_b, nr_a)) continue;
          if (bit_on(mr_j, nr_a)) {
            double x = XGET(nr_j, nr_b, nr_a, nc_j, nc_b, nc_a);
            unsigned long long cz = (unsigned long long)(mlt * (double)(x - mn));
            if (cz < 1) cz = 1;
            if (cz > (unsigned long long)(g_d_mlt - 1)) cz = (unsigned long long)(g_d_mlt - 1);
            for (int nb = 0; nb < ncols_per - 1; nb++)
              if ((cz >> nb) & 1) bit_set(bZ + (long)(ncols_per * nc_j + ncols_per - 1 - nb) * brows, nr_a);
            nr_j++;
          }
          nr_b++;
        }
        nc_j++;
      }
      nc_b++;
    }
  }
#undef XGET
  M_X->nrows = ncols_bZ; M_X->ncols = nrows_bZ;
  M_X->nrows_extend = (16 - M_X->nrows % 16) % 16; M_X->mr_length = bsize_c(M_X->nrows);
  M_X->ncols_extend = (16 - M_X->ncols % 16) % 16; M_X->mc_length = bsize_c(M_X->ncols);
  for (int j = 0; j < ncols_bZ; j++) { bit_set(M_X->mr_b, j); bit_set(M_X->mr_j, j); }
  M_X->rpop_b = ncols_bZ; M_X->rpop_j = ncols_bZ;
  for (unsigned long i = 0; i < M_X->mc_length; i++) { M_X->mc_b[i] = mr_b[i]; M_X->mc_j[i] = mr_j[i]; }
  M_X->cpop_b = rpop_b; M_X->cpop_j = rpop_j;
  M_X->wX = M_X->Ara;
  M_X->ncols_per_z = ncols_per; M_X->max_d = mx; M_X->min_d = mn; M_X->mlt_d = mlt;
  if (!isfinite(M_X->mlt_d) || M_X->mlt_d <= 0) M_X->mlt_d = 1;
  mxget(M_X);
}

/* dir_c/At_T_YnWt_S_Zn_ww.c:5-190 (serial branch, :44-111) */
int lako_At_T_YnWt_S_Zn_ww(int spacing_a, int spacing_t, struct M_handle *M_At, struct M_handle *M_Tt,
                           struct M_handle *M_Yn, struct M_handle *M_Wn, struct M_handle *M_St,
                           struct M_handle *M_Zt, double *A_ajdk, struct M_handle *M_YnWt,
                           struct L_handle **out_p)
{
  (void)M_Yn;
  unsigned long long la = spacing_len(spacing_a, M_At), lt = spacing_len(spacing_t, M_Tt);
  struct L_handle *out = ensure(out_p, la * lt);
  if (!out) return (int)(la * lt);
  out->spacing_row = spacing_a; out->row_stride = la;
  out->spacing_col = spacing_t; out->col_stride = lt;
  const int A_pcols = (int)psize_c(M_At->nrows);
  const double *a_An = A_ajdk + 1 * A_pcols; /* AJDK_1_0 */
  const long nb = (long)M_At->mc_length;
  const int ncp = M_YnWt->ncols_per_z;
  const long long nT = M_Tt->rpop_j < M_St->rpop_j ? M_Tt->rpop_j : M_St->rpop_j;
  const long long nP = M_At->rpop_j < M_Zt->rpop_j ? M_At->rpop_j : M_Zt->rpop_j;
  const long long nW = M_Wn->rpop_j;
  double *ttmp = (double *)calloc((size_t)(nW ? nW : 1), sizeof(double));
  for (long long t = 0; t < nT; t++) {
    const unsigned char *St = M_St->wX + (long long)M_St->m_b_[t] * M_St->mc_length;
    const unsigned char *Tt = M_Tt->wX + (long long)M_Tt->m_b_[t] * M_Tt->mc_length;
    const unsigned char *p0 = M_YnWt->wX;
    const unsigned long long tab_t = pick(spacing_t, t, M_Tt->m_b_[t], M_Tt->m_a_[t]);
    const double tbase = (double)row_pmpm0(p0, Tt, p0, M_At->mc_j, nb) * M_YnWt->min_d * M_YnWt->mlt_d;
    for (long long mw = 0; mw < nW; mw++) {
      double s = 0;
      long long n2 = 1;
      for (int mx = ncp - 1; mx > 0; mx--) {
        double d = (double)row_pmpm0(p0, Tt, M_YnWt->wX + (long long)(ncp * mw + mx) * M_YnWt->mc_length, M_At->mc_j, nb);
        s += n2 * d;
        n2 *= 2;
      }
      ttmp[mw] = s;
    }
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads())
    for (long long i = 0; i < nP; i++) {
      const unsigned na_a = M_At->m_a_[i], nz_a = M_Zt->m_a_[i];
      const unsigned char *At = M_At->wX + (long long)M_At->m_b_[i] * M_At->mc_length;
      const unsigned char *Zt = M_Zt->wX + (long long)M_Zt->m_b_[i] * M_Zt->mc_length;
      const double Abase = (double)row_pmpm0(At, Tt, M_YnWt->wX, M_At->mc_j, nb) * M_YnWt->min_d * M_YnWt->mlt_d;
      double acc = 0;
      for (long long mw = 0; mw < nW; mw++) {
        const unsigned mw_a = M_Wn->m_a_[mw];
        const int vS = bit_pm(St, mw_a), vZ = bit_pm(Zt, mw_a);
        double Atmp = 0;
        long long n2 = 1;
        for (int mx = ncp - 1; mx > 0; mx--) {
          Atmp += n2 * row_pmpm0(At, Tt, M_YnWt->wX + (long long)(ncp * mw + mx) * M_YnWt->mc_length, M_At->mc_j, nb);
          n2 *= 2;
        }
        const double abase = tbase * a_An[na_a / 1920], atmp = ttmp[mw] * a_An[na_a / 1920];
        const double X = (double)(Abase + Atmp) / M_YnWt->mlt_d - (double)(abase + atmp) / M_YnWt->mlt_d;
        acc += X * vS * (vZ - a_An[nz_a / 1920]);
      }
      out->lf[pick(spacing_a, i, M_At->m_b_[i], na_a) + tab_t * la] = acc;
    }
  }
  free(ttmp);
  return (int)(la * lt);
}

/* dir_c/An_ZtSn_ww.c:5-136 */
int lako_An_ZtSn_ww(int spacing_a, int spacing_s, struct M_handle *M_An, struct M_handle *M_ZtSn,
                    struct M_handle *M_St, struct L_handle **out_p)
{
  unsigned long long la = spacing_len(spacing_a, M_An), ls = spacing_len(spacing_s, M_St);
  struct L_handle *out = ensure(out_p, la * ls);
  if (!out) return (int)(la * ls);
  out->spacing_row = spacing_a; out->row_stride = la;
  out->spacing_col = spacing_s; out->col_stride = ls;
  const long nb = (long)M_An->mc_length;
  const int ncp = M_ZtSn->ncols_per_z;
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (long long i = 0; i < M_An->rpop_j; i++) {
    const unsigned char *a = M_An->wX + (long long)M_An->m_b_[i] * M_An->mc_length;
    const double base = (double)row_pm0(a, M_ZtSn->wX, M_An->mc_j, nb) * M_ZtSn->min_d * M_ZtSn->mlt_d;
    for (long long s = 0; s < M_St->rpop_j; s++) {
      double tmp = 0;
      long long n2 = 1;
      for (int mx = ncp - 1; mx > 0; mx--) {
        double d = (double)row_pm0(a, M_ZtSn->wX + (long long)(ncp * s + mx) * M_ZtSn->mc_length, M_An->mc_j, nb);
        tmp += n2 * d;
        n2 *= 2;
      }
      out->lf[pick(spacing_a, i, M_An->m_b_[i], M_An->m_a_[i]) +
              pick(spacing_s, s, M_St->m_b_[s], M_St->m_a_[s]) * la] = (double)(base + tmp) / M_ZtSn->mlt_d;
    }
  }
  return (int)(la * ls);
}

/* dir_c/AnZt_S_WnYt_vv.c:5-101 */
int lako_AnZt_S_WnYt_vv(int spacing_a, int spacing_s, struct M_handle *M_An, struct M_handle *M_St,
                        struct M_handle *M_Zn, struct L_handle *lf_AnZt, struct L_handle *lf_YnWt,
                        struct L_handle **out_p)
{
  unsigned long long la = spacing_len(spacing_a, M_An), ls = spacing_len(spacing_s, M_St);
  struct L_handle *out = ensure(out_p, la * ls);
  if (!out) return (int)(la * ls);
  out->spacing_row = spacing_a; out->row_stride = la;
  out->spacing_col = spacing_s; out->col_stride = ls;
  if (!lf_AnZt || !lf_YnWt) return (int)(la * ls);
  for (long long s = 0; s < M_St->rpop_j; s++) {
    const unsigned char *St = M_St->wX + (long long)M_St->m_b_[s] * M_St->mc_length;
    const unsigned long long ts = pick(spacing_s, s, M_St->m_b_[s], M_St->m_a_[s]);
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads())
    for (long long ma = 0; ma < M_An->rpop_j; ma++) {
      const unsigned ma_a = M_An->m_a_[ma], ma_b = M_An->m_b_[ma];
      double acc = 0;
      for (long long mz = 0; mz < M_Zn->rpop_j; mz++) {
        const unsigned mz_a = M_Zn->m_a_[mz], mz_b = M_Zn->m_b_[mz];
        const int vS = bit_pm(St, mz_a);
        acc += (*L2(lf_AnZt, ma, ma_b, ma_a, mz, mz_b, mz_a)) * vS * (*L2(lf_YnWt, ma, ma_b, ma_a, mz, mz_b, mz_a));
      }
      out->lf[pick(spacing_a, ma, ma_b, ma_a) + ts * la] = acc;
    }
  }
  return (int)(la * ls);
}

/* dir_c/AtTYn_vv.c:5-202 */
int lako_AtTYn_vv(int spacing_a, int spacing_y, int spacing_t, struct M_handle *M_At, struct M_handle *M_Tt,
                  struct M_handle *M_Yt, double *A_ajdk, double *Y_ajdk, struct L_handle *lf_AtTn,
                  struct L_handle *lf_YtTn, struct L_handle **out_p)
{
  unsigned long long la = spacing_len(spacing_a, M_At), ly = spacing_len(spacing_y, M_Yt),
                     lt = spacing_len(spacing_t, M_Tt);
  struct L_handle *out = ensure(out_p, la * ly * lt);
  if (!out) return (int)(la * ly * lt);
  out->spacing_row = spacing_a; out->row_stride = la;
  out->spacing_col = spacing_y; out->col_stride = ly;
  out->spacing_lyr = spacing_t; out->lyr_stride = lt;
  const double *a_An = A_ajdk + 1 * psize_c(M_At->nrows), *a_Yn = Y_ajdk + 1 * psize_c(M_Yt->nrows);
  const long nb = (long)M_At->mc_length;
  for (long long t = 0; t < M_Tt->rpop_j; t++) {
    const unsigned t_a = M_Tt->m_a_[t], t_b = M_Tt->m_b_[t];
    const unsigned char *Tt = M_Tt->wX + (long long)t_b * M_Tt->mc_length;
    const long long hhay = -M_Tt->cpop_j + 2 * row_and(Tt, M_Tt->mc_j, (long)M_Tt->mc_length);
    const unsigned long long tab_t = pick(spacing_t, t, t_b, t_a);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads())
    for (long long na = 0; na < M_At->rpop_j; na++) {
      const unsigned na_a = M_At->m_a_[na], na_b = M_At->m_b_[na];
      const unsigned char *At = M_At->wX + (long long)na_b * M_At->mc_length;
      const long long hhAy = (long long)*L2(lf_AtTn, na, na_b, na_a, t, t_b, t_a);
      for (long long ny = 0; ny < M_Yt->rpop_j; ny++) {
        const unsigned ny_a = M_Yt->m_a_[ny], ny_b = M_Yt->m_b_[ny];
        const long long hhaY = (long long)*L2(lf_YtTn, ny, ny_b, ny_a, t, t_b, t_a);
        long long hhAY = M_At->cpop_j;
        hhAY -= 2 * row_notxorxor(At, Tt, M_Yt->wX + (long long)ny_b * M_Yt->mc_length, M_At->mc_j, nb);
        out->lf[pick(spacing_a, na, na_b, na_a) + pick(spacing_y, ny, ny_b, ny_a) * la + tab_t * la * ly] =
            (hhAY - hhAy * a_Yn[ny_a / 1920] - a_An[na_a / 1920] * hhaY + a_An[na_a / 1920] * hhay * a_Yn[ny_a / 1920]);
      }
    }
  }
  return (int)(la * ly * lt);
}

/* dir_c/AtTYn____WtSZn_vv.c:5-115 */
int lako_AtTYn____WtSZn_vv(int spacing_a, int spacing_s, struct M_handle *M_At, struct M_handle *M_Tt,
                           struct M_handle *M_Yt, struct M_handle *M_Wt, struct M_handle *M_St,
                           struct M_handle *M_Zt, double *Y_ajdk, struct L_handle *lf_AtTYn,
                           struct L_handle *lf_ZtSWn, struct L_handle **out_p)
{
  (void)M_Tt;
  unsigned long long la = spacing_len(spacing_a, M_At), ls = spacing_len(spacing_s, M_St);
  struct L_handle *out = ensure(out_p, la * ls);
  if (!out) return (int)(la * ls);
  out->spacing_row = spacing_a; out->row_stride = la;
  out->spacing_col = spacing_s; out->col_stride = ls;
  const double *D_Yn = Y_ajdk + 5 * psize_c(M_Yt->nrows); /* AJDK_0_1 */
  const long long nP = M_At->rpop_j < M_Zt->rpop_j ? M_At->rpop_j : M_Zt->rpop_j;
  const long long nI = M_Yt->rpop_j < M_Wt->rpop_j ? M_Yt->rpop_j : M_Wt->rpop_j;
  for (long long s = 0; s < M_St->rpop_j; s++) {
    const unsigned s_a = M_St->m_a_[s], s_b = M_St->m_b_[s];
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads())
    for (long long i = 0; i < nP; i++) {
      const unsigned na_a = M_At->m_a_[i], na_b = M_At->m_b_[i], nz_a = M_Zt->m_a_[i], nz_b = M_Zt->m_b_[i];
      double acc = 0;
      for (long long k = 0; k < nI; k++) {
        const unsigned ny_a = M_Yt->m_a_[k], ny_b = M_Yt->m_b_[k], nw_a = M_Wt->m_a_[k], nw_b = M_Wt->m_b_[k];
        acc += (*L3(lf_AtTYn, i, na_b, na_a, k, ny_b, ny_a, s, s_b, s_a)) * D_Yn[ny_a / 1920] *
               (*L3(lf_ZtSWn, i, nz_b, nz_a, k, nw_b, nw_a, s, s_b, s_a));
      }
      out->lf[pick(spacing_a, i, na_b, na_a) + pick(spacing_s, s, s_b, s_a) * la] = acc;
    }
  }
  return (int)(la * ls);
}

/* dir_c/AtTAn_vv.c:5-172: AtTYn_vv with Yt = At; each pair na_j <= ny_j is
   computed once and stored at (na, ny) and at (ny, na) (:99-113). */
int lako_AtTAn_vv(int spacing_a, int spacing_y, int spacing_t, struct M_handle *M_At, struct M_handle *M_Tt,
                  struct M_handle *M_Yt, double *A_ajdk, double *Y_ajdk, struct L_handle *lf_AtTn,
                  struct L_handle *lf_YtTn, struct L_handle **out_p)
{
  unsigned long long la = spacing_len(spacing_a, M_At), ly = spacing_len(spacing_y, M_Yt),
                     lt = spacing_len(spacing_t, M_Tt);
  struct L_handle *out = ensure(out_p, la * ly * lt);
  if (!out) return (int)(la * ly * lt);
  out->spacing_row = spacing_a; out->row_stride = la;
  out->spacing_col = spacing_y; out->col_stride = ly;
  out->spacing_lyr = spacing_t; out->lyr_stride = lt;
  const double *a_An = A_ajdk + 1 * psize_c(M_At->nrows), *a_Yn = Y_ajdk + 1 * psize_c(M_Yt->nrows);
  const long nb = (long)M_At->mc_length;
  for (long long t = 0; t < M_Tt->rpop_j; t++) {
    const unsigned t_a = M_Tt->m_a_[t], t_b = M_Tt->m_b_[t];
    const unsigned char *Tt = M_Tt->wX + (long long)t_b * M_Tt->mc_length;
    const long long hhay = -M_Tt->cpop_j + 2 * row_and(Tt, M_Tt->mc_j, (long)M_Tt->mc_length);
    const unsigned long long tab_t = pick(spacing_t, t, t_b, t_a);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads())
    for (long long na = 0; na < M_At->rpop_j; na++) {
      const unsigned na_a = M_At->m_a_[na], na_b = M_At->m_b_[na];
      const unsigned char *At = M_At->wX + (long long)na_b * M_At->mc_length;
      const long long hhAy = (long long)*L2(lf_AtTn, na, na_b, na_a, t, t_b, t_a);
      for (long long ny = na; ny < M_Yt->rpop_j; ny++) {
        const unsigned ny_a = M_Yt->m_a_[ny], ny_b = M_Yt->m_b_[ny];
        const long long hhaY = (long long)*L2(lf_YtTn, ny, ny_b, ny_a, t, t_b, t_a);
        long long hhAY = M_At->cpop_j;
        hhAY -= 2 * row_notxorxor(At, Tt, M_Yt->wX + (long long)ny_b * M_Yt->mc_length, M_At->mc_j, nb);
        const double v =
            (hhAY - hhAy * a_Yn[ny_a / 1920] - a_An[na_a / 1920] * hhaY + a_An[na_a / 1920] * hhay * a_Yn[ny_a / 1920]);
        out->lf[pick(spacing_a, na, na_b, na_a) + pick(spacing_y, ny, ny_b, ny_a) * la + tab_t * la * ly] = v;
        out->lf[pick(spacing_a, ny, ny_b, ny_a) + pick(spacing_y, na, na_b, na_a) * la + tab_t * la * ly] = v;
      }
    }
  }
  return (int)(la * ly * lt);
}

/* dir_c/At_T_YnWt_S_Zn_vv.c:5-85: the loop product element by element from
   the FP64 YnWt (no quantisation):
   out[na, ns] = sum_my (vA - a_An[na]) * vT * (sum_mw YnWt[my, mw] * vS * (vZ - a_An[nz])),
   At row na paired with Zt row nz, both sums in index order (:62-77). */
int lako_At_T_YnWt_S_Zn_vv(int spacing_a, int spacing_s, struct M_handle *M_At, struct M_handle *M_Tt,
                           struct M_handle *M_St, struct M_handle *M_Zt, double *A_ajdk,
                           struct L_handle *lf_YnWt, struct L_handle **out_p)
{
  unsigned long long la = spacing_len(spacing_a, M_At), ls = spacing_len(spacing_s, M_St);
  struct L_handle *out = ensure(out_p, la * ls);
  if (!out) return (int)(la * ls);
  out->spacing_row = spacing_a; out->row_stride = la;
  out->spacing_col = spacing_s; out->col_stride = ls;
  const double *a_An = A_ajdk + 1 * psize_c(M_At->nrows); /* AJDK_1_0 */
  const long long nP = M_At->rpop_j < M_Zt->rpop_j ? M_At->rpop_j : M_Zt->rpop_j;
  for (long long s = 0; s < M_St->rpop_j; s++) {
    const unsigned s_a = M_St->m_a_[s], s_b = M_St->m_b_[s];
    const unsigned char *Tt = M_Tt->wX + (long long)s_b * M_Tt->mc_length;
    const unsigned char *St = M_St->wX + (long long)s_b * M_St->mc_length;
    const unsigned long long ts = pick(spacing_s, s, s_b, s_a);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads())
    for (long long i = 0; i < nP; i++) {
      const unsigned na_a = M_At->m_a_[i], na_b = M_At->m_b_[i], nz_a = M_Zt->m_a_[i], nz_b = M_Zt->m_b_[i];
      const unsigned char *At = M_At->wX + (long long)na_b * M_At->mc_length;
      const unsigned char *Zt = M_Zt->wX + (long long)nz_b * M_Zt->mc_length;
      double acc = 0;
      for (long long my = 0; my < M_At->cpop_j; my++) {
        const unsigned my_a = M_At->n_a_[my], my_b = M_At->n_b_[my];
        const int vA = bit_pm(At, my_a), vT = bit_pm(Tt, my_a);
        double tmp = 0;
        for (long long mw = 0; mw < M_Zt->cpop_j; mw++) {
          const unsigned mw_a = M_Zt->n_a_[mw], mw_b = M_Zt->n_b_[mw];
          const int vS = bit_pm(St, mw_a), vZ = bit_pm(Zt, mw_a);
          tmp += (*L2(lf_YnWt, my, my_b, my_a, mw, mw_b, mw_a)) * vS * (vZ - a_An[nz_a / 1920]);
        }
        acc += (vA - a_An[na_a / 1920]) * vT * tmp;
      }
      out->lf[pick(spacing_a, i, na_b, na_a) + ts * la] = acc;
    }
  }
  return (int)(la * ls);
}

/* dir_c/An_ZtSWn_Yt_vv.c:5-130: out[ma, ns] = sum_ny [ (sum_na (vA - a_An[na]) * D_An[na] *
   ZtSWn[na, ny, ns]) * (D_Yn[ny] * (vY - a_Yn[ny])) ], An row ma paired with Yn row my,
   both sums in index order (:69-79; the OpenMP branch :95-115 keeps the same order per output). */
int lako_An_ZtSWn_Yt_vv(int spacing_a, int spacing_s, struct M_handle *M_An, struct M_handle *M_St,
                        struct M_handle *M_Yn, double *A_ajdk, double *Y_ajdk, struct L_handle *lf_ZtSWn,
                        struct L_handle **out_p)
{
  unsigned long long la = spacing_len(spacing_a, M_An), ls = spacing_len(spacing_s, M_St);
  struct L_handle *out = ensure(out_p, la * ls);
  if (!out) return (int)(la * ls);
  out->spacing_row = spacing_a; out->row_stride = la;
  out->spacing_col = spacing_s; out->col_stride = ls;
  if (!lf_ZtSWn) return (int)(la * ls);
  const long A_pcols = psize_c(M_An->ncols), Y_pcols = psize_c(M_Yn->ncols);
  const double *D_An = A_ajdk + 5 * A_pcols, *a_An = A_ajdk + 1 * A_pcols; /* AJDK_0_1, AJDK_1_0 */
  const double *D_Yn = Y_ajdk + 5 * Y_pcols, *a_Yn = Y_ajdk + 1 * Y_pcols;
  const long long nP = M_An->rpop_j < M_Yn->rpop_j ? M_An->rpop_j : M_Yn->rpop_j;
  for (long long s = 0; s < M_St->rpop_j; s++) {
    const unsigned s_a = M_St->m_a_[s], s_b = M_St->m_b_[s];
    const unsigned long long ts = pick(spacing_s, s, s_b, s_a);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads())
    for (long long i = 0; i < nP; i++) {
      const unsigned ma_a = M_An->m_a_[i], ma_b = M_An->m_b_[i], my_b = M_Yn->m_b_[i];
      const unsigned char *An = M_An->wX + (long long)ma_b * M_An->mc_length;
      const unsigned char *Yn = M_Yn->wX + (long long)my_b * M_Yn->mc_length;
      double acc = 0;
      for (long long ny = 0; ny < M_Yn->cpop_j; ny++) {
        const unsigned ny_a = M_Yn->n_a_[ny], ny_b = M_Yn->n_b_[ny];
        const int vY = bit_pm(Yn, ny_a);
        double tmp = 0;
        for (long long na = 0; na < M_An->cpop_j; na++) {
          const unsigned na_a = M_An->n_a_[na], na_b = M_An->n_b_[na];
          const int vA = bit_pm(An, na_a);
          tmp += (vA - a_An[na_a / 1920]) * D_An[na_a / 1920] * (*L3(lf_ZtSWn, na, na_b, na_a, ny, ny_b, ny_a, s, s_b, s_a));
        }
        tmp *= D_Yn[ny_a / 1920] * (vY - a_Yn[ny_a / 1920]);
        acc += tmp;
      }
      out->lf[pick(spacing_a, i, ma_b, ma_a) + ts * la] = acc;
    }
  }
  return (int)(la * ls);
}

/* popcount_pm0_lf (dir_c/popcount.c:556-621): per 1920-bit block the exact
   pm0 count d, then dout += D[block] * d in block order. */
static double row_pm0_lf(const unsigned char *a, const unsigned char *y, const unsigned char *m, long nbytes,
                         const double *D)
{
  double dout = 0;
  for (long b = 0; b < nbytes / BLK_BYTES; b++) {
    const long o = b * BLK_BYTES;
    const long long d = row_pm0(a + o, y + o, m + o, BLK_BYTES);
    dout += D[b] * (double)d;
  }
  return dout;
}

/* dir_c/An_ZtSWn_Yt_ww.c:5-111: the bit-plane form of An_ZtSWn_Yt_vv.  For
   each retained St row s, M_ZtSWn_[s] holds the planes (wrap_xcalc layout,
   ncols_per_z rows per retained Wt row, row 0 = the first mask plane) of one
   ZtSWn slice.  With pm0_lf(x, y; D) as above (mask M_An->mc_j),
     X(a, w) = (pm0_lf(An_a, p0; D01)*min*mlt + sum_k 2^k pm0_lf(An_a, plane(w, k); D01)) / mlt
             - (pm0_lf(p0, p0; D11)*min*mlt + sum_k 2^k pm0_lf(p0, plane(w, k); D11)) / mlt
     out[a, s] = sum over retained Wt rows w, in order, of X(a, w) * D_Yn[w] * (vY(a, w) - a_Yn[w])
   with the k sums taken from the least significant plane up (:59-67, :89-97)
   and An row a paired with Yn row a (:71). */
int lako_An_ZtSWn_Yt_ww(int spacing_a, int spacing_s, struct M_handle *M_An, struct M_handle *M_St,
                        struct M_handle **M_ZtSWn_, struct M_handle *M_Wt, struct M_handle *M_Yn,
                        double *A_ajdk, double *Y_ajdk, struct L_handle **out_p)
{
  unsigned long long la = spacing_len(spacing_a, M_An), ls = spacing_len(spacing_s, M_St);
  struct L_handle *out = ensure(out_p, la * ls);
  if (!out) return (int)(la * ls);
  out->spacing_row = spacing_a; out->row_stride = la;
  out->spacing_col = spacing_s; out->col_stride = ls;
  const long A_pcols = psize_c(M_An->ncols), Y_pcols = psize_c(M_Yn->ncols);
  const double *D01 = A_ajdk + AJDK_0_1 * A_pcols, *D11 = A_ajdk + AJDK_1_1 * A_pcols;
  const double *D_Yn = Y_ajdk + AJDK_0_1 * Y_pcols, *a_Yn = Y_ajdk + 1 * Y_pcols; /* AJDK_1_0 */
  const long nb = (long)M_An->mc_length;
  const long long nW = M_Wt->rpop_j;
  const long long nP = M_An->rpop_j < M_Yn->rpop_j ? M_An->rpop_j : M_Yn->rpop_j;
  double *t_ = (double *)malloc(sizeof(double) * (nW > 0 ? nW : 1));
  for (long long s = 0; s < M_St->rpop_j; s++) {
    const struct M_handle *Z = M_ZtSWn_[s];
    const int ncp = Z->ncols_per_z;
    const unsigned long long ts = pick(spacing_s, s, M_St->m_b_[s], M_St->m_a_[s]);
    const unsigned char *p0 = Z->wX;
    const double base_ = row_pm0_lf(p0, p0, M_An->mc_j, nb, D11) * Z->min_d * Z->mlt_d;
    for (long long w = 0; w < nW; w++) {
      double tmp = 0;
      long long n2 = 1;
      for (int mx = ncp - 1; mx > 0; mx--) {
        tmp += n2 * row_pm0_lf(p0, Z->wX + (long long)(ncp * w + mx) * Z->mc_length, M_An->mc_j, nb, D11);
        n2 *= 2;
      }
      t_[w] = tmp;
    }
#pragma omp parallel for schedule(dynamic, 4) num_threads(nthreads())
    for (long long i = 0; i < nP; i++) {
      const unsigned char *An = M_An->wX + (long long)M_An->m_b_[i] * M_An->mc_length;
      const unsigned char *Yn = M_Yn->wX + (long long)M_Yn->m_b_[i] * M_Yn->mc_length;
      const double baseA = row_pm0_lf(An, p0, M_An->mc_j, nb, D01) * Z->min_d * Z->mlt_d;
      double acc = 0;
      for (long long w = 0; w < nW; w++) {
        double tmp = 0;
        long long n2 = 1;
        for (int mx = ncp - 1; mx > 0; mx--) {
          tmp += n2 * row_pm0_lf(An, Z->wX + (long long)(ncp * w + mx) * Z->mc_length, M_An->mc_j, nb, D01);
          n2 *= 2;
        }
        const double X = (double)(baseA + tmp) / Z->mlt_d - (double)(base_ + t_[w]) / Z->mlt_d;
        const unsigned w_a = M_Wt->m_a_[w];
        const int vY = bit_pm(Yn, w_a);
        acc += X * D_Yn[w_a / 1920] * (vY - a_Yn[w_a / 1920]);
      }
      out->lf[pick(spacing_a, i, M_An->m_b_[i], M_An->m_a_[i]) + ts * la] = acc;
    }
  }
  free(t_);
  return (int)(la * ls);
}

/* dir_c/binary_read.c:174-269: wrap_transpose sets bit (7 - nc % 8) of byte
 * nc / 8 of output row nf from bit (7 - nf % 8) of byte nf / 8 of input record
 * nc, and clears the bits of the padding columns n_col..n_col+extend-1.  Here
 * every output byte starts at zero, so the padding bits stay zero. */
void lako_bits_transpose(const unsigned char *in, long long in_rec_bytes, int n_in_rec, unsigned char *out,
                         long long out_rec_bytes, int n_out_rec)
{
  memset(out, 0, (size_t)out_rec_bytes * (size_t)(n_out_rec > 0 ? n_out_rec : 0));
#pragma omp parallel for schedule(static)
  for (int r = 0; r < n_out_rec; ++r) {
    unsigned char *o = out + (size_t)r * (size_t)out_rec_bytes;
    for (int c = 0; c < n_in_rec; ++c) {
      const unsigned char b = (in[(size_t)c * (size_t)in_rec_bytes + (size_t)(r / 8)] >> (7 - r % 8)) & 1;
      o[c / 8] |= (unsigned char)(b << (7 - c % 8));
    }
  }
}

/* dir_c/M_Ax_to_L2.c:5-100 (at = 0, SNPs are the columns of M) and :137-280
 * (at = 1, SNPs are the rows): each retained entry becomes (b - a) * sqrt(d),
 * b = +1/-1 (TYPE_pm) or 1/0 (TYPE_00), a and d the A_ajdk terms of the
 * entry's SNP (b alone without A_ajdk); the whole output handle is zeroed
 * first (L_zero).  TYPE_p0 leaves it zero. */
int lako_M_to_L2(int at, int type_flag, int spacing_r, int spacing_c, struct M_handle *M, double *A_ajdk,
                 struct L_handle **out_p)
{
  unsigned long long lr = spacing_len(spacing_r, M), lc = 0;
  switch (spacing_c) {
    case LAKGB_SPACING_j: lc = (unsigned long long)M->cpop_j; break;
    case LAKGB_SPACING_b: lc = (unsigned long long)M->cpop_b; break;
    case LAKGB_SPACING_a: lc = (unsigned long long)M->ncols; break;
    default: break;
  }
  struct L_handle *out = ensure(out_p, lr * lc);
  if (!out) return (int)(lr * lc);
  memset(out->lf, 0, out->length * sizeof(double));
  out->spacing_row = spacing_r; out->row_stride = lr;
  out->spacing_col = spacing_c; out->col_stride = lc;
  out->spacing_lyr = LAKGB_SPACING_b; out->lyr_stride = 0;
  if (type_flag != LAKGB_TYPE_pm && type_flag != LAKGB_TYPE_00) return (int)(lr * lc);
  const long long P = psize_c(at ? M->nrows : M->ncols);
  for (long long ma = 0; ma < M->rpop_j; ma++) {
    const unsigned char *row = M->wX + (long long)M->m_b_[ma] * M->mc_length;
    for (long long na = 0; na < M->cpop_j; na++) {
      const unsigned int ca = M->n_a_[na];
      double v = (type_flag == LAKGB_TYPE_pm) ? (double)bit_pm(row, ca) : (double)bit_on(row, ca);
      if (A_ajdk) {
        const unsigned int snp = at ? M->m_a_[ma] : ca;
        const double a = A_ajdk[snp / 1920 + 1 * P], d = A_ajdk[snp / 1920 + AJDK_0_1 * P];
        v = (v - a) * sqrt(d);
      }
      unsigned long long tc = 0;
      switch (spacing_c) {
        case LAKGB_SPACING_j: tc = (unsigned long long)na; break;
        case LAKGB_SPACING_b: tc = M->n_b_[na]; break;
        case LAKGB_SPACING_a: tc = ca; break;
        default: break;
      }
      out->lf[tab(spacing_r, M, ma) + tc * lr] = v;
    }
  }
  return (int)(lr * lc);
}

/* dir_c/AnZt_mm.c:6-109 with the GSL CBLAS dgemm the reference links: every
 * element one running sum from +0 over k ascending, product and sum each
 * rounded once (this file is compiled without FP contraction). */
int lako_AnZt_mm(struct L_handle *lf_At, struct L_handle *lf_Zt, struct L_handle **out_p)
{
  const unsigned long long m = lf_At->col_stride, n = lf_Zt->col_stride, K = lf_At->row_stride;
  struct L_handle *out = ensure(out_p, m * n);
  if (!out) return (int)(m * n);
  out->spacing_row = lf_At->spacing_col; out->row_stride = m;
  out->spacing_col = lf_Zt->spacing_col; out->col_stride = n;
  if (K == 0 || lf_Zt->row_stride < K) return (int)(m * n);
  const unsigned long long ldb = lf_Zt->row_stride;
#pragma omp parallel for schedule(static) num_threads(nthreads())
  for (long long j = 0; j < (long long)n; j++)
    for (unsigned long long i = 0; i < m; i++) {
      double s = 0.0;
      for (unsigned long long k = 0; k < K; k++) s += lf_At->lf[k + i * K] * lf_Zt->lf[k + j * ldb];
      out->lf[i + j * m] = s;
    }
  return (int)(m * n);
}
