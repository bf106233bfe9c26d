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
