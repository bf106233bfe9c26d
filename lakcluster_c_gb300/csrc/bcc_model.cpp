// Host-side reference data model helpers (see bcc_model.h).
#include "bcc_model.h"

#include <stdio.h>

namespace lakbcc {

static void mh_init(MH *M, int nrows, int ncols, unsigned char *rows, const unsigned char *mr_b,
                    const unsigned char *mc_b) {
  M_handle &h = M->h;
  memset(&h, 0, sizeof(h));
  h.header_length = 3 * (int)sizeof(int);
  h.bitj = BITJ;
  h.nrows = nrows;
  h.ncols = ncols;
  h.nrows_extend = (BITJ - nrows % BITJ) % BITJ;
  h.ncols_extend = (BITJ - ncols % BITJ) % BITJ;
  h.mr_length = (unsigned long)bsize(nrows);
  h.mc_length = (unsigned long)bsize(ncols);
  h.cc_length = (unsigned long)((ncols + h.ncols_extend) / BIT8);
  // Masks carry one zeroed 1920-bit block of slack: the reference's SSE
  // popcount loops always process at least one block, even for zero-length
  // rows (e.g. a transposed control matrix with no controls).
  M->mr_b.assign(h.mr_length + POPLENGTH / BIT8, 0);
  M->mr_j.assign(h.mr_length + POPLENGTH / BIT8, 0);
  M->mc_b.assign(h.mc_length + POPLENGTH / BIT8, 0);
  M->mc_j.assign(h.mc_length + POPLENGTH / BIT8, 0);
  if (mr_b) memcpy(M->mr_b.data(), mr_b, h.mr_length);
  else for (int r = 0; r < nrows; ++r) bset_on(M->mr_b.data(), r);
  if (mc_b) memcpy(M->mc_b.data(), mc_b, h.mc_length);
  else for (int c = 0; c < ncols; ++c) bset_on(M->mc_b.data(), c);
  M->mr_j = M->mr_b;
  M->mc_j = M->mc_b;
  M->m_a.assign(nrows > 0 ? nrows : 1, 0);
  M->m_b.assign(nrows > 0 ? nrows : 1, 0);
  M->n_a.assign(ncols > 0 ? ncols : 1, 0);
  M->n_b.assign(ncols > 0 ? ncols : 1, 0);
  M->rsum.assign(nrows > 0 ? nrows : 1, 0.0);
  h.mr_b = M->mr_b.data(); h.mr_j = M->mr_j.data();
  h.mc_b = M->mc_b.data(); h.mc_j = M->mc_j.data();
  h.m_a_ = M->m_a.data(); h.m_b_ = M->m_b.data();
  h.n_a_ = M->n_a.data(); h.n_b_ = M->n_b.data();
  h.rsum = M->rsum.data();
  h.Ara = rows;
  h.wX = rows;
  h.mlt_d = 1.0;
  mh_mxget(M);
}

MH *mh_make(int nrows, int ncols, unsigned char *rows, const unsigned char *mr_b,
            const unsigned char *mc_b) {
  MH *M = new MH();
  mh_init(M, nrows, ncols, rows, mr_b, mc_b);
  return M;
}

MH *mh_make_owned(int nrows, int ncols) {
  MH *M = new MH();
  M->own_rows.assign((size_t)(nrows > 0 ? nrows : 1) * (size_t)bsize(ncols) + POPLENGTH / BIT8, 0);
  mh_init(M, nrows, ncols, M->own_rows.data(), nullptr, nullptr);
  return M;
}

static void mxget_excerpt(int n, const unsigned char *mb, const unsigned char *mj, long long *pop_b,
                          long long *pop_j, unsigned int *a_, unsigned int *b_, long length) {
  *pop_b = popcount_bytes(mb, length);
  *pop_j = popcount_bytes(mj, length);
  int a = 0, b = 0, j = 0;
  while (a < n) {
    while (a < n && !bget_on(mb, a)) a++;
    if (a < n && bget_on(mb, a) && bget_on(mj, a)) {
      b_[j] = (unsigned)b; a_[j] = (unsigned)a;
      j++; b++; a++;
    } else if (a < n && bget_on(mb, a)) {
      b++; a++;
    }
  }
}

void mhandle_mxget(M_handle *h) {
  mxget_excerpt(h->nrows, h->mr_b, h->mr_j, &h->rpop_b, &h->rpop_j, h->m_a_, h->m_b_, (long)h->mr_length);
  mxget_excerpt(h->ncols, h->mc_b, h->mc_j, &h->cpop_b, &h->cpop_j, h->n_a_, h->n_b_, (long)h->mc_length);
}

void mh_mxget(MH *M) { mhandle_mxget(&M->h); }

void mh_mxset(MH *M, const unsigned char *mr_j, const unsigned char *mc_j) {
  M_handle &h = M->h;
  if (mr_j) {
    for (unsigned long i = 0; i < h.mr_length; ++i) h.mr_j[i] = mr_j[i] & h.mr_b[i];
  }
  if (mc_j) {
    for (unsigned long i = 0; i < h.mc_length; ++i) h.mc_j[i] = mc_j[i] & h.mc_b[i];
  }
  mh_mxget(M);
}

L_handle *lh_make(unsigned long long length) {
  L_handle *L = (L_handle *)calloc(1, sizeof(L_handle));
  L->length = length;
  L->lf = (double *)calloc(length ? length : 1, sizeof(double));
  if (!L->lf) {
    fprintf(stderr, " %% Warning! out of memory in lh_make (%llu doubles)\n", length);
    exit(1);
  }
  L->spacing_row = SP_b; L->spacing_col = SP_b; L->spacing_lyr = SP_b;
  return L;
}

void lh_free(L_handle *L) {
  if (!L) return;
  free(L->lf);
  free(L);
}

void lh_zero(L_handle *L) {
  if (L) memset(L->lf, 0, L->length * sizeof(double));
}

void lh_transpose(L_handle *L1, const L_handle *L2) {
  L1->spacing_row = L2->spacing_col; L1->spacing_col = L2->spacing_row; L1->spacing_lyr = L2->spacing_lyr;
  L1->row_stride = L2->col_stride; L1->col_stride = L2->row_stride; L1->lyr_stride = L2->lyr_stride;
  for (unsigned long long c = 0; c < L2->col_stride; ++c)
    for (unsigned long long r = 0; r < L2->row_stride; ++r)
      L1->lf[c + r * L1->row_stride] = L2->lf[r + c * L2->row_stride];
}

void lh_duplicate(L_handle *L1, const L_handle *L2) {
  L1->spacing_row = L2->spacing_row; L1->spacing_col = L2->spacing_col; L1->spacing_lyr = L2->spacing_lyr;
  L1->row_stride = L2->row_stride; L1->col_stride = L2->col_stride; L1->lyr_stride = L2->lyr_stride;
  for (unsigned long long c = 0; c < L2->col_stride; ++c)
    for (unsigned long long r = 0; r < L2->row_stride; ++r)
      L1->lf[r + c * L1->row_stride] = L2->lf[r + c * L2->row_stride];
}

}  // namespace lakbcc
