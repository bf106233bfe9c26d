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
  // The reference walks the n bits one at a time: every bit on in mb takes
  // the next b index, and those also on in mj are listed with their a and b
  // indices.  Same lists here, 64 elements at a time (bit 7 of a byte is its
  // first element, so a big-endian word holds element 64w + k at bit 63 - k):
  // empty words are skipped, full words written as one run, and in the
  // others only the listed bits are visited, their b index being b plus the
  // mb bits before them.
  if (n <= 0) return;
  unsigned b = 0, j = 0;
  const long nwords = (long)n / 64;
  for (long w = 0; w < nwords; ++w) {
    const uint64_t on_b = load_be64(mb + 8 * w);
    if (!on_b) continue;
    uint64_t on_j = on_b & load_be64(mj + 8 * w);
    const unsigned a0 = (unsigned)(64 * w);
    if (on_j == ~0ull) {
      for (unsigned k = 0; k < 64; ++k) { a_[j + k] = a0 + k; b_[j + k] = b + k; }
      j += 64; b += 64;
      continue;
    }
    while (on_j) {
      const int k = __builtin_clzll(on_j);
      const uint64_t before = k ? on_b >> (64 - k) : 0;  // mb bits of elements 64w .. 64w + k - 1
      a_[j] = a0 + (unsigned)k; b_[j] = b + (unsigned)__builtin_popcountll(before); ++j;
      on_j &= ~(0x8000000000000000ull >> k);
    }
    b += (unsigned)__builtin_popcountll(on_b);
  }
  const long nbytes = ((long)n + 7) / 8;
  for (long i = nwords * 8; i < nbytes; ++i) {
    unsigned on_b = mb[i];
    const long rest = (long)n - i * 8;
    if (rest < 8) on_b &= (0xFFu << (8 - rest)) & 0xFFu;  // bits past n are not elements
    if (!on_b) continue;
    const unsigned on_j = on_b & mj[i];
    while (on_b) {
      const int k = __builtin_clz(on_b) - 24;  // position from the byte's first element
      const unsigned bit = 0x80u >> k;
      if (on_j & bit) { b_[j] = b; a_[j] = (unsigned)(i * 8 + k); ++j; }
      ++b;
      on_b &= ~bit;
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
