// Host-side helpers for the reference data model used by the bcc driver:
// building M_handles over packed rows, maintaining their masks and index
// lists, and element access to L_handles in the three index spacings.
// Semantics follow dir_c/M_init.c (M_handle_v_make :376-416, M_mxget :268-295,
// M_mxset :359-374) and dir_c/L_init.c (L2_get/L2_set/... :74-170).
#pragma once
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "../../include/lakcluster_gb300.h"

namespace lakbcc {

constexpr int BITJ = 16;
constexpr int BIT8 = 8;
constexpr int POPLENGTH = 1920;
constexpr int SP_b = LAKGB_SPACING_b, SP_j = LAKGB_SPACING_j, SP_a = LAKGB_SPACING_a;
constexpr int T_pm = LAKGB_TYPE_pm;
enum {
  AJDK_0_0 = 0, AJDK_1_0, AJDK_2_0, AJDK_3_0, AJDK_4_0,
  AJDK_0_1, AJDK_1_1, AJDK_2_1, AJDK_3_1, AJDK_4_1,
  AJDK_0_2, AJDK_1_2, AJDK_2_2, AJDK_3_2, AJDK_4_2, AJDK_TOT
};

inline long rup(long a, long b) { return a + (a % b ? b - a % b : 0); }
inline long bsize(long n) { return rup(n + (BITJ - n % BITJ) % BITJ, POPLENGTH) / BIT8; }
inline long psize(long n) { return rup(n + (BITJ - n % BITJ) % BITJ, POPLENGTH) / POPLENGTH; }

inline int bget_on(const unsigned char *b, long n) { return (b[n / 8] >> (7 - n % 8)) & 1; }
inline int bget_pm(const unsigned char *b, long n) { return (int)(((b[n / 8] >> (7 - n % 8)) & 1) << 1) - 1; }
inline void bset_on(unsigned char *b, long n) { b[n / 8] |= (unsigned char)(1 << (7 - n % 8)); }
inline void bset_off(unsigned char *b, long n) { b[n / 8] &= (unsigned char)~(1 << (7 - n % 8)); }

inline unsigned popcount_bytes(const unsigned char *p, long n) {
  unsigned c = 0;
  long i = 0;
  for (; i + 8 <= n; i += 8) {
    uint64_t w;
    memcpy(&w, p + i, 8);
    c += (unsigned)__builtin_popcountll(w);
  }
  for (; i < n; ++i) c += (unsigned)__builtin_popcount((unsigned)p[i]);
  return c;
}

// Eight mask bytes as one word whose bit 63 is the first byte's bit 7 (the
// masks' first element), whatever the host's byte order.
inline uint64_t load_be64(const unsigned char *p) {
  uint64_t w;
  memcpy(&w, p, 8);
#if defined(__BYTE_ORDER__) && __BYTE_ORDER__ == __ORDER_LITTLE_ENDIAN__
  w = __builtin_bswap64(w);
#endif
  return w;
}

// Owning wrapper around an M_handle.  wX either points at another handle's
// rows (shared, never freed here) or at rows owned by this object.
struct MH {
  M_handle h{};
  std::vector<unsigned char> own_rows;
  std::vector<unsigned char> mr_b, mr_j, mc_b, mc_j;
  std::vector<unsigned int> m_a, m_b, n_a, n_b;
  std::vector<double> rsum;
  M_handle *p() { return &h; }
};

// M_handle_v_make (M_init.c:376-416) over rows already compacted by mr_b.
// mr_b / mc_b may be null (all on).  The current masks start equal to the
// base masks.
MH *mh_make(int nrows, int ncols, unsigned char *rows, const unsigned char *mr_b,
            const unsigned char *mc_b);
// Same, owning a zeroed row buffer of nrows x bsize(ncols) bytes.
MH *mh_make_owned(int nrows, int ncols);
// M_mxget (M_init.c:268-295): pops and index lists from the masks.
void mh_mxget(MH *M);
// The same on a bare M_handle whose mask and index arrays are already sized.
void mhandle_mxget(M_handle *h);
// M_mxset (M_init.c:359-374): current masks = given & base, then mxget.
void mh_mxset(MH *M, const unsigned char *mr_j, const unsigned char *mc_j);

// L_handle helpers -----------------------------------------------------------
L_handle *lh_make(unsigned long long length);
void lh_free(L_handle *L);
void lh_zero(L_handle *L);
inline unsigned long long pick(int spacing, unsigned long long j, unsigned long long b,
                               unsigned long long a) {
  return spacing == SP_j ? j : (spacing == SP_b ? b : a);
}
inline double *L2_get(L_handle *L, unsigned long long rj, unsigned long long rb, unsigned long long ra,
                      unsigned long long cj, unsigned long long cb, unsigned long long ca) {
  return &L->lf[pick(L->spacing_row, rj, rb, ra) + pick(L->spacing_col, cj, cb, ca) * L->row_stride];
}
inline double *L1_get(L_handle *L, unsigned long long rj, unsigned long long rb, unsigned long long ra) {
  return &L->lf[pick(L->spacing_row, rj, rb, ra)];
}
inline double *L3_get(L_handle *L, unsigned long long rj, unsigned long long rb, unsigned long long ra,
                      unsigned long long cj, unsigned long long cb, unsigned long long ca,
                      unsigned long long lj, unsigned long long lb, unsigned long long la) {
  return &L->lf[pick(L->spacing_row, rj, rb, ra) + pick(L->spacing_col, cj, cb, ca) * L->row_stride +
                pick(L->spacing_lyr, lj, lb, la) * L->row_stride * L->col_stride];
}
// L2_transpose / L2_duplicate (L_init.c:31-45): L1 takes L2's values.
void lh_transpose(L_handle *L1, const L_handle *L2);
void lh_duplicate(L_handle *L1, const L_handle *L2);

}  // namespace lakbcc
