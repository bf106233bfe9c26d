// Device entry for the row-vector scans An_v and An_ajdk_v.
#pragma once
#include <stdint.h>

namespace lakgb {

struct RowvecParams {
  const uint8_t *w;        // packed rows (M_An->wX)
  const uint32_t *rowb;    // wX row of the i-th retained row (M_An->m_b_)
  int n;                   // retained rows (rpop_j)
  long long row_bytes;     // mc_length
  const uint8_t *mask;     // mc_j
  int P;                   // 1920-bit blocks per row
  int type;                // 1: TYPE_pm, 2: TYPE_00
  long long cpop_j;        // An_v: retained column count
  const double *ajdk;      // An_ajdk: 15*P weights, weight k of block b at [b + k*P]
  const double *base;      // An_ajdk: 15 per-weight mask sums sum_b w_kb*popcnt(mask_b)
  const uint32_t *out_r;   // output row index of the i-th retained row
  long long out_stride;    // An_ajdk: output row stride (layer k at k*out_stride)
  double *out;
};

void launch_an_v(const RowvecParams &p);
void launch_an_ajdk(const RowvecParams &p);

}  // namespace lakgb
