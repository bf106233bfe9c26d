// 32 x 32 bit-matrix transpose in registers, one row per lane.
#pragma once

#include <cstdint>

namespace lakgb {

// Element (i, c) at bit 31 - c of lane i's word; afterwards lane r holds row
// r of the transpose.  Each step swaps the off-diagonal blocks of every
// 2j x 2j diagonal block (lanes j apart, bit groups j apart).
__device__ __forceinline__ uint32_t transpose32(uint32_t x, int lane) {
  const uint32_t masks[5] = {0x0000FFFFu, 0x00FF00FFu, 0x0F0F0F0Fu, 0x33333333u, 0x55555555u};
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int j = 16 >> k;
    const uint32_t m = masks[k];
    const uint32_t y = __shfl_xor_sync(0xffffffffu, x, j);
    x = (lane & j) ? ((x & m) | ((y << j) & ~m)) : ((x & ~m) | ((y >> j) & m));
  }
  return x;
}

}  // namespace lakgb
