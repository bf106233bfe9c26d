// Device mirrors of L_handles (see lmirror.cu).
#pragma once
#include "lakgb_runtime.cuh"

namespace lakgb {

struct Mirror {
  double *d = nullptr;          // L->length doubles on the device
  unsigned long long n = 0;
  bool host_stale = false;      // the device copy is newer than L->lf
};

// The mirror of L, or null when L is not mirrored.
Mirror *find_mirror(const L_handle *L);

}  // namespace lakgb
