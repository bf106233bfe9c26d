// Host-side helpers shared by the reference-compatible entry points:
// output allocation with the reference's semantics, spacing arithmetic and
// small upload / download wrappers.
#pragma once
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <vector>

#include "lakgb_runtime.cuh"

namespace lakgb {

inline unsigned long long spacing_length(int spacing, const M_handle *M) {
  switch (spacing) {
    case LAKGB_SPACING_j: return (unsigned long long)M->rpop_j;
    case LAKGB_SPACING_b: return (unsigned long long)M->rpop_b;
    case LAKGB_SPACING_a: return (unsigned long long)M->nrows;
    default: return 0;
  }
}

// Index of the j-th retained row in the given spacing (AnZt_vv.c:71-77).
inline std::vector<uint32_t> spacing_index(int spacing, const M_handle *M) {
  std::vector<uint32_t> v((size_t)M->rpop_j);
  for (long long j = 0; j < M->rpop_j; ++j) {
    switch (spacing) {
      case LAKGB_SPACING_j: v[j] = (uint32_t)j; break;
      case LAKGB_SPACING_b: v[j] = M->m_b_[j]; break;
      case LAKGB_SPACING_a: v[j] = M->m_a_[j]; break;
      default: v[j] = 0; break;
    }
  }
  return v;
}

// Allocate (malloc, zero-filled) or check-and-zero the output, as the
// reference wrappers do (AnZt_vv.c:203-204).  zero_host = false leaves an
// existing buffer's zero-fill to a HostOutputFill (below), for calls whose
// device result, zeros included, is copied over the whole output anyway.
inline L_handle *ensure_output(L_handle **pp, unsigned long long length, const char *who,
                               bool zero_host = true) {
  if (*pp == nullptr) {
    L_handle *L = (L_handle *)calloc(1, sizeof(L_handle));
    L->length = length;
    L->lf = (double *)calloc(length ? length : 1, sizeof(double));
    if (!L->lf) {
      fprintf(stderr, " %% Warning! out of memory in %s\n", who);
      exit(1);  // RET_NOMEM
    }
    *pp = L;
  }
  L_handle *L = *pp;
  if (L->length < length) {
    printf(" %% Warning! length %llu<%llu in %s\n", L->length, length, who);
    set_error(2, "output length %llu < %llu in %s", L->length, length, who);
    return nullptr;
  }
  if (zero_host) memset(L->lf, 0, length * sizeof(double));
  return L;
}

// The zero-fill of a host output that ensure_output(..., false) skipped: done
// when the call returns without copying the full device result over it.
struct HostOutputFill {
  L_handle *L = nullptr;
  unsigned long long n = 0;
  bool copied = false;
  HostOutputFill() = default;
  HostOutputFill(const HostOutputFill &) = delete;
  HostOutputFill &operator=(const HostOutputFill &) = delete;
  ~HostOutputFill() {
    if (L && !copied && n) memset(L->lf, 0, n * sizeof(double));
  }
};

inline int popcount_bytes(const unsigned char *p, long n) {
  int c = 0;
  for (long i = 0; i < n; ++i) c += __builtin_popcount((unsigned)p[i]);
  return c;
}

inline long long popcount_bytes_masked(const unsigned char *p, const unsigned char *m, long n) {
  long long c = 0;
  for (long i = 0; i < n; ++i) c += __builtin_popcount((unsigned)(p[i] & m[i]));
  return c;
}

template <class T>
inline DBuf upload_vec(const std::vector<T> &v) {
  return upload_bytes(v.data(), v.size() * sizeof(T));
}

// Deferral scopes (lakgb_defer_begin / lakgb_defer_end, loopsum.cu): whether
// this host thread is inside one, and a group of held-back calls that another
// translation unit keeps -- `enqueue` launches them and their copies back to
// the host on the library stream when the outermost scope ends, `clear`
// (after the stream has drained) sets what they leave in host structs and
// releases them.
bool defer_active();
void defer_register(void (*enqueue)(), void (*clear)());
// A copy of `length` doubles of `dev` into `host`, made when the scope ends.
void defer_copy(double *host, DBuf &&dev, unsigned long long length);
// Small inputs of a held-back call: copied into this thread's page-locked
// scope chunks (reused from scope to scope) and sent by defer_flush() with one
// asynchronous copy per call; the device pointer stays valid until the
// outermost scope ends.
const void *defer_put(const void *h, size_t n);
void defer_flush();
template <class T>
inline DBuf defer_upload(const std::vector<T> &v) {
  const size_t n = v.size() * sizeof(T);
  return DBuf::view(defer_put(v.data(), n), n);
}

// The call's device output into its host L_handle -- inside a deferral scope
// when the scope ends (the device buffer is kept until then).
inline void copy_back(double *host, DBuf &dev, unsigned long long length, HostOutputFill *fill = nullptr) {
  if (defer_active()) {
    if (fill) fill->copied = true;
    defer_copy(host, std::move(dev), length);
    return;
  }
  if (profile_calls_on()) {  // time the wait for the producing kernels apart from the copy
    LAKGB_PROFILE_CALL("(kernel wait)");
    LAKGB_CUDA(cudaStreamSynchronize(stream()));
  }
  LAKGB_PROFILE_CALL("(copy back + sync)");
  if (fill) fill->copied = true;
  if (length) LAKGB_CUDA(cudaMemcpyAsync(host, dev.p, length * sizeof(double), cudaMemcpyDeviceToHost, stream()));
  LAKGB_CUDA(cudaStreamSynchronize(stream()));
}

}  // namespace lakgb
