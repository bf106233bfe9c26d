// Runtime shared by every translation unit of liblakgb300.so: the library's
// CUDA stream, error recording, launch accounting and a small residency cache
// that keeps uploaded bit matrices on the device between calls.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string>
#include <vector>

#include "../../include/lakcluster_gb300.h"

namespace lakgb {

// 1920-bit column block (POPLENGTH, dir_h/lakcluster_header.h:268): the unit
// over which the reference's column weights are constant.
constexpr int kBlockBits = 1920;
constexpr int kBlockBytes = 240;
constexpr int kBlockWords = 60;  // 32-bit words per block

// Record an error (first one wins until lakgb_last_error() reads it).
void set_error(int code, const char *fmt, ...);
// Abort on a CUDA error the way the reference aborts on fatal conditions.
void check_cuda(cudaError_t e, const char *what, const char *file, int line);
#define LAKGB_CUDA(x) ::lakgb::check_cuda((x), #x, __FILE__, __LINE__)

cudaStream_t stream();
// A second per-thread stream (non-blocking) for downloads that overlap the
// kernels on stream().
cudaStream_t copy_stream();
void count_launch(unsigned long long n = 1);

// Device allocation on the library stream (stream-ordered allocator).
void *dalloc(size_t bytes);
void dfree(void *p);

// Device copy of a host buffer.  With residency on (residency_enabled()),
// buffers are cached by (host pointer, size) and reused without re-upload;
// otherwise the copy goes into the call's staging arena (the caller holds a
// Stager across the call).
const void *resident(const void *host, size_t bytes);
bool residency_enabled();

// Whether wrap_xcalc copies its bit planes back into the host M_X (always,
// except inside a solve that does not trace its stages).
bool host_planes_wanted();

// Residency on for this thread while the object lives; cache entries this
// thread inserts meanwhile are dropped when the outermost scope ends.
struct ResidencyScope {
  ResidencyScope();
  ~ResidencyScope();
  ResidencyScope(const ResidencyScope &) = delete;
  ResidencyScope &operator=(const ResidencyScope &) = delete;
};

// A device buffer freed when the object goes out of scope (after the stream
// has drained the work that uses it).
struct DBuf {
  void *p = nullptr;
  size_t n = 0;
  bool owned = true;   // false: a view into the staging arena
  DBuf() = default;
  explicit DBuf(size_t bytes) : p(bytes ? dalloc(bytes) : nullptr), n(bytes) {}
  static DBuf view(const void *p, size_t n) {
    DBuf d;
    d.p = const_cast<void *>(p);
    d.n = n;
    d.owned = false;
    return d;
  }
  DBuf(const DBuf &) = delete;
  DBuf &operator=(const DBuf &) = delete;
  DBuf(DBuf &&o) noexcept : p(o.p), n(o.n), owned(o.owned) { o.p = nullptr; o.n = 0; }
  DBuf &operator=(DBuf &&o) noexcept {
    if (this != &o) {
      if (p && owned) dfree(p);
      p = o.p; n = o.n; owned = o.owned;
      o.p = nullptr; o.n = 0;
    }
    return *this;
  }
  ~DBuf() { if (p && owned) dfree(p); }
  template <class T> T *as() const { return static_cast<T *>(p); }
  void upload(const void *h, size_t bytes);
  void zero();
};

// Per-thread staging of a call's small host-to-device inputs: begin(), put()
// each array (host bytes are copied into a pinned arena, the returned device
// pointer is valid for kernels enqueued after flush()), flush() issues one
// copy for all of them.  Arrays that do not fit the arena are uploaded on
// their own.  One Stager per call; the arena is reused by the next call once
// its copy has completed.
constexpr size_t kStageBytes = 32u << 20;
// Arrays of at least this many bytes skip the arena (one direct copy each).
constexpr size_t kDirectUploadBytes = 1u << 20;
class Stager {
 public:
  Stager() { begin(); }
  ~Stager() { flush(); }
  Stager(const Stager &) = delete;
  Stager &operator=(const Stager &) = delete;
  void begin();
  template <class T> const T *put(const T *h, size_t n) {
    return static_cast<const T *>(put_bytes(h, n * sizeof(T)));
  }
  template <class V> const typename V::value_type *put(const V &v) { return put(v.data(), v.size()); }
  void flush();
  // Copy n host bytes in (arena or a dedicated buffer); the returned device
  // pointer is valid for kernels enqueued after flush() and before the
  // Stager is destroyed (a dedicated buffer is freed with it).
  const void *put_bytes(const void *h, size_t n);
 private:
  bool active_ = false;
  std::vector<DBuf> spill_;
  friend DBuf upload_bytes(const void *h, size_t n);
};

// The Stager of the current call on this thread (null outside one).
Stager *active_stager();

// Upload n host bytes: into the active Stager when there is one (a view into
// its arena, valid after its flush), else into a new device buffer.
DBuf upload_bytes(const void *h, size_t n);

// Make the device buffer `d`, which holds the current contents of the host
// buffer `host` (`bytes` bytes), its resident copy, replacing any earlier copy
// of that host buffer.  The cache takes ownership of the device memory.  With
// residency off the buffer is simply released.
void resident_put(const void *host, size_t bytes, DBuf &&d);

// Per-entry-point call counts and wall time (host clock, the call's own
// synchronisations included), collected when LAKGB_PROFILE_CALLS is set in
// the environment; read with lakgb_call_profile.
struct CallTimer {
  const char *name;
  long long t0;
  long long saved = 0;
  explicit CallTimer(const char *n);
  ~CallTimer();
  CallTimer(const CallTimer &) = delete;
  CallTimer &operator=(const CallTimer &) = delete;
};
#define LAKGB_PROFILE_CALL(name) ::lakgb::CallTimer lakgb_call_timer_(name)

// True when LAKGB_PROFILE_CALLS is set: the call timers above are collecting.
bool profile_calls_on();

// True while stream s is being captured into a CUDA graph.
bool capturing(cudaStream_t s);

// Events bracketing the most recent Gram launch (not recorded while s is
// being captured).
void gram_timer_begin(cudaStream_t s);
void gram_timer_end(cudaStream_t s);

}  // namespace lakgb
