// Library runtime: stream, errors, allocation, residency cache.
#include "lakgb_runtime.cuh"

#include <stdarg.h>
#include <stdlib.h>
#include <string.h>

#include <atomic>
#include <chrono>
#include <map>
#include <mutex>
#include <string>
#include <utility>

namespace lakgb {

namespace {
std::mutex g_mu;
int g_err = 0;
char g_msg[512] = {0};
std::atomic<unsigned long long> g_launches{0};
bool g_residency = false;
struct ResEntry { void *d; size_t n; };
std::map<std::pair<const void *, size_t>, ResEntry> g_res;
cudaEvent_t g_ev0 = nullptr, g_ev1 = nullptr;
bool g_ev_pending = false;
}  // namespace

// The first error of the calling thread since lakgb_thread_error_take read it
// (a solve checks its own thread's entry points; another thread's errors are
// not its own).
thread_local int t_err = 0;
thread_local char t_msg[256];

void set_error(int code, const char *fmt, ...) {
  char msg[256];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(msg, sizeof(msg), fmt, ap);
  va_end(ap);
  if (!t_err) {
    t_err = code;
    memcpy(t_msg, msg, sizeof(t_msg));
  }
  std::lock_guard<std::mutex> lk(g_mu);
  if (g_err) return;
  g_err = code;
  memcpy(g_msg, msg, sizeof(g_msg));
}

void check_cuda(cudaError_t e, const char *what, const char *file, int line) {
  if (e == cudaSuccess) return;
  set_error(1000 + (int)e, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
  fprintf(stderr, " %% Error! %s failed: %s (%s:%d)\n", what, cudaGetErrorString(e), file, line);
  exit(1);  // RET_NOMEM-style hard stop, as the reference does on fatal errors
}

// One non-blocking stream per host thread: solves run from different
// threads overlap on the device, while the calls of one solve stay ordered.
cudaStream_t stream() {
  thread_local cudaStream_t s = nullptr;
  if (!s) {
    cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      fprintf(stderr, " %% Error! no CUDA device usable by liblakgb300: %s\n", cudaGetErrorString(e));
      exit(1);
    }
  }
  return s;
}

cudaStream_t copy_stream() {
  thread_local cudaStream_t s = nullptr;
  if (!s) LAKGB_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
  return s;
}

// --- per-thread staging arena -----------------------------------------------

namespace {
struct Arena {
  unsigned char *host = nullptr;   // pinned
  unsigned char *dev = nullptr;
  size_t cap = 0, used = 0;
  cudaEvent_t done = nullptr;      // the last flush's copy has completed
  bool pending = false;
};
Arena &arena() {
  thread_local Arena a;
  return a;
}
}  // namespace

namespace {
thread_local Stager *t_active = nullptr;
// Residency scope of this thread (a whole solve): depth, and the cache keys
// inserted inside it, which are dropped when the outermost scope ends.
thread_local int t_scope_depth = 0;
thread_local std::vector<std::pair<const void *, size_t>> t_scope_keys;
}

Stager *active_stager() { return t_active; }

DBuf upload_bytes(const void *h, size_t n) {
  if (Stager *s = t_active) {
    const void *d = s->put_bytes(h, n);
    return DBuf::view(d, n);
  }
  DBuf d(n ? n : 1);
  d.upload(h, n);
  return d;
}

void Stager::begin() {
  t_active = this;
  Arena &a = arena();
  if (!a.host) {
    a.cap = kStageBytes;
    LAKGB_CUDA(cudaMallocHost((void **)&a.host, a.cap));
    LAKGB_CUDA(cudaMalloc((void **)&a.dev, a.cap));
    LAKGB_CUDA(cudaEventCreateWithFlags(&a.done, cudaEventDisableTiming));
  }
  if (a.pending) LAKGB_CUDA(cudaEventSynchronize(a.done));  // the host bytes are free again
  a.pending = false;
  a.used = 0;
  active_ = true;
}

const void *Stager::put_bytes(const void *h, size_t n) {
  LAKGB_PROFILE_CALL("(stage copy)");
  Arena &a = arena();
  const size_t off = (a.used + 255) & ~(size_t)255;
  if (!active_ || off + n > a.cap || n >= kDirectUploadBytes) {
    // Too large for the arena, or large enough that a direct copy from the
    // caller's memory beats a host-side copy into the arena first: a
    // dedicated buffer, uploaded in order.
    spill_.emplace_back(n ? n : 1);
    spill_.back().upload(h, n);
    return spill_.back().p;
  }
  if (n) memcpy(a.host + off, h, n);
  a.used = off + n;
  return a.dev + off;
}

void Stager::flush() {
  LAKGB_PROFILE_CALL("(staged upload)");
  Arena &a = arena();
  if (t_active == this) t_active = nullptr;
  if (!active_) return;
  if (a.used) {
    LAKGB_CUDA(cudaMemcpyAsync(a.dev, a.host, a.used, cudaMemcpyHostToDevice, stream()));
    LAKGB_CUDA(cudaEventRecord(a.done, stream()));
    a.pending = true;
  }
  active_ = false;
}

void count_launch(unsigned long long n) { g_launches += n; }

void *dalloc(size_t bytes) {
  LAKGB_PROFILE_CALL("(device alloc)");
  void *p = nullptr;
  LAKGB_CUDA(cudaMallocAsync(&p, bytes, stream()));
  return p;
}

void dfree(void *p) {
  LAKGB_PROFILE_CALL("(device free)");
  if (p) LAKGB_CUDA(cudaFreeAsync(p, stream()));
}

void DBuf::upload(const void *h, size_t bytes) {
  if (bytes) LAKGB_CUDA(cudaMemcpyAsync(p, h, bytes, cudaMemcpyHostToDevice, stream()));
}

void DBuf::zero() {
  if (n) LAKGB_CUDA(cudaMemsetAsync(p, 0, n, stream()));
}

// Caching is on for a thread inside a residency scope (a whole solve, which
// forgets every buffer it frees or rewrites) or process-wide after
// lakgb_set_residency(1).  Otherwise a call's matrices are uploaded afresh
// into its staging arena: a host buffer freed and reallocated at the same
// address must never be served from an old device copy.
bool residency_enabled() { return t_scope_depth > 0 || g_residency; }

// The cache entries of one host buffer (any size): the map is ordered by host
// pointer first, so they form one range.  Caller holds g_mu.
void erase_host_locked(const void *host) {
  auto it = g_res.lower_bound(std::make_pair(host, (size_t)0));
  while (it != g_res.end() && it->first.first == host) {
    cudaFreeAsync(it->second.d, stream());
    it = g_res.erase(it);
  }
}

const void *resident(const void *host, size_t bytes) {
  if (bytes == 0) return nullptr;
  stream();  // create the stream before taking the lock
  const auto key = std::make_pair(host, bytes);
  const bool on = residency_enabled();
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_res.find(key);
    if (on && it != g_res.end()) return it->second.d;
    if (it != g_res.end()) {
      cudaFreeAsync(it->second.d, stream());
      g_res.erase(it);
    }
  }
  if (!on && t_active) return t_active->put_bytes(host, bytes);
  // The copy is made without the lock, so other threads' lookups do not wait
  // for it; it completes before other threads' streams may read it.
  void *d = nullptr;
  LAKGB_CUDA(cudaMallocAsync(&d, bytes, stream()));
  LAKGB_CUDA(cudaMemcpyAsync(d, host, bytes, cudaMemcpyHostToDevice, stream()));
  LAKGB_CUDA(cudaStreamSynchronize(stream()));
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_res.find(key);
  if (it != g_res.end()) {  // another thread cached the same buffer meanwhile
    if (on) {
      cudaFreeAsync(d, stream());
      return it->second.d;
    }
    cudaFreeAsync(it->second.d, stream());
    g_res.erase(it);
  }
  g_res[key] = ResEntry{d, bytes};
  if (t_scope_depth > 0) t_scope_keys.push_back(key);
  return d;
}

void resident_put(const void *host, size_t bytes, DBuf &&d) {
  stream();
  std::lock_guard<std::mutex> lk(g_mu);
  erase_host_locked(host);
  if (!residency_enabled() || bytes == 0 || !d.p) return;  // d frees itself
  const auto key = std::make_pair(host, bytes);
  g_res[key] = ResEntry{d.p, bytes};
  if (t_scope_depth > 0) t_scope_keys.push_back(key);
  d.p = nullptr;
  d.n = 0;
}

ResidencyScope::ResidencyScope() { ++t_scope_depth; }

ResidencyScope::~ResidencyScope() {
  if (--t_scope_depth > 0) return;
  std::lock_guard<std::mutex> lk(g_mu);
  for (const auto &key : t_scope_keys) {
    auto it = g_res.find(key);
    if (it != g_res.end()) {
      cudaFreeAsync(it->second.d, stream());
      g_res.erase(it);
    }
  }
  t_scope_keys.clear();
}

bool profile_calls_on() {
  static const bool on = [] {
    const char *e = getenv("LAKGB_PROFILE_CALLS");
    return e && *e && *e != '0';
  }();
  return on;
}

namespace {
long long now_ns() {
  return std::chrono::duration_cast<std::chrono::nanoseconds>(std::chrono::steady_clock::now().time_since_epoch())
      .count();
}
struct CallStat {
  long long calls = 0, ns = 0, self_ns = 0;
};
std::mutex g_call_mu;
std::map<std::string, CallStat> g_calls;
thread_local long long t_child_ns = 0;  // time of the calls nested in the open one
}  // namespace

// LAKGB_SYNC_CALLS=1: every profiled entry point synchronises its stream on
// return and names itself if a device error is pending (a diagnostic for
// locating a failing kernel; it costs the overlap of host and device work).
bool sync_calls_on() {
  static const bool on = [] {
    const char *e = getenv("LAKGB_SYNC_CALLS");
    return e && *e && *e != '0';
  }();
  return on;
}

// Names of the profiled calls open on this thread, outermost first (for the
// LAKGB_SYNC_CALLS report).
thread_local std::vector<const char *> t_open_calls;

CallTimer::CallTimer(const char *n) : name(n), t0(0) {
  if (sync_calls_on()) t_open_calls.push_back(n);
  if (!profile_calls_on()) return;
  saved = t_child_ns;
  t_child_ns = 0;
  t0 = now_ns();
}

CallTimer::~CallTimer() {
  if (sync_calls_on()) {
    const cudaError_t e = cudaStreamSynchronize(stream());
    if (e != cudaSuccess) {
      fprintf(stderr, " %% Error! device error detected on leaving");
      for (const char *c : t_open_calls) fprintf(stderr, " %s", c);
      fprintf(stderr, ": %s\n", cudaGetErrorString(e));
      exit(1);
    }
    if (!t_open_calls.empty()) t_open_calls.pop_back();
  }
  if (!t0) return;
  const long long dt = now_ns() - t0;
  const long long self = dt - t_child_ns;
  t_child_ns = saved + dt;
  std::lock_guard<std::mutex> lk(g_call_mu);
  CallStat &c = g_calls[name];
  c.calls += 1;
  c.ns += dt;
  c.self_ns += self;
}

// True while s is being captured into a CUDA graph: nothing may synchronise
// or time it then.
bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  LAKGB_CUDA(cudaStreamIsCapturing(s, &st));
  return st != cudaStreamCaptureStatusNone;
}

void gram_timer_begin(cudaStream_t s) {
  if (capturing(s)) return;
  if (!g_ev0) {
    LAKGB_CUDA(cudaEventCreate(&g_ev0));
    LAKGB_CUDA(cudaEventCreate(&g_ev1));
  }
  LAKGB_CUDA(cudaEventRecord(g_ev0, s));
}

void gram_timer_end(cudaStream_t s) {
  if (capturing(s)) return;
  LAKGB_CUDA(cudaEventRecord(g_ev1, s));
  g_ev_pending = true;
}

}  // namespace lakgb

using namespace lakgb;

// High-water mark of the device memory the library's stream-ordered
// allocations hold (the current device's default memory pool, from which
// every working buffer, mirror and resident copy comes), optionally reset.
extern "C" long long lakgb_pool_high_water(int reset) {
  int dev = 0;
  LAKGB_CUDA(cudaGetDevice(&dev));
  cudaMemPool_t pool;
  LAKGB_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
  unsigned long long v = 0;
  LAKGB_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &v));
  if (reset) {
    unsigned long long zero = 0;
    LAKGB_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &zero));
  }
  return (long long)v;
}

extern "C" int lakgb_thread_error_take(char *msg, int msg_len) {
  const int e = lakgb::t_err;
  if (msg && msg_len > 0) {
    strncpy(msg, lakgb::t_msg, (size_t)msg_len - 1);
    msg[msg_len - 1] = 0;
  }
  lakgb::t_err = 0;
  lakgb::t_msg[0] = 0;
  return e;
}

extern "C" int lakgb_last_error(char *msg, int msg_len) {
  std::lock_guard<std::mutex> lk(g_mu);
  int e = g_err;
  if (msg && msg_len > 0) {
    strncpy(msg, g_msg, (size_t)msg_len - 1);
    msg[msg_len - 1] = 0;
  }
  g_err = 0;
  g_msg[0] = 0;
  return e;
}

extern "C" void lakgb_set_residency(int on) {
  stream();
  std::lock_guard<std::mutex> lk(g_mu);
  g_residency = (on != 0);
  if (!g_residency) {
    for (auto &kv : g_res) cudaFreeAsync(kv.second.d, stream());
    g_res.clear();
  }
}

namespace lakgb {
namespace {
thread_local int t_device_only_planes = 0;
}
bool host_planes_wanted() { return !t_device_only_planes || !residency_enabled(); }
}  // namespace lakgb

// Inside a solve: bit planes made by wrap_xcalc stay on the device only (the
// driver reads them through the residency cache, never on the host).
extern "C" void lakgb_device_only_planes(int on) { lakgb::t_device_only_planes = on ? 1 : 0; }

extern "C" void lakgb_residency_scope(int enter) {
  thread_local std::vector<lakgb::ResidencyScope *> scopes;
  if (enter) {
    scopes.push_back(new lakgb::ResidencyScope());
  } else if (!scopes.empty()) {
    delete scopes.back();
    scopes.pop_back();
  }
}

extern "C" void lakgb_forget_host_buffer(const void *host_ptr) {
  stream();
  std::lock_guard<std::mutex> lk(lakgb::g_mu);
  lakgb::erase_host_locked(host_ptr);
}

extern "C" unsigned long long lakgb_kernel_launches(void) { return g_launches.load(); }

extern "C" int lakgb_call_profile(char *buf, int buf_len) {
  std::string out = "{";
  {
    std::lock_guard<std::mutex> lk(g_call_mu);
    bool first = true;
    for (const auto &kv : g_calls) {
      char line[256];
      snprintf(line, sizeof line, "%s\"%s\":{\"calls\":%lld,\"seconds\":%.6f,\"self_seconds\":%.6f}",
               first ? "" : ",", kv.first.c_str(), kv.second.calls, kv.second.ns * 1e-9, kv.second.self_ns * 1e-9);
      out += line;
      first = false;
    }
  }
  out += "}";
  if (buf && buf_len > 0) {
    strncpy(buf, out.c_str(), (size_t)buf_len - 1);
    buf[buf_len - 1] = 0;
  }
  return (int)out.size();
}

extern "C" void lakgb_call_profile_reset(void) {
  std::lock_guard<std::mutex> lk(g_call_mu);
  g_calls.clear();
}

extern "C" double lakgb_last_gram_ms(void) {
  if (!g_ev_pending) return 0.0;
  float ms = 0.f;
  LAKGB_CUDA(cudaEventSynchronize(g_ev1));
  LAKGB_CUDA(cudaEventElapsedTime(&ms, g_ev0, g_ev1));
  return (double)ms;
}
