// +/-1 Gram of packed bit rows, popcount path.
//
// out[i,k] = a0d1 - 2*S_ik - ((lfA_i + lfZ_k) - a2d1),   S_ik = sum_blocks D_b * c_ikb
// where c_ikb = popcount((A_i xor Z_k) & mask) over 1920-bit block b (TYPE_pm)
// or popcount(A_i & Z_k & mask) (TYPE_00, out = S_ik).
// This is the arithmetic of get_AnZt_vv__run (dir_c/AnZt_vv.c:62-95) with the
// block-weighted popcount of popcount_xor_lf / popcount_and_lf
// (dir_c/popcount.c:310-423).  The integer counts are exact; the FP64 combine
// keeps the reference's order -- one multiply and one add per block, blocks in
// ascending order, no fused multiply-add -- so every output is bit-identical.
//
// Layout: each CTA owns a BM x BN tile of (A rows) x (Z rows).  Per 1920-bit
// block it stages the tile's BM + BN masked row segments (240 B each) in
// shared memory (row pitch 61 words: conflict-free column reads), every
// thread accumulates a TM x TN micro-tile of integer counts over the block's
// 60 words, then folds them into FP64 accumulators with the block weight.
// For launches with few tiles the same staging and counting run split over
// blocks (one CTA per tile and block, counts to a scratch array), followed by
// a kernel that does the fold in block order.
#include <string.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>
#include <climits>

#include "gram.cuh"
#include "lakgb_runtime.cuh"

namespace lakgb {

namespace {

constexpr int kLd = kBlockWords + 1;  // smem row pitch in words

// Stage the masked 240-byte segments of block `blk` of the tile's BM + BN
// rows in shared memory (zeros for rows past the end).
template <int BM, int BN, int NT>
__device__ __forceinline__ void stage_block(const GramParams &p, int blk, uint32_t *As, uint32_t *Zs,
                                            const long long *a_off, const long long *z_off, int tid) {
  const long long boff = (long long)blk * kBlockBytes;
  const uint4 *mk = reinterpret_cast<const uint4 *>(p.mask + boff);
  for (int idx = tid; idx < BM * 15; idx += NT) {
    const int r = idx / 15, v = idx - r * 15;
    uint4 x = make_uint4(0u, 0u, 0u, 0u);
    const long long o = a_off[r];
    if (o >= 0) {
      const uint4 m = __ldg(mk + v);
      x = __ldg(reinterpret_cast<const uint4 *>(p.wA + o + boff) + v);
      x.x &= m.x; x.y &= m.y; x.z &= m.z; x.w &= m.w;
    }
    uint32_t *d = As + r * kLd + 4 * v;
    d[0] = x.x; d[1] = x.y; d[2] = x.z; d[3] = x.w;
  }
  for (int idx = tid; idx < BN * 15; idx += NT) {
    const int r = idx / 15, v = idx - r * 15;
    uint4 x = make_uint4(0u, 0u, 0u, 0u);
    const long long o = z_off[r];
    if (o >= 0) {
      const uint4 m = __ldg(mk + v);
      x = __ldg(reinterpret_cast<const uint4 *>(p.wZ + o + boff) + v);
      x.x &= m.x; x.y &= m.y; x.z &= m.z; x.w &= m.w;
    }
    uint32_t *d = Zs + r * kLd + 4 * v;
    d[0] = x.x; d[1] = x.y; d[2] = x.z; d[3] = x.w;
  }
}

// Integer counts of one staged block for this thread's TM x TN micro-tile
// (rows ty + i*TY of A, tx + j*TX of Z).
template <int TM, int TN, int TX, int TY, int TYPE>
__device__ __forceinline__ void count_block(const uint32_t *As, const uint32_t *Zs, int tx, int ty,
                                            int (&cnt)[TM][TN]) {
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) cnt[i][j] = 0;
#pragma unroll 4
  for (int w = 0; w < kBlockWords; ++w) {
    uint32_t a[TM], z[TN];
#pragma unroll
    for (int i = 0; i < TM; ++i) a[i] = As[(ty + i * TY) * kLd + w];
#pragma unroll
    for (int j = 0; j < TN; ++j) z[j] = Zs[(tx + j * TX) * kLd + w];
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j) cnt[i][j] += __popc(TYPE == 1 ? (a[i] ^ z[j]) : (a[i] & z[j]));
  }
}

// The score combine of one output element and its store (and its mirror for
// a symmetric Gram), in the reference's operation order.
template <int TYPE>
__device__ __forceinline__ void store_element(const GramParams &p, int ga, int gz, double acc) {
  double o = (TYPE == 1) ? __dsub_rn(p.a0d1, __dmul_rn(2.0, acc)) : acc;
  if (p.lfA && p.lfZ) o = __dsub_rn(o, __dsub_rn(__dadd_rn(p.lfA[ga], p.lfZ[gz]), p.a2d1));
  p.out[(long long)p.out_r[ga] + (long long)p.out_c[gz] * p.out_stride] = o;
  if (p.symmetric) p.out[(long long)p.out_r2[gz] + (long long)p.out_c2[ga] * p.out_stride] = o;
}

template <int BM, int BN>
__device__ __forceinline__ void row_offsets(const GramParams &p, int tile_m, int tile_n, long long *a_off,
                                            long long *z_off, int tid, int nt) {
  for (int i = tid; i < BM; i += nt)
    a_off[i] = (tile_m + i < p.nA) ? (long long)p.a_rowb[tile_m + i] * p.a_row_bytes : -1;
  for (int i = tid; i < BN; i += nt)
    z_off[i] = (tile_n + i < p.nZ) ? (long long)p.z_rowb[tile_n + i] * p.z_row_bytes : -1;
}

template <int BM, int BN, int TM, int TN, int TYPE>
__global__ void __launch_bounds__((BM / TM) * (BN / TN), 2)
gram_popc_kernel(GramParams p) {
  constexpr int TX = BN / TN;
  constexpr int TY = BM / TM;
  constexpr int NT = TX * TY;
  extern __shared__ uint32_t smem[];
  uint32_t *As = smem;
  uint32_t *Zs = smem + BM * kLd;
  __shared__ long long a_off[BM];
  __shared__ long long z_off[BN];

  const int tile_n = blockIdx.x * BN;
  const int tile_m = blockIdx.y * BM;
  // Symmetric Gram: only pairs i <= k are computed (and mirrored).  A tile
  // whose smallest row index exceeds its largest column index has none.
  if (p.symmetric && tile_m > tile_n + BN - 1) return;

  const int tid = threadIdx.x;
  const int tx = tid % TX;
  const int ty = tid / TX;
  row_offsets<BM, BN>(p, tile_m, tile_n, a_off, z_off, tid, NT);

  double acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = 0.0;

  for (int blk = 0; blk < p.P; ++blk) {
    __syncthreads();
    stage_block<BM, BN, NT>(p, blk, As, Zs, a_off, z_off, tid);
    __syncthreads();
    int cnt[TM][TN];
    count_block<TM, TN, TX, TY, TYPE>(As, Zs, tx, ty, cnt);
    const double d = p.D ? p.D[blk] : 1.0;
#pragma unroll
    for (int i = 0; i < TM; ++i)
#pragma unroll
      for (int j = 0; j < TN; ++j)
        acc[i][j] = __dadd_rn(acc[i][j], __dmul_rn(d, (double)cnt[i][j]));
  }

#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int ga = tile_m + ty + i * TY;
    if (ga >= p.nA) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int gz = tile_n + tx + j * TX;
      if (gz >= p.nZ) continue;
      if (p.symmetric && ga > gz) continue;
      store_element<TYPE>(p, ga, gz, acc[i][j]);
    }
  }
}

// Split over blocks, for launches with few output tiles (a few hundred rows
// or fewer on a side), where one CTA per tile would walk all P blocks alone
// while most SMs idle.  Every (tile, block) pair is its own CTA and writes
// the tile's integer counts of that block (<= 1920, uint16) to a scratch
// array cnt[(b * nZ + k) * nA + i]; the fold kernel then adds each element's
// weighted counts over the blocks in ascending order, with the same multiply
// and add as above, so the outputs are the same bit for bit.
template <int BM, int BN, int TM, int TN, int TYPE>
__global__ void __launch_bounds__((BM / TM) * (BN / TN))
gram_split_counts_kernel(GramParams p, uint16_t *__restrict__ cnt_out) {
  constexpr int TX = BN / TN;
  constexpr int TY = BM / TM;
  constexpr int NT = TX * TY;
  extern __shared__ uint32_t smem[];
  uint32_t *As = smem;
  uint32_t *Zs = smem + BM * kLd;
  __shared__ long long a_off[BM];
  __shared__ long long z_off[BN];

  const int tile_n = blockIdx.x * BN;
  const int tile_m = blockIdx.y * BM;
  const int blk = blockIdx.z;
  if (p.symmetric && tile_m > tile_n + BN - 1) return;
  const int tid = threadIdx.x;
  const int tx = tid % TX;
  const int ty = tid / TX;
  row_offsets<BM, BN>(p, tile_m, tile_n, a_off, z_off, tid, NT);
  __syncthreads();
  stage_block<BM, BN, NT>(p, blk, As, Zs, a_off, z_off, tid);
  __syncthreads();
  int cnt[TM][TN];
  count_block<TM, TN, TX, TY, TYPE>(As, Zs, tx, ty, cnt);
  uint16_t *o = cnt_out + (size_t)blk * p.nZ * p.nA;
#pragma unroll
  for (int i = 0; i < TM; ++i) {
    const int ga = tile_m + ty + i * TY;
    if (ga >= p.nA) continue;
#pragma unroll
    for (int j = 0; j < TN; ++j) {
      const int gz = tile_n + tx + j * TX;
      if (gz < p.nZ) o[(size_t)gz * p.nA + ga] = (uint16_t)cnt[i][j];
    }
  }
}

template <int TYPE>
__global__ void __launch_bounds__(256) gram_split_fold_kernel(GramParams p, const uint16_t *__restrict__ cnt) {
  const long long n = (long long)p.nA * p.nZ, plane = n;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < n; e += (long long)gridDim.x * blockDim.x) {
    const int gz = (int)(e / p.nA), ga = (int)(e - (long long)gz * p.nA);
    if (p.symmetric && ga > gz) continue;
    double acc = 0.0;
    for (int b = 0; b < p.P; ++b) {
      const double d = p.D ? p.D[b] : 1.0;
      acc = __dadd_rn(acc, __dmul_rn(d, (double)cnt[(size_t)b * plane + e]));
    }
    store_element<TYPE>(p, ga, gz, acc);
  }
}

template <int BM, int BN, int TM, int TN, int TYPE>
void launch_tile(const GramParams &p) {
  constexpr int NT = (BM / TM) * (BN / TN);
  const size_t smem = (size_t)(BM + BN) * kLd * sizeof(uint32_t);
  static bool configured = false;
  if (!configured) {
    LAKGB_CUDA(cudaFuncSetAttribute(gram_popc_kernel<BM, BN, TM, TN, TYPE>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured = true;
  }
  dim3 grid((p.nZ + BN - 1) / BN, (p.nA + BM - 1) / BM);
  gram_popc_kernel<BM, BN, TM, TN, TYPE><<<grid, NT, smem, p.stream ? p.stream : stream()>>>(p);
  LAKGB_CUDA(cudaGetLastError());
  count_launch();
}

// Scratch bytes of the split launch; above kSplitMaxBytes it is not used.
constexpr size_t kSplitMaxBytes = size_t(256) << 20;
size_t split_bytes(const GramParams &p) { return (size_t)p.P * (size_t)p.nA * (size_t)p.nZ * sizeof(uint16_t); }

template <int TYPE>
void launch_split(const GramParams &p, cudaStream_t s) {
  constexpr int BM = 64, BN = 64, TM = 4, TN = 4, NT = (BM / TM) * (BN / TN);
  const size_t smem = (size_t)(BM + BN) * kLd * sizeof(uint32_t);
  static bool configured = false;
  if (!configured) {
    LAKGB_CUDA(cudaFuncSetAttribute(gram_split_counts_kernel<BM, BN, TM, TN, TYPE>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    configured = true;
  }
  uint16_t *cnt = nullptr;
  LAKGB_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&cnt), split_bytes(p), s));
  dim3 grid((p.nZ + BN - 1) / BN, (p.nA + BM - 1) / BM, p.P);
  gram_split_counts_kernel<BM, BN, TM, TN, TYPE><<<grid, NT, smem, s>>>(p, cnt);
  LAKGB_CUDA(cudaGetLastError());
  const long long n = (long long)p.nA * p.nZ;
  const int blocks = (int)std::min<long long>((n + 255) / 256, 152ll * 8);
  gram_split_fold_kernel<TYPE><<<blocks, 256, 0, s>>>(p, cnt);
  LAKGB_CUDA(cudaGetLastError());
  count_launch(2);
  LAKGB_CUDA(cudaFreeAsync(cnt, s));
}

}  // namespace

// ---------------------------------------------------------------------------
// Kernel choice.  Every candidate computes the same outputs bit for bit, so
// the choice is a matter of speed only.  With LAKGB_IMPL_AUTO (the default)
// a launch with at least kTensorRows rows on both sides takes the tensor-core
// kernel (it wins there by 3x or more); for smaller launches the first one of
// each shape class -- (type, symmetric, log2 of the A rows, of the Z rows and
// of the blocks) -- runs the candidates (tensor kernel, popcount kernel with
// two tile shapes, popcount kernel split over blocks) on its real arguments,
// timed with CUDA events on the launching stream, and the fastest serves that
// class from then on.

enum GramVariant { kTensor = 0, kPopc128x64, kPopc64x64, kSplit64x64, kPopc64x128, kNumVariants };
constexpr int kTunedVariants = 4;   // tensor, popcount 128x64, popcount 64x64, split over blocks
constexpr int kTensorRows = 512;
const char *const kVariantName[kNumVariants] = {"tensor_128x128", "popcount_128x64", "popcount_64x64",
                                                "split_64x64", "popcount_64x128"};

void launch_variant(int v, const GramParams &p, cudaStream_t s) {
  GramParams q = p;
  q.stream = s;
  if (v == kSplit64x64 && (split_bytes(q) > kSplitMaxBytes || q.P > 65535)) v = kPopc64x64;
  if (v == kTensor) {
    launch_gram_tc(q, s);
  } else if (v == kSplit64x64) {
    if (q.type == 1)
      launch_split<1>(q, s);
    else
      launch_split<2>(q, s);
  } else if (q.type == 1) {
    if (v == kPopc128x64) launch_tile<128, 64, 8, 4, 1>(q);
    else if (v == kPopc64x64) launch_tile<64, 64, 4, 4, 1>(q);
    else launch_tile<64, 128, 4, 8, 1>(q);
  } else {
    if (v == kPopc128x64) launch_tile<128, 64, 8, 4, 2>(q);
    else if (v == kPopc64x64) launch_tile<64, 64, 4, 4, 2>(q);
    else launch_tile<64, 128, 4, 8, 2>(q);
  }
}

inline int log2_bucket(long long n) {
  int b = 0;
  while ((1ll << b) < n) ++b;
  return b;
}

struct TuneKey {
  int type, sym, la, lz, lp;
  bool operator<(const TuneKey &o) const {
    return std::tie(type, sym, la, lz, lp) < std::tie(o.type, o.sym, o.la, o.lz, o.lp);
  }
};

struct TuneEntry {
  int choice;
  float ms[kNumVariants];
};

std::mutex g_tune_mu;
std::map<TuneKey, TuneEntry> g_tune;

int tuned_variant(const GramParams &p, cudaStream_t s, bool *ran) {
  if (p.nA >= kTensorRows && p.nZ >= kTensorRows) return kTensor;
  const TuneKey key{p.type, p.symmetric ? 1 : 0, log2_bucket(p.nA), log2_bucket(p.nZ), log2_bucket(p.P)};
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    auto it = g_tune.find(key);
    if (it != g_tune.end()) return it->second.choice;
  }
  // Under stream capture nothing can be timed: an untuned class takes the
  // tensor-core kernel (tune by running the launch once before capturing).
  if (capturing(s)) return kTensor;
  // Measure the candidates on this launch; each overwrites the same output
  // elements with the same values, so the call's result is unaffected.  One
  // untimed round first (first launches can carry one-time costs such as
  // module loading), then one timed round.
  TuneEntry e{};
  for (int v = 0; v < kNumVariants; ++v) e.ms[v] = -1.f;  // not measured
  for (int v = 0; v < kTunedVariants; ++v) launch_variant(v, p, s);
  constexpr int kRounds = 1;
  cudaEvent_t ev[kRounds][kTunedVariants + 1];
  for (auto &r : ev)
    for (auto &x : r) LAKGB_CUDA(cudaEventCreate(&x));
  for (int r = 0; r < kRounds; ++r) {
    LAKGB_CUDA(cudaEventRecord(ev[r][0], s));
    for (int v = 0; v < kTunedVariants; ++v) {
      launch_variant(v, p, s);
      LAKGB_CUDA(cudaEventRecord(ev[r][v + 1], s));
    }
  }
  LAKGB_CUDA(cudaEventSynchronize(ev[kRounds - 1][kTunedVariants]));
  int best = 0;
  for (int v = 0; v < kTunedVariants; ++v) {
    e.ms[v] = 1e30f;
    for (int r = 0; r < kRounds; ++r) {
      float ms = 0.f;
      LAKGB_CUDA(cudaEventElapsedTime(&ms, ev[r][v], ev[r][v + 1]));
      e.ms[v] = std::min(e.ms[v], ms);
    }
    if (e.ms[v] < e.ms[best]) best = v;
  }
  for (auto &r : ev)
    for (auto &x : r) LAKGB_CUDA(cudaEventDestroy(x));
  e.choice = best;
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune.emplace(key, e);
  }
  *ran = true;
  return best;
}

std::atomic<int> g_gram_impl{LAKGB_IMPL_AUTO};

void launch_gram(const GramParams &p) {
  if (p.nA <= 0 || p.nZ <= 0 || p.P <= 0) return;
  cudaStream_t s = p.stream ? p.stream : stream();
  gram_timer_begin(s);
  const int impl = g_gram_impl.load(std::memory_order_relaxed);
  if (impl == LAKGB_IMPL_TENSOR) {
    launch_variant(kTensor, p, s);
  } else if (impl == LAKGB_IMPL_SPLIT) {
    launch_variant(kSplit64x64, p, s);
  } else if (impl == LAKGB_IMPL_POPCOUNT) {
    launch_variant(kPopc128x64, p, s);
  } else {
    bool ran = false;
    const int v = tuned_variant(p, s, &ran);
    if (!ran) launch_variant(v, p, s);
  }
  gram_timer_end(s);
}

}  // namespace lakgb

extern "C" void lakgb_set_gram_impl(int impl) {
  lakgb::g_gram_impl.store((impl == LAKGB_IMPL_POPCOUNT || impl == LAKGB_IMPL_TENSOR || impl == LAKGB_IMPL_SPLIT)
                               ? impl
                               : LAKGB_IMPL_AUTO);
}

extern "C" int lakgb_gram_autotune_table(char *buf, int buf_len) {
  using namespace lakgb;
  std::string out = "[";
  {
    std::lock_guard<std::mutex> lk(g_tune_mu);
    bool first = true;
    for (const auto &kv : g_tune) {
      char line[512];
      int n = snprintf(line, sizeof line, "%s{\"type\":%d,\"symmetric\":%d,\"log2_rows_a\":%d,\"log2_rows_z\":%d,"
                       "\"log2_blocks\":%d,\"choice\":\"%s\",\"ms\":{",
                       first ? "" : ",", kv.first.type, kv.first.sym, kv.first.la, kv.first.lz, kv.first.lp,
                       kVariantName[kv.second.choice]);
      for (int v = 0; v < kNumVariants; ++v)
        n += snprintf(line + n, sizeof line - n, "%s\"%s\":%.4f", v ? "," : "", kVariantName[v], kv.second.ms[v]);
      snprintf(line + n, sizeof line - n, "}}");
      out += line;
      first = false;
    }
  }
  out += "]";
  if (buf && buf_len > 0) {
    strncpy(buf, out.c_str(), (size_t)buf_len - 1);
    buf[buf_len - 1] = 0;
  }
  return (int)out.size();
}

extern "C" void lakgb_gram_autotune_reset(void) {
  std::lock_guard<std::mutex> lk(lakgb::g_tune_mu);
  lakgb::g_tune.clear();
}

extern "C" int lakgb_gram_impl(void) { return lakgb::g_gram_impl.load(); }

extern "C" int lakgb_device_status(void) { return lakgb::tc_status_take(); }

extern "C" int lakgb_thread_device_status(void) { return lakgb::tc_status_take_stream(); }

extern "C" void lakgb_debug_tc_pipeline(unsigned long long wait_limit_ns, int withhold) {
  lakgb::tc_debug_set(wait_limit_ns ? wait_limit_ns : 2000000000ull, withhold);
}

namespace {

bool params_from_args(const lakgb_gram_args *a, lakgb::GramParams *p) {
  if (!a || (a->type_flag != LAKGB_TYPE_pm && a->type_flag != LAKGB_TYPE_00)) return false;
  *p = lakgb::GramParams{};
  p->wA = a->wA; p->a_rowb = a->a_rowb; p->nA = a->nA; p->a_row_bytes = a->a_row_bytes;
  p->wZ = a->wZ; p->z_rowb = a->z_rowb; p->nZ = a->nZ; p->z_row_bytes = a->z_row_bytes;
  p->mask = a->mask; p->P = a->P; p->D = a->D;
  p->type = (a->type_flag == LAKGB_TYPE_pm) ? 1 : 2;
  p->a0d1 = a->a0d1; p->a2d1 = a->a2d1; p->lfA = a->lfA; p->lfZ = a->lfZ;
  p->out_r = a->out_r; p->out_c = a->out_c; p->out_r2 = a->out_r2; p->out_c2 = a->out_c2;
  p->out_stride = a->out_stride; p->out = a->out; p->symmetric = a->symmetric;
  p->stream = (cudaStream_t)a->stream;
  return true;
}

}  // namespace

extern "C" int lakgb_gram_device(const lakgb_gram_args *a) {
  using namespace lakgb;
  GramParams p;
  if (!params_from_args(a, &p)) {
    set_error(3, "lakgb_gram_device: bad arguments");
    return -1;
  }
  launch_gram(p);
  return 0;
}

// Grouped Gram: the descriptors live on the device for the group's lifetime,
// so a run is two kernel launches and nothing else (capturable in a graph).
struct lakgb_gram_group {
  int n = 0, type = 1, total_tiles = 0;
  long long total_blocks = 0;
  lakgb::GramParams *d_ps = nullptr;
  int *d_tile0 = nullptr;
  long long *d_blk0 = nullptr;
  double *d_T = nullptr;
};

extern "C" lakgb_gram_group *lakgb_gram_group_create(const lakgb_gram_args *args, int n) {
  using namespace lakgb;
  if (!args || n <= 0) {
    set_error(3, "lakgb_gram_group_create: no instances");
    return nullptr;
  }
  std::vector<GramParams> ps((size_t)n);
  std::vector<int> tile0((size_t)n + 1, 0);
  std::vector<long long> blk0((size_t)n + 1, 0);
  for (int i = 0; i < n; ++i) {
    if (!params_from_args(&args[i], &ps[i]) || ps[i].type != ps[0].type) {
      set_error(3, "lakgb_gram_group_create: instance %d: bad arguments or a type unlike instance 0", i);
      return nullptr;
    }
    const GramParams &p = ps[i];
    const bool empty = p.nA <= 0 || p.nZ <= 0 || p.P <= 0;
    const int ntm = (p.nA + 127) / 128, ntn = (p.nZ + 127) / 128;
    if (!empty && p.symmetric && ntm != ntn) {
      set_error(3, "lakgb_gram_group_create: instance %d: symmetric with unequal tile rows and columns", i);
      return nullptr;
    }
    const long long tiles = empty ? 0 : gram_tc_tiles(p);
    if ((long long)tile0[i] + tiles > INT_MAX) {
      set_error(3, "lakgb_gram_group_create: too many tiles");
      return nullptr;
    }
    tile0[i + 1] = tile0[i] + (int)tiles;
    blk0[i + 1] = blk0[i] + (empty ? 0 : p.P);
  }
  if (blk0[n] > INT_MAX) {
    set_error(3, "lakgb_gram_group_create: too many blocks");
    return nullptr;
  }
  auto *g = new lakgb_gram_group;
  g->n = n;
  g->type = ps[0].type;
  g->total_tiles = tile0[n];
  g->total_blocks = blk0[n];
  LAKGB_CUDA(cudaMalloc(&g->d_ps, sizeof(GramParams) * n));
  LAKGB_CUDA(cudaMalloc(&g->d_tile0, sizeof(int) * (n + 1)));
  LAKGB_CUDA(cudaMalloc(&g->d_blk0, sizeof(long long) * (n + 1)));
  LAKGB_CUDA(cudaMalloc(&g->d_T, gram_tc_table_row_bytes() * (size_t)std::max(1ll, g->total_blocks)));
  // Copied on this thread's stream and waited for: a plain cudaMemcpy from
  // pageable memory may return before its DMA lands, and the launches that
  // read these arrays run on non-blocking streams that do not wait for it.
  cudaStream_t s = stream();
  LAKGB_CUDA(cudaMemcpyAsync(g->d_ps, ps.data(), sizeof(GramParams) * n, cudaMemcpyHostToDevice, s));
  LAKGB_CUDA(cudaMemcpyAsync(g->d_tile0, tile0.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s));
  LAKGB_CUDA(cudaMemcpyAsync(g->d_blk0, blk0.data(), sizeof(long long) * (n + 1), cudaMemcpyHostToDevice, s));
  LAKGB_CUDA(cudaStreamSynchronize(s));
  return g;
}

extern "C" int lakgb_gram_group_run(lakgb_gram_group *g, void *stream) {
  using namespace lakgb;
  if (!g) return -1;
  cudaStream_t s = stream ? (cudaStream_t)stream : lakgb::stream();
  gram_timer_begin(s);
  launch_gram_tc_group(GramGroupDev{g->d_ps, g->d_tile0, g->d_blk0, g->n}, g->type, g->total_tiles,
                       g->total_blocks, g->d_T, s);
  gram_timer_end(s);
  return 0;
}

extern "C" void lakgb_gram_group_destroy(lakgb_gram_group *g) {
  if (!g) return;
  cudaFree(g->d_ps);
  cudaFree(g->d_tile0);
  cudaFree(g->d_blk0);
  cudaFree(g->d_T);
  delete g;
}

namespace lakgb {

double gram_bitops(const GramParams &p, long long retained_cols) {
  return (double)p.nA * (double)p.nZ * (double)retained_cols;
}

}  // namespace lakgb
