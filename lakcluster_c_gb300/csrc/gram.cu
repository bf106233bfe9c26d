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
#include <string.h>

#include <algorithm>
#include <atomic>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "gram.cuh"
#include "lakgb_runtime.cuh"

namespace lakgb {

namespace {

constexpr int kLd = kBlockWords + 1;  // smem row pitch in words

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

  for (int i = tid; i < BM; i += NT)
    a_off[i] = (tile_m + i < p.nA) ? (long long)p.a_rowb[tile_m + i] * p.a_row_bytes : -1;
  for (int i = tid; i < BN; i += NT)
    z_off[i] = (tile_n + i < p.nZ) ? (long long)p.z_rowb[tile_n + i] * p.z_row_bytes : -1;

  double acc[TM][TN];
#pragma unroll
  for (int i = 0; i < TM; ++i)
#pragma unroll
    for (int j = 0; j < TN; ++j) acc[i][j] = 0.0;

  for (int blk = 0; blk < p.P; ++blk) {
    __syncthreads();
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
    __syncthreads();

    int cnt[TM][TN];
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
        for (int j = 0; j < TN; ++j)
          cnt[i][j] += __popc(TYPE == 1 ? (a[i] ^ z[j]) : (a[i] & z[j]));
    }
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
      double o = (TYPE == 1) ? __dsub_rn(p.a0d1, __dmul_rn(2.0, acc[i][j])) : acc[i][j];
      if (p.lfA && p.lfZ) o = __dsub_rn(o, __dsub_rn(__dadd_rn(p.lfA[ga], p.lfZ[gz]), p.a2d1));
      p.out[(long long)p.out_r[ga] + (long long)p.out_c[gz] * p.out_stride] = o;
      if (p.symmetric)
        p.out[(long long)p.out_r2[gz] + (long long)p.out_c2[ga] * p.out_stride] = o;
    }
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

}  // namespace

// ---------------------------------------------------------------------------
// Kernel choice.  Every candidate computes the same outputs bit for bit, so
// the choice is a matter of speed only.  With LAKGB_IMPL_AUTO (the default)
// a launch with at least kTensorRows rows on both sides takes the tensor-core
// kernel (it wins there by 3x or more); for smaller launches the first one of
// each shape class -- (type, symmetric, log2 of the A rows, of the Z rows and
// of the blocks) -- runs the candidates on its real arguments, timed with CUDA
// events on the launching stream, and the fastest serves that class from
// then on.

enum GramVariant { kTensor = 0, kPopc128x64, kPopc64x64, kPopc64x128, kNumVariants };
constexpr int kTunedVariants = 3;   // tensor, popcount 128x64, popcount 64x64
constexpr int kTensorRows = 512;
const char *const kVariantName[kNumVariants] = {"tensor_128x128", "popcount_128x64", "popcount_64x64",
                                                "popcount_64x128"};

void launch_variant(int v, const GramParams &p, cudaStream_t s) {
  GramParams q = p;
  q.stream = s;
  if (v == kTensor) {
    launch_gram_tc(q, s);
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
  lakgb::g_gram_impl.store(impl == LAKGB_IMPL_POPCOUNT ? LAKGB_IMPL_POPCOUNT
                                                       : (impl == LAKGB_IMPL_TENSOR ? LAKGB_IMPL_TENSOR
                                                                                    : LAKGB_IMPL_AUTO));
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

extern "C" int lakgb_gram_device(const lakgb_gram_args *a) {
  using namespace lakgb;
  if (!a || (a->type_flag != LAKGB_TYPE_pm && a->type_flag != LAKGB_TYPE_00)) {
    set_error(3, "lakgb_gram_device: bad arguments");
    return -1;
  }
  GramParams p{};
  p.wA = a->wA; p.a_rowb = a->a_rowb; p.nA = a->nA; p.a_row_bytes = a->a_row_bytes;
  p.wZ = a->wZ; p.z_rowb = a->z_rowb; p.nZ = a->nZ; p.z_row_bytes = a->z_row_bytes;
  p.mask = a->mask; p.P = a->P; p.D = a->D;
  p.type = (a->type_flag == LAKGB_TYPE_pm) ? 1 : 2;
  p.a0d1 = a->a0d1; p.a2d1 = a->a2d1; p.lfA = a->lfA; p.lfZ = a->lfZ;
  p.out_r = a->out_r; p.out_c = a->out_c; p.out_r2 = a->out_r2; p.out_c2 = a->out_c2;
  p.out_stride = a->out_stride; p.out = a->out; p.symmetric = a->symmetric;
  p.stream = (cudaStream_t)a->stream;
  launch_gram(p);
  return 0;
}

namespace lakgb {

double gram_bitops(const GramParams &p, long long retained_cols) {
  return (double)p.nA * (double)p.nZ * (double)retained_cols;
}

}  // namespace lakgb
