// Device mirrors of L_handles: FP64 score matrices that stay in HBM across
// kernel calls (no reference counterpart -- the reference has no device).
//
// A mirrored L_handle's values live on the device from the moment it is
// mirrored; the host array L->lf is refreshed only by lakgb_L_to_host.  The
// kernel entry points that read or write a mirrored handle (the Gram, xcalc,
// AnZt_S_WnYt) use the device copy directly, and the two host-side matrix
// operations the bcc driver applies to these matrices -- the low-rank
// subtraction (dir_c/bcc_lrup.c:863-892) and L2_transpose
// (dir_c/L_init.c:31-38) -- have device forms here.  Both are exact
// (one IEEE subtraction per element; a permutation), so results do not
// depend on where they run.
#include <mutex>
#include <unordered_map>

#include "abi_common.cuh"
#include "lmirror.cuh"

namespace lakgb {

namespace {

std::mutex g_mu;
std::unordered_map<const L_handle *, Mirror> g_mirrors;

__global__ void l_sub_kernel(double *dst, const double *src, unsigned long long n) {
  for (unsigned long long i = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; i < n;
       i += (unsigned long long)gridDim.x * blockDim.x)
    dst[i] = __dsub_rn(dst[i], src[i]);
}

// dst[c + r*dst_rs] = src[r + c*src_rs] for r < nr, c < nc: 32x32 tiles
// through shared memory so both sides are read / written in rows.
__global__ void l_transpose_kernel(double *dst, unsigned long long dst_rs, const double *src,
                                   unsigned long long src_rs, unsigned long long nr, unsigned long long nc) {
  __shared__ double tile[32][33];
  const unsigned long long r0 = blockIdx.x * 32ull, c0 = blockIdx.y * 32ull;
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const unsigned long long r = r0 + threadIdx.x, c = c0 + k;
    if (r < nr && c < nc) tile[k][threadIdx.x] = src[r + c * src_rs];
  }
  __syncthreads();
  for (int k = threadIdx.y; k < 32; k += blockDim.y) {
    const unsigned long long c = c0 + threadIdx.x, r = r0 + k;
    if (r < nr && c < nc) dst[c + r * dst_rs] = tile[threadIdx.x][k];
  }
}

}  // namespace

Mirror *find_mirror(const L_handle *L) {
  if (!L) return nullptr;
  std::lock_guard<std::mutex> lk(g_mu);
  auto it = g_mirrors.find(L);
  return it == g_mirrors.end() ? nullptr : &it->second;
}

}  // namespace lakgb

using namespace lakgb;

extern "C" void lakgb_L_mirror(L_handle *L) {
  LAKGB_PROFILE_CALL("lakgb_L_mirror");
  if (!L || find_mirror(L)) return;
  Mirror m{};
  m.n = L->length;
  LAKGB_CUDA(cudaMallocAsync((void **)&m.d, (m.n ? m.n : 1) * sizeof(double), stream()));
  if (m.n) LAKGB_CUDA(cudaMemcpyAsync(m.d, L->lf, m.n * sizeof(double), cudaMemcpyHostToDevice, stream()));
  LAKGB_CUDA(cudaStreamSynchronize(stream()));
  m.host_stale = false;
  std::lock_guard<std::mutex> lk(g_mu);
  g_mirrors[L] = m;
}

extern "C" void lakgb_L_mirror_zero(L_handle *L) {
  LAKGB_PROFILE_CALL("lakgb_L_mirror_zero");
  if (!L || find_mirror(L)) return;
  Mirror m{};
  m.n = L->length;
  LAKGB_CUDA(cudaMallocAsync((void **)&m.d, (m.n ? m.n : 1) * sizeof(double), stream()));
  if (m.n) LAKGB_CUDA(cudaMemsetAsync(m.d, 0, m.n * sizeof(double), stream()));
  LAKGB_CUDA(cudaStreamSynchronize(stream()));
  m.host_stale = false;
  std::lock_guard<std::mutex> lk(g_mu);
  g_mirrors[L] = m;
}

extern "C" void lakgb_L_to_host(L_handle *L) {
  LAKGB_PROFILE_CALL("lakgb_L_to_host");
  Mirror *m = find_mirror(L);
  if (!m || !m->host_stale) return;
  if (m->n) LAKGB_CUDA(cudaMemcpyAsync(L->lf, m->d, m->n * sizeof(double), cudaMemcpyDeviceToHost, stream()));
  LAKGB_CUDA(cudaStreamSynchronize(stream()));
  m->host_stale = false;
}

extern "C" void lakgb_L_release_mirror(L_handle *L) {
  LAKGB_PROFILE_CALL("lakgb_L_release_mirror");
  Mirror m{};
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_mirrors.find(L);
    if (it == g_mirrors.end()) return;
    m = it->second;
    g_mirrors.erase(it);
  }
  LAKGB_CUDA(cudaFreeAsync(m.d, stream()));
}

extern "C" void lakgb_L_sub(L_handle *dst, const L_handle *src) {
  LAKGB_PROFILE_CALL("lakgb_L_sub");
  Mirror *md = find_mirror(dst), *ms = find_mirror(src);
  const unsigned long long n = dst->length;
  if (md && ms && ms->n >= n) {
    if (n) {
      const unsigned long long blocks = std::min<unsigned long long>((n + 255) / 256, 4096);
      l_sub_kernel<<<(unsigned)blocks, 256, 0, stream()>>>(md->d, ms->d, n);
      LAKGB_CUDA(cudaGetLastError());
      count_launch();
    }
    md->host_stale = true;
    return;
  }
  lakgb_L_to_host(dst);
  lakgb_L_to_host(const_cast<L_handle *>(src));
  for (unsigned long long i = 0; i < n; ++i) dst->lf[i] -= src->lf[i];
  if (md) {
    LAKGB_CUDA(cudaMemcpyAsync(md->d, dst->lf, n * sizeof(double), cudaMemcpyHostToDevice, stream()));
    LAKGB_CUDA(cudaStreamSynchronize(stream()));
  }
}

extern "C" void lakgb_L_transpose(L_handle *dst, const L_handle *src) {
  LAKGB_PROFILE_CALL("lakgb_L_transpose");
  dst->spacing_row = src->spacing_col; dst->spacing_col = src->spacing_row; dst->spacing_lyr = src->spacing_lyr;
  dst->row_stride = src->col_stride; dst->col_stride = src->row_stride; dst->lyr_stride = src->lyr_stride;
  Mirror *md = find_mirror(dst), *ms = find_mirror(src);
  const unsigned long long nr = src->row_stride, nc = src->col_stride;
  if (md && ms && nr * nc <= md->n && nr * nc <= ms->n) {
    if (nr && nc) {
      dim3 grid((unsigned)((nr + 31) / 32), (unsigned)((nc + 31) / 32));
      l_transpose_kernel<<<grid, dim3(32, 8), 0, stream()>>>(md->d, dst->row_stride, ms->d, src->row_stride, nr, nc);
      LAKGB_CUDA(cudaGetLastError());
      count_launch();
    }
    md->host_stale = true;
    return;
  }
  lakgb_L_to_host(const_cast<L_handle *>(src));
  lakgb_L_to_host(dst);
  for (unsigned long long c = 0; c < nc; ++c)
    for (unsigned long long r = 0; r < nr; ++r) dst->lf[c + r * dst->row_stride] = src->lf[r + c * src->row_stride];
  if (md) {
    LAKGB_CUDA(cudaMemcpyAsync(md->d, dst->lf, md->n * sizeof(double), cudaMemcpyHostToDevice, stream()));
    LAKGB_CUDA(cudaStreamSynchronize(stream()));
  }
}
