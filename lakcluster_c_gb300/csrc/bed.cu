// PLINK .bed to .b16 conversion: the reference's bed_to_b16
// (dir_c/bed_to_b16.c:711-1355), the input pipeline's first step.
//
// A .bed file holds, after three magic bytes (108, 27, 1), one record per SNP
// (.bim line) of n_bam = ceil(n_fam / 4) bytes: patient p's genotype is the
// 2-bit code (byte[p / 4] >> 2 (p % 4)) & 3 -- 0 homozygous minor ("nor"),
// 1 missing, 2 heterozygous ("xor"), 3 homozygous major ("and").  The
// conversion
//   1. counts the four codes of every SNP over all 4 * n_bam code slots (the
//      reference counts the padding slots of the last byte too, as code 0)
//      and the missing codes of every patient over all SNPs;
//   2. on the host, in the reference's operation order: per-SNP code
//      frequencies, the fitted allele frequencies p = and + xor/2 and
//      q = nor + xor/2, the relative entropy I of the genotype counts against
//      Hardy-Weinberg proportions, and the mode among the three observed
//      codes; keeps the SNPs with all three codes present, min(p, q) >= the
//      maf threshold, missing fraction <= the SNP threshold and I <= the
//      entropy threshold, and the patients with missing fraction <= the
//      patient threshold; makes three alleles per kept SNP (nor, xor, and)
//      and orders them by frequency with the reference's quicksort (ties in
//      its order);
//   3. writes, for every kept SNP and kept patient, one bit in the row of
//      the allele matching the patient's code (a missing code counts as the
//      SNP's mode): alleles x patients, patients MSB first in bytes, rows of
//      rup(n_pat, 16) / 8 bytes in allele order -- the .b16 payload.
// Steps 1 and 3 run on the GPU (one pass over the .bed each, streamed in
// chunks of SNP records); the allele matrix is built in device memory.
// Outputs: the .b16 (header 16, patients, alleles), the kept patients' .fam
// lines and one .bim line per allele, as the reference writes them.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <string>
#include <vector>

#include "abi_common.cuh"
#include "lakgb_runtime.cuh"

namespace lakgb {

namespace {

constexpr long long kChunkBytes = 256ll << 20;  // device bytes of .bed records per chunk

// Pass 1a: the four code counts of each record over its 4 * n_bam slots.
// One warp per record, 32-bit words (records start 16-byte aligned).
__global__ void bed_snp_counts_kernel(const uint8_t *__restrict__ rows, long long pitch, int nrows, long long n_bam,
                                      unsigned *__restrict__ cnt) {
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
  const long long nwords = (n_bam + 3) / 4;
  for (long long r = warp; r < nrows; r += nwarps) {
    const uint32_t *w = reinterpret_cast<const uint32_t *>(rows + r * pitch);
    unsigned c1 = 0, c2 = 0, c3 = 0;
    for (long long i = lane; i < nwords; i += 32) {
      uint32_t x = w[i];
      const long long vb = n_bam - 4 * i;  // valid bytes in this word
      const uint32_t keep = vb >= 4 ? 0xFFFFFFFFu : ((1u << (8 * vb)) - 1u);
      x &= keep;
      const uint32_t lo = x & 0x55555555u & keep, hi = (x >> 1) & 0x55555555u & keep;
      c3 += __popc(lo & hi);
      c2 += __popc(hi & ~lo);
      c1 += __popc(lo & ~hi);
    }
    for (int o = 16; o; o >>= 1) {
      c1 += __shfl_xor_sync(0xFFFFFFFFu, c1, o);
      c2 += __shfl_xor_sync(0xFFFFFFFFu, c2, o);
      c3 += __shfl_xor_sync(0xFFFFFFFFu, c3, o);
    }
    if (lane == 0) {
      const unsigned tot = (unsigned)(4 * n_bam);
      cnt[r * 4 + 0] = tot - c1 - c2 - c3;
      cnt[r * 4 + 1] = c1;
      cnt[r * 4 + 2] = c2;
      cnt[r * 4 + 3] = c3;
    }
  }
}

// Pass 1b: missing codes of each patient slot over the chunk's records.  A
// thread owns one byte column (four slots) of a group of records and keeps
// four 8-bit counters in one word, spilled to 32-bit counters every 255
// records and added to the global counts at the end.
__global__ void bed_pat_missing_kernel(const uint8_t *__restrict__ rows, long long pitch, int nrows, long long n_bam,
                                       int rows_per_group, unsigned long long *__restrict__ miss) {
  const long long b = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= n_bam) return;
  const int r0 = blockIdx.y * rows_per_group, r1 = min(nrows, r0 + rows_per_group);
  unsigned m[4] = {0, 0, 0, 0};
  uint32_t acc = 0;
  int k = 0;
  for (int r = r0; r < r1; ++r) {
    const uint32_t v = rows[(long long)r * pitch + b];
    const uint32_t x = v & ~(v >> 1) & 0x55u;  // slot codes 01 (lo set, hi clear)
    acc += (x & 1u) | ((x & 4u) << 6) | ((x & 16u) << 12) | ((x & 64u) << 18);
    if (++k == 255) {
      for (int j = 0; j < 4; ++j) m[j] += (acc >> (8 * j)) & 0xFFu;
      acc = 0;
      k = 0;
    }
  }
  for (int j = 0; j < 4; ++j) m[j] += (acc >> (8 * j)) & 0xFFu;
  for (int j = 0; j < 4; ++j)
    if (m[j]) atomicAdd(&miss[4 * b + j], (unsigned long long)m[j]);
}

// Pass 2: the allele rows of the chunk's kept records.  rec[i] is the
// chunk-local record of the i-th kept record and dst[i] its three sorted
// allele rows (nor, xor, and) with its mode code in .w; a thread builds one
// byte (eight kept patients) of the three rows.
__global__ void bed_expand_kernel(const uint8_t *__restrict__ rows, long long pitch, const int *__restrict__ rec,
                                  const int4 *__restrict__ dst, int nkeep, const int *__restrict__ fam_of_pat,
                                  int n_pat, long long row_bytes, uint8_t *__restrict__ A_n) {
  const long long jb = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (jb >= row_bytes) return;
  for (int i = blockIdx.y; i < nkeep; i += gridDim.y) {
    const uint8_t *row = rows + (long long)rec[i] * pitch;
    const int4 d = dst[i];
    uint32_t bn = 0, bx = 0, ba = 0;
    for (int t = 0; t < 8; ++t) {
      const long long j = jb * 8 + t;
      if (j >= n_pat) break;
      const int p = fam_of_pat[j];
      uint32_t c = (row[p >> 2] >> (2 * (p & 3))) & 3u;
      if (c == 1u) c = (uint32_t)d.w;
      const uint32_t bit = 0x80u >> t;
      bn |= (c == 0u) ? bit : 0u;
      bx |= (c == 2u) ? bit : 0u;
      ba |= (c == 3u) ? bit : 0u;
    }
    A_n[(long long)d.x * row_bytes + jb] = (uint8_t)bn;
    A_n[(long long)d.y * row_bytes + jb] = (uint8_t)bx;
    A_n[(long long)d.z * row_bytes + jb] = (uint8_t)ba;
  }
}

// Records come from memory or from a .bed file.
struct BedRecords {
  const uint8_t *mem = nullptr;
  FILE *fp = nullptr;
  long long n_bam = 0;
  // rows [r0, r0 + n) into host memory (a pointer into mem, or buf)
  const uint8_t *fetch(long long r0, long long n, std::vector<uint8_t> &buf, std::string &err) const {
    if (mem) return mem + r0 * n_bam;
    buf.resize((size_t)(n * n_bam));
    if (fseeko(fp, (off_t)(3 + r0 * n_bam), SEEK_SET) != 0 ||
        fread(buf.data(), 1, buf.size(), fp) != buf.size()) {
      err = "short .bed file";
      return nullptr;
    }
    return buf.data();
  }
};

// dQuickSort_index (dir_c/Quicksort.c:216-248) and charpQuickSort_index
// (:364-414, strcmp order): first-element pivot, "<= pivot" from the left and
// "> pivot" from the right, the index array permuted alongside; subranges
// past the recursion limit stay unsorted.  Written with an explicit stack:
// the subranges are disjoint, so the order they are done in does not change
// the result.
template <typename K>
void quicksort_index(std::vector<K> &d, std::vector<int> &idx, unsigned limit) {
  struct Range { int l, r; unsigned depth; };
  std::vector<Range> st;
  if (!d.empty()) st.push_back({0, (int)d.size() - 1, 0});
  while (!st.empty()) {
    const Range g = st.back();
    st.pop_back();
    if (g.l >= g.r) continue;
    const K pivot = d[g.l];
    int i = g.l, j = g.r + 1;
    for (;;) {
      do { ++i; } while (i <= g.r && d[i] <= pivot);
      do { --j; } while (d[j] > pivot);
      if (i >= j) break;
      std::swap(d[i], d[j]);
      std::swap(idx[i], idx[j]);
    }
    std::swap(d[g.l], d[j]);
    std::swap(idx[g.l], idx[j]);
    if (g.depth < limit) {
      st.push_back({g.l, j - 1, g.depth + 1});
      st.push_back({j + 1, g.r, g.depth + 1});
    }
  }
}

int bed_convert(const BedRecords &src, int n_bim, int n_fam, const lakgb_bed_params &prm, lakgb_bed_result &R,
                std::string &err) {
  memset(&R, 0, sizeof(R));
  if (n_bim <= 0 || n_fam <= 0) { err = "no SNPs or no patients"; return 2; }
  const long long n_bam = (n_fam + 3) / 4;
  const long long pitch = (n_bam + 15) / 16 * 16;
  const long long chunk = std::max(1ll, std::min((long long)n_bim, kChunkBytes / pitch));
  DBuf d_rows((size_t)(chunk * pitch));
  LAKGB_CUDA(cudaMemsetAsync(d_rows.p, 0, d_rows.n, stream()));
  std::vector<uint8_t> hbuf;
  // pass 1
  DBuf d_cnt((size_t)chunk * 4 * sizeof(unsigned));
  DBuf d_miss((size_t)(4 * n_bam) * sizeof(unsigned long long));
  LAKGB_CUDA(cudaMemsetAsync(d_miss.p, 0, d_miss.n, stream()));
  std::vector<unsigned> cnt((size_t)n_bim * 4);
  const int gy_rows = 256;
  for (long long r0 = 0; r0 < n_bim; r0 += chunk) {
    const long long n = std::min(chunk, (long long)n_bim - r0);
    const uint8_t *h = src.fetch(r0, n, hbuf, err);
    if (!h) return 2;
    LAKGB_CUDA(cudaMemcpy2DAsync(d_rows.p, (size_t)pitch, h, (size_t)n_bam, (size_t)n_bam, (size_t)n,
                                 cudaMemcpyHostToDevice, stream()));
    const int blocks = (int)std::min<long long>((n * 32 + 255) / 256, 152 * 16);
    bed_snp_counts_kernel<<<blocks, 256, 0, stream()>>>(d_rows.as<uint8_t>(), pitch, (int)n, n_bam,
                                                        d_cnt.as<unsigned>());
    LAKGB_CUDA(cudaGetLastError());
    const long long groups = std::min<long long>(65535, (n + gy_rows - 1) / gy_rows);
    const int rows_per_group = (int)((n + groups - 1) / groups);
    dim3 g((unsigned)((n_bam + 255) / 256), (unsigned)groups);
    bed_pat_missing_kernel<<<g, 256, 0, stream()>>>(d_rows.as<uint8_t>(), pitch, (int)n, n_bam, rows_per_group,
                                                    d_miss.as<unsigned long long>());
    LAKGB_CUDA(cudaGetLastError());
    count_launch(2);
    LAKGB_CUDA(cudaMemcpyAsync(&cnt[(size_t)r0 * 4], d_cnt.p, (size_t)n * 4 * sizeof(unsigned),
                               cudaMemcpyDeviceToHost, stream()));
    LAKGB_CUDA(cudaStreamSynchronize(stream()));
  }
  std::vector<unsigned long long> miss((size_t)(4 * n_bam));
  LAKGB_CUDA(cudaMemcpyAsync(miss.data(), d_miss.p, d_miss.n, cudaMemcpyDeviceToHost, stream()));
  LAKGB_CUDA(cudaStreamSynchronize(stream()));
  // SNP statistics (bed_to_b16.c:880-930)
  const int t_nor = 0, t_mss = 1, t_xor = 2, t_and = 3;
  std::vector<double> frq_and(n_bim), frq_xor(n_bim), frq_nor(n_bim), frq_mss(n_bim), p_opt(n_bim), q_opt(n_bim),
      I_opt(n_bim);
  std::vector<unsigned long long> tot_dat(n_bim);
  std::vector<unsigned char> tag_mode(n_bim);
  for (int s = 0; s < n_bim; ++s) {
    const unsigned *c = &cnt[(size_t)s * 4];
    tot_dat[s] = (unsigned long long)c[t_and] + c[t_xor] + c[t_nor];
    const double tmp_min = (double)1 / (double)tot_dat[s];
    frq_mss[s] = (double)c[t_mss] / (double)n_fam;
    frq_and[s] = (double)c[t_and] / (double)tot_dat[s];
    frq_xor[s] = (double)c[t_xor] / (double)tot_dat[s];
    frq_nor[s] = (double)c[t_nor] / (double)tot_dat[s];
    p_opt[s] = frq_and[s] + 0.5 * frq_xor[s];
    q_opt[s] = frq_nor[s] + 0.5 * frq_xor[s];
    const double ta = frq_and[s] * log(frq_and[s] / std::max(tmp_min, pow(p_opt[s], 2)));
    const double tx = frq_xor[s] * log(frq_xor[s] / std::max(tmp_min, (2 * p_opt[s] * q_opt[s])));
    const double tn = frq_nor[s] * log(frq_nor[s] / std::max(tmp_min, pow(q_opt[s], 2)));
    I_opt[s] = ta + tx + tn;
    unsigned char m = t_xor;  // the mode among the observed codes, and > nor > xor on ties (:932-941)
    if (c[t_xor] >= c[t_and] && c[t_xor] >= c[t_nor]) m = t_xor;
    if (c[t_nor] >= c[t_and] && c[t_nor] >= c[t_xor]) m = t_nor;
    if (c[t_and] >= c[t_xor] && c[t_and] >= c[t_nor]) m = t_and;
    tag_mode[s] = m;
  }
  // kept SNPs and patients (:956-975)
  std::vector<int> snp_keep, pat_keep;
  for (int s = 0; s < n_bim; ++s)
    if (tot_dat[s] > 0 && frq_and[s] > 0 && frq_xor[s] > 0 && frq_nor[s] > 0 &&
        std::min(p_opt[s], q_opt[s]) >= prm.snp_maf_threshold && frq_mss[s] <= prm.snp_mss_threshold &&
        I_opt[s] <= prm.snp_I_opt_threshold)
      snp_keep.push_back(s);
  for (int f = 0; f < n_fam; ++f) {
    const unsigned long long tot = (unsigned long long)n_bim - miss[f];
    const double fm = (double)miss[f] / (double)n_bim;
    if (tot > 0 && fm <= prm.pat_mss_threshold) pat_keep.push_back(f);
  }
  // alleles and their order (:977-1003)
  const int n_snp = (int)snp_keep.size(), n_pat = (int)pat_keep.size(), n_allele = 3 * n_snp;
  std::vector<double> freq(n_allele), maf(n_allele), mss(n_allele), Iopt(n_allele);
  for (int k = 0; k < n_snp; ++k) {
    const int s = snp_keep[k];
    freq[3 * k + 0] = frq_nor[s]; freq[3 * k + 1] = frq_xor[s]; freq[3 * k + 2] = frq_and[s];
    for (int a = 0; a < 3; ++a) {
      maf[3 * k + a] = std::min(p_opt[s], q_opt[s]);
      mss[3 * k + a] = frq_mss[s];
      Iopt[3 * k + a] = I_opt[s];
    }
  }
  std::vector<double> work = freq;
  std::vector<int> orig_from_sort(n_allele), sort_from_orig(n_allele);
  for (int a = 0; a < n_allele; ++a) orig_from_sort[a] = a;
  quicksort_index(work, orig_from_sort, 1024u * 32u);
  for (int a = 0; a < n_allele; ++a) sort_from_orig[orig_from_sort[a]] = a;
  // pass 2: the allele matrix
  const long long row_bytes = (long long)((n_pat + 15) / 16 * 2);
  const size_t an_bytes = (size_t)(row_bytes * n_allele);
  DBuf d_An(an_bytes ? an_bytes : 1);
  LAKGB_CUDA(cudaMemsetAsync(d_An.p, 0, d_An.n, stream()));
  if (n_snp > 0 && n_pat > 0) {
    DBuf d_fam = upload_vec(pat_keep);
    std::vector<int> keep_idx(n_bim, -1);
    for (int k = 0; k < n_snp; ++k) keep_idx[snp_keep[k]] = k;
    for (long long r0 = 0; r0 < n_bim; r0 += chunk) {
      const long long n = std::min(chunk, (long long)n_bim - r0);
      std::vector<int> rec;
      std::vector<int4> dst;
      for (long long r = 0; r < n; ++r) {
        const int k = keep_idx[r0 + r];
        if (k < 0) continue;
        rec.push_back((int)r);
        dst.push_back(make_int4(sort_from_orig[3 * k], sort_from_orig[3 * k + 1], sort_from_orig[3 * k + 2],
                                tag_mode[r0 + r]));
      }
      if (rec.empty()) continue;
      const uint8_t *h = src.fetch(r0, n, hbuf, err);
      if (!h) return 2;
      LAKGB_CUDA(cudaMemcpy2DAsync(d_rows.p, (size_t)pitch, h, (size_t)n_bam, (size_t)n_bam, (size_t)n,
                                   cudaMemcpyHostToDevice, stream()));
      DBuf d_rec = upload_vec(rec), d_dst = upload_vec(dst);
      dim3 g((unsigned)((row_bytes + 255) / 256), (unsigned)std::min<size_t>(rec.size(), 65535));
      bed_expand_kernel<<<g, 256, 0, stream()>>>(d_rows.as<uint8_t>(), pitch, d_rec.as<int>(), d_dst.as<int4>(),
                                                 (int)rec.size(), d_fam.as<int>(), n_pat, row_bytes,
                                                 d_An.as<uint8_t>());
      LAKGB_CUDA(cudaGetLastError());
      count_launch();
      LAKGB_CUDA(cudaStreamSynchronize(stream()));
    }
  }
  // results
  R.n_snp = n_bim; R.n_fam = n_fam;
  R.n_snp_retain = n_snp; R.n_pat_retain = n_pat; R.n_allele = n_allele; R.row_bytes = row_bytes;
  auto copy_i = [](const std::vector<int> &v) {
    int *p = (int *)malloc(sizeof(int) * (v.empty() ? 1 : v.size()));
    if (p && !v.empty()) memcpy(p, v.data(), sizeof(int) * v.size());
    return p;
  };
  auto copy_d = [](const std::vector<double> &v) {
    double *p = (double *)malloc(sizeof(double) * (v.empty() ? 1 : v.size()));
    if (p && !v.empty()) memcpy(p, v.data(), sizeof(double) * v.size());
    return p;
  };
  R.snp_from_retain = copy_i(snp_keep);
  R.pat_from_retain = copy_i(pat_keep);
  R.allele_orig_from_sort = copy_i(orig_from_sort);
  R.allele_frequency = copy_d(freq);
  R.allele_maf = copy_d(maf);
  R.allele_mss = copy_d(mss);
  R.allele_I_opt = copy_d(Iopt);
  R.A_n = (unsigned char *)malloc(an_bytes ? an_bytes : 1);
  if (!R.snp_from_retain || !R.pat_from_retain || !R.allele_orig_from_sort || !R.allele_frequency ||
      !R.allele_maf || !R.allele_mss || !R.allele_I_opt || !R.A_n) {
    lakgb_bed_result_free(&R);
    err = "out of host memory";
    return 2;
  }
  if (an_bytes) LAKGB_CUDA(cudaMemcpyAsync(R.A_n, d_An.p, an_bytes, cudaMemcpyDeviceToHost, stream()));
  LAKGB_CUDA(cudaStreamSynchronize(stream()));
  return 0;
}

// wc_0 (bed_to_b16.c:14-28): lines as getline counts them.
long long count_lines(const char *path) {
  FILE *fp = fopen(path, "rb");
  if (!fp) return -1;
  long long n = 0;
  int c, last = '\n';
  while ((c = fgetc(fp)) != EOF) {
    if (c == '\n') ++n;
    last = c;
  }
  if (last != '\n') ++n;
  fclose(fp);
  return n;
}

// The whitespace-separated fields of a text file, as fscanf("%s") reads them.
int read_fields(const char *path, std::vector<std::string> &out) {
  FILE *fp = fopen(path, "rb");
  if (!fp) return 2;
  std::string cur;
  int c;
  while ((c = fgetc(fp)) != EOF) {
    if (c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f') {
      if (!cur.empty()) { out.push_back(cur); cur.clear(); }
    } else {
      cur.push_back((char)c);
    }
  }
  if (!cur.empty()) out.push_back(cur);
  fclose(fp);
  return 0;
}

// The lines of a text file as getline reads them, without their newlines.
int read_lines(const char *path, std::vector<std::string> &out) {
  FILE *fp = fopen(path, "rb");
  if (!fp) return 2;
  std::string cur;
  int c;
  bool any = false;
  while ((c = fgetc(fp)) != EOF) {
    any = true;
    if (c == '\n') { out.push_back(cur); cur.clear(); any = false; }
    else cur.push_back((char)c);
  }
  if (any) out.push_back(cur);
  fclose(fp);
  return 0;
}

// b16_merge's bit gather: output row r (one allele) holds, at bit k, the bit
// of common patient k in the source row (idx: per study, the patient's
// position in that study).  One thread per output byte, grid-stride; bytes
// past the last patient stay zero.
__global__ void b16_gather_kernel(const uint8_t *__restrict__ in, const long long *__restrict__ row_off,
                                  const int *__restrict__ row_study, const int *__restrict__ idx, int n_int,
                                  long long out_bytes, long long n_rows, uint8_t *__restrict__ out) {
  const long long total = n_rows * out_bytes;
  for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
       t += (long long)gridDim.x * blockDim.x) {
    const long long r = t / out_bytes, j = t - r * out_bytes;
    const uint8_t *row = in + row_off[r];
    const int *ix = idx + (long long)row_study[r] * n_int;
    unsigned v = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
      const long long k = 8 * j + q;
      if (k < n_int) {
        const int p = ix[k];
        v |= (unsigned)((row[p >> 3] >> (7 - (p & 7))) & 1) << (7 - q);
      }
    }
    out[t] = (uint8_t)v;
  }
}

// b16_merge (dir_c/bed_to_b16.c:1659-1985):
//   1. per study: the .fam keys FID + IID (the first two fields of each line,
//      concatenated), sorted with the reference's string quicksort;
//   2. the intersection (charpIntersectall_index_index_driver,
//      dir_c/Quicksort.c:624-690): step the sorted lists together, advance
//      the list holding the smallest key, and when all current keys are
//      equal take them as the next common patient -- sorted key order, each
//      study's patient at that key;
//   3. the .fam lines of the common patients from the first study;
//   4. the alleles of every study interleaved by the allele frequency of
//      their .bim lines (field 9): repeatedly the study whose next allele has
//      the smallest frequency, ties to the lower study; its .bim line (11
//      fields, tab-joined) and its row with the common patients' bits (the
//      GPU gather above);
//   5. the .b16: header 16, common patients, alleles of all studies; rows of
//      rup(patients, 16) / 8 bytes.
int b16_merge_files(int n_file, const char *const *b16_in, const char *const *bim_in, const char *const *fam_in,
                    const char *b16_out, const char *bim_out, const char *fam_out, std::string &err) {
  if (n_file < 1) { err = "no studies"; return 2; }
  std::vector<long long> n_bim(n_file), n_fam(n_file), l_fam(n_file), base(n_file + 1, 0);
  std::vector<std::vector<std::string>> keys(n_file), bim_tok(n_file);
  std::vector<std::string> fam0;
  std::vector<uint8_t> all;
  for (int f = 0; f < n_file; ++f) {
    n_bim[f] = count_lines(bim_in[f]);
    n_fam[f] = count_lines(fam_in[f]);
    if (n_bim[f] < 0) { err = std::string("cannot open ") + bim_in[f]; return 2; }
    if (n_fam[f] < 0) { err = std::string("cannot open ") + fam_in[f]; return 2; }
    FILE *fp = fopen(b16_in[f], "rb");
    if (!fp) { err = std::string("cannot open ") + b16_in[f]; return 2; }
    int hdr[3] = {0, 0, 0};
    if (fread(hdr, sizeof(int), 3, fp) != 3) { fclose(fp); err = std::string("short .b16 file ") + b16_in[f]; return 2; }
    if (hdr[2] != n_bim[f]) printf(" %% Warning, n_bim_[%d] %lld vs %d\n", f, n_bim[f], hdr[2]);
    if (hdr[1] != n_fam[f]) printf(" %% Warning, n_fam_[%d] %lld vs %d\n", f, n_fam[f], hdr[1]);
    l_fam[f] = (n_fam[f] + (16 - n_fam[f] % 16) % 16) / 8;
    base[f + 1] = base[f] + n_bim[f] * l_fam[f];
    all.resize((size_t)base[f + 1]);
    const size_t want = (size_t)(n_bim[f] * l_fam[f]);
    const bool short_rows = want && fread(all.data() + base[f], 1, want, fp) != want;
    fclose(fp);
    if (short_rows) { err = std::string("short .b16 file ") + b16_in[f]; return 2; }
    std::vector<std::string> lines;
    if (read_lines(fam_in[f], lines)) { err = std::string("cannot open ") + fam_in[f]; return 2; }
    for (long long i = 0; i < n_fam[f]; ++i) {
      char a[4096], b[4096];
      if ((size_t)i >= lines.size() || lines[i].size() >= sizeof(a) || sscanf(lines[i].c_str(), "%s %s", a, b) != 2) {
        err = std::string("bad .fam line in ") + fam_in[f];
        return 2;
      }
      keys[f].push_back(std::string(a) + b);
    }
    if (read_fields(bim_in[f], bim_tok[f]) || (long long)bim_tok[f].size() < 11 * n_bim[f]) {
      err = std::string("bad .bim file ") + bim_in[f];
      return 2;
    }
  }
  if (read_fields(fam_in[0], fam0) || (long long)fam0.size() < 6 * n_fam[0]) { err = "bad .fam file"; return 2; }
  // 1-2: sorted keys and their intersection
  std::vector<std::vector<int>> order(n_file);
  for (int f = 0; f < n_file; ++f) {
    order[f].resize(keys[f].size());
    for (size_t i = 0; i < order[f].size(); ++i) order[f][i] = (int)i;
    quicksort_index(keys[f], order[f], 1024u * 32u);
  }
  std::vector<size_t> pos(n_file, 0);
  std::vector<int> common;  // n_int x n_file: each study's patient
  long long n_int = 0;
  auto all_left = [&] {
    for (int f = 0; f < n_file; ++f) if (pos[f] >= keys[f].size()) return false;
    return true;
  };
  while (all_left()) {
    int fmin = 0;
    bool found = false;
    for (int f = 0; f < n_file; ++f) {
      const int c = keys[fmin][pos[fmin]].compare(keys[f][pos[f]]);
      if (c > 0) { found = true; fmin = f; }
      if (c < 0) found = true;
    }
    if (found) {
      ++pos[fmin];
      continue;
    }
    for (int f = 0; f < n_file; ++f) common.push_back(order[f][pos[f]++]);
    ++n_int;
  }
  // 3: .fam of the common patients (first study's lines)
  FILE *fo = fopen(fam_out, "wb");
  if (!fo) { err = std::string("cannot write ") + fam_out; return 2; }
  for (long long k = 0; k < n_int; ++k) {
    const size_t p = (size_t)common[(size_t)k * n_file] * 6;
    fprintf(fo, "%s %s %s %s %s %s\n", fam0[p].c_str(), fam0[p + 1].c_str(), fam0[p + 2].c_str(), fam0[p + 3].c_str(),
            fam0[p + 4].c_str(), fam0[p + 5].c_str());
  }
  fclose(fo);
  // 4: alleles interleaved by frequency
  long long n_rows = 0;
  for (int f = 0; f < n_file; ++f) n_rows += n_bim[f];
  std::vector<long long> row_off;
  std::vector<int> row_study;
  row_off.reserve((size_t)n_rows);
  row_study.reserve((size_t)n_rows);
  FILE *bo = fopen(bim_out, "wb");
  if (!bo) { err = std::string("cannot write ") + bim_out; return 2; }
  std::vector<long long> nb(n_file, 0);
  for (;;) {
    int fmin = -1;
    double fr_min = 0.0;
    for (int f = 0; f < n_file; ++f) {
      if (nb[f] >= n_bim[f]) continue;
      const double fr = atof(bim_tok[f][(size_t)(11 * nb[f] + 8)].c_str());
      if (fmin < 0 || fr < fr_min) { fmin = f; fr_min = fr; }
    }
    if (fmin < 0) break;
    const std::string *t = &bim_tok[fmin][(size_t)(11 * nb[fmin])];
    for (int q = 0; q < 11; ++q) fprintf(bo, q < 10 ? "%s\t" : "%s\n", t[q].c_str());
    row_off.push_back(base[fmin] + nb[fmin] * l_fam[fmin]);
    row_study.push_back(fmin);
    ++nb[fmin];
  }
  fclose(bo);
  // 5: the merged rows, gathered on the device
  const long long l_int = (n_int + (16 - n_int % 16) % 16) / 8;
  std::vector<uint8_t> out((size_t)(n_rows * l_int), 0);
  if (n_rows > 0 && l_int > 0) {
    std::vector<int> idx((size_t)(n_int * n_file));
    for (long long k = 0; k < n_int; ++k)
      for (int f = 0; f < n_file; ++f) idx[(size_t)(f * n_int + k)] = common[(size_t)(k * n_file + f)];
    DBuf d_in = upload_bytes(all.data(), all.size());
    DBuf d_off = upload_vec(row_off), d_study = upload_vec(row_study), d_idx = upload_vec(idx);
    DBuf d_out(out.size());
    const long long total = n_rows * l_int;
    const int blocks = (int)std::min<long long>((total + 255) / 256, 152 * 32);
    b16_gather_kernel<<<blocks, 256, 0, stream()>>>(d_in.as<uint8_t>(), d_off.as<long long>(), d_study.as<int>(),
                                                    d_idx.as<int>(), (int)n_int, l_int, n_rows, d_out.as<uint8_t>());
    LAKGB_CUDA(cudaGetLastError());
    count_launch();
    LAKGB_CUDA(cudaMemcpyAsync(out.data(), d_out.p, out.size(), cudaMemcpyDeviceToHost, stream()));
    LAKGB_CUDA(cudaStreamSynchronize(stream()));
  }
  FILE *b16 = fopen(b16_out, "wb");
  if (!b16) { err = std::string("cannot write ") + b16_out; return 2; }
  const int hdr[3] = {16, (int)n_int, (int)n_rows};
  fwrite(hdr, sizeof(int), 3, b16);
  const bool ok = out.empty() || fwrite(out.data(), 1, out.size(), b16) == out.size();
  const bool closed = fclose(b16) == 0;
  if (!ok || !closed) { err = std::string("cannot write ") + b16_out; return 2; }
  return 0;
}

thread_local std::string t_bed_err;

}  // namespace
}  // namespace lakgb

using namespace lakgb;

extern "C" void lakgb_bed_params_init(struct lakgb_bed_params *p) {
  if (!p) return;
  // the reference's defaults (dir_c/lakcluster_ver18.c:158-161)
  p->snp_mss_threshold = 0.01;
  p->snp_maf_threshold = 0.25;
  p->snp_I_opt_threshold = 0.01;
  p->pat_mss_threshold = 0.04;
}

extern "C" void lakgb_bed_result_free(struct lakgb_bed_result *r) {
  if (!r) return;
  free(r->snp_from_retain); free(r->pat_from_retain); free(r->allele_orig_from_sort);
  free(r->allele_frequency); free(r->allele_maf); free(r->allele_mss); free(r->allele_I_opt); free(r->A_n);
  memset(r, 0, sizeof(*r));
}

extern "C" int lakgb_bed_to_b16_mem(const unsigned char *bed_records, int n_snp, int n_fam,
                                    const struct lakgb_bed_params *params, struct lakgb_bed_result *out) {
  LAKGB_PROFILE_CALL("lakgb_bed_to_b16_mem");
  t_bed_err.clear();
  if (!bed_records || !out) { t_bed_err = "null argument"; set_error(2, "lakgb_bed_to_b16_mem: null argument"); return 2; }
  lakgb_bed_params prm;
  lakgb_bed_params_init(&prm);
  if (params) prm = *params;
  BedRecords src;
  src.mem = bed_records;
  src.n_bam = (n_fam + 3) / 4;
  const int rc = bed_convert(src, n_snp, n_fam, prm, *out, t_bed_err);
  if (rc) set_error(rc, "lakgb_bed_to_b16_mem: %s", t_bed_err.c_str());
  return rc;
}

extern "C" int lakgb_bed_to_b16(const char *bed, const char *bim, const char *fam, const char *b16_out,
                                const char *bim_out, const char *fam_out, const struct lakgb_bed_params *params) {
  LAKGB_PROFILE_CALL("lakgb_bed_to_b16");
  t_bed_err.clear();
  auto fail = [](const std::string &m) {
    t_bed_err = m;
    set_error(2, "lakgb_bed_to_b16: %s", m.c_str());
    return 2;
  };
  if (!bed || !bim || !fam || !b16_out || !bim_out || !fam_out) return fail("null file name");
  lakgb_bed_params prm;
  lakgb_bed_params_init(&prm);
  if (params) prm = *params;
  const long long n_bim = count_lines(bim), n_fam = count_lines(fam);
  if (n_bim < 0) return fail(std::string("cannot open ") + bim);
  if (n_fam < 0) return fail(std::string("cannot open ") + fam);
  FILE *fp = fopen(bed, "rb");
  if (!fp) return fail(std::string("cannot open ") + bed);
  unsigned char key[3] = {0, 0, 0};
  if (fread(key, 1, 3, fp) != 3) { fclose(fp); return fail("short .bed file"); }
  if (key[0] != 108 || key[1] != 27 || key[2] != 1)
    printf(" %% Warning, .bed magic %d %d %d != 108 27 1\n", key[0], key[1], key[2]);  // the reference goes on too
  BedRecords src;
  src.fp = fp;
  src.n_bam = (n_fam + 3) / 4;
  fseeko(fp, 0, SEEK_END);
  const long long size = (long long)ftello(fp);
  if (size < 3 + n_bim * src.n_bam) { fclose(fp); return fail("the .bed file is shorter than its .bim and .fam say"); }
  lakgb_bed_result R;
  const int rc = bed_convert(src, (int)n_bim, (int)n_fam, prm, R, t_bed_err);
  fclose(fp);
  if (rc) return fail(t_bed_err);
  // .fam of the kept patients (:1204-1239): six fields each, joined by spaces
  std::vector<std::string> ff, bf;
  if (read_fields(fam, ff) || (long long)ff.size() < 6 * n_fam) { lakgb_bed_result_free(&R); return fail("bad .fam file"); }
  if (read_fields(bim, bf) || (long long)bf.size() < 6 * n_bim) { lakgb_bed_result_free(&R); return fail("bad .bim file"); }
  FILE *fo = fopen(fam_out, "wb");
  if (!fo) { lakgb_bed_result_free(&R); return fail(std::string("cannot write ") + fam_out); }
  for (int k = 0; k < R.n_pat_retain; ++k) {
    const size_t f = (size_t)R.pat_from_retain[k] * 6;
    fprintf(fo, "%s %s %s %s %s %s\n", ff[f].c_str(), ff[f + 1].c_str(), ff[f + 2].c_str(), ff[f + 3].c_str(),
            ff[f + 4].c_str(), ff[f + 5].c_str());
  }
  fclose(fo);
  // .bim, one line per allele in sorted order (:1257-1300).  The reference
  // picks the type label by testing the allele tags 0, 1, 2 as booleans, so
  // the last test wins and every line says "and(orig)"; kept as written.
  FILE *bo = fopen(bim_out, "wb");
  if (!bo) { lakgb_bed_result_free(&R); return fail(std::string("cannot write ") + bim_out); }
  for (int a = 0; a < R.n_allele; ++a) {
    const int orig = R.allele_orig_from_sort[a];
    const size_t f = (size_t)R.snp_from_retain[orig / 3] * 6;
    fprintf(bo, "%s\t%s\t%s\t%s\t%s\t%s\t%s\t%f\t%f\t%f\t%f\n", bf[f].c_str(), bf[f + 1].c_str(), bf[f + 2].c_str(),
            bf[f + 3].c_str(), bf[f + 4].c_str(), bf[f + 5].c_str(), "and(orig)", R.allele_I_opt[orig],
            R.allele_frequency[orig], R.allele_mss[orig], R.allele_maf[orig]);
  }
  fclose(bo);
  // .b16: bitj, patients, alleles, then the rows (:1301-1309)
  FILE *b16 = fopen(b16_out, "wb");
  if (!b16) { lakgb_bed_result_free(&R); return fail(std::string("cannot write ") + b16_out); }
  const int hdr[3] = {16, R.n_pat_retain, R.n_allele};
  fwrite(hdr, sizeof(int), 3, b16);
  const size_t n = (size_t)R.row_bytes * (size_t)R.n_allele;
  const bool ok = n == 0 || fwrite(R.A_n, 1, n, b16) == n;
  const bool closed = fclose(b16) == 0;
  lakgb_bed_result_free(&R);
  if (!ok || !closed) return fail(std::string("cannot write ") + b16_out);
  return 0;
}

extern "C" int lakgb_bed_last_error(char *msg, int msg_len) {
  if (msg && msg_len > 0) {
    strncpy(msg, t_bed_err.c_str(), (size_t)msg_len - 1);
    msg[msg_len - 1] = 0;
  }
  return t_bed_err.empty() ? 0 : 1;
}

extern "C" int lakgb_b16_merge(int n_file, const char *const *b16_in, const char *const *bim_in,
                               const char *const *fam_in, const char *b16_out, const char *bim_out,
                               const char *fam_out) {
  LAKGB_PROFILE_CALL("lakgb_b16_merge");
  t_bed_err.clear();
  bool null_name = !b16_in || !bim_in || !fam_in || !b16_out || !bim_out || !fam_out;
  for (int f = 0; !null_name && f < n_file; ++f) null_name = !b16_in[f] || !bim_in[f] || !fam_in[f];
  const int rc = null_name ? 2 : b16_merge_files(n_file, b16_in, bim_in, fam_in, b16_out, bim_out, fam_out, t_bed_err);
  if (null_name) t_bed_err = "null file name";
  if (rc) set_error(rc, "lakgb_b16_merge: %s", t_bed_err.c_str());
  return rc;
}
