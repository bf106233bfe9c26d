// Host sorts of the elimination loop (see bcc_sort.h).
#include "bcc_sort.h"

#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <vector>

namespace lakbcc {

// dQuickSort_xij, dir_c/Quicksort.c:83-141 (first-element pivot, recursion
// limit), written with an explicit stack.  The reference swaps the value and
// its six index arrays together at every step; here the values are sorted
// with one permutation array swapped alongside, and the index arrays are
// permuted by it once at the end -- the same comparisons and the same swaps,
// so the same order, equal values included.
static int partition_xij(double *d, int *perm, int l, int r) {
  const double pivot = d[l];
  int i = l, j = r + 1;
  while (true) {
    do { i++; } while (i <= r && d[i] <= pivot);
    do { j--; } while (d[j] > pivot);
    if (i >= j) break;
    std::swap(d[i], d[j]);
    std::swap(perm[i], perm[j]);
  }
  std::swap(d[l], d[j]);
  std::swap(perm[l], perm[j]);
  return j;
}

// The permutation that sorts d[l .. r] ascending, when those values are all
// distinct and none is NaN (false otherwise): an LSD radix sort, 11 bits a
// pass, of order-preserving integer keys (a non-negative value's bits with
// the sign bit set, a negative value's bits inverted).  Distinct values have
// one ascending order, so any correct sort of them gives the quicksort's.
bool sort_distinct(const double *d, int l, int r, int *pm) {
  const int n = r - l + 1;
  std::vector<uint64_t> key((size_t)n), key2((size_t)n);
  std::vector<int> idx((size_t)n), idx2((size_t)n);
  constexpr int kBits = 11, kPasses = 6, kBins = 1 << kBits;
  std::vector<unsigned> hist((size_t)kPasses * kBins, 0);
  for (int k = 0; k < n; ++k) {
    const double v = d[l + k];
    if (v != v) return false;
    uint64_t u;
    memcpy(&u, &v, 8);
    u = (u >> 63) ? ~u : (u | 0x8000000000000000ull);
    key[k] = u;
    idx[k] = l + k;
    for (int p = 0; p < kPasses; ++p) hist[(size_t)p * kBins + ((u >> (kBits * p)) & (kBins - 1))]++;
  }
  for (int p = 0; p < kPasses; ++p) {
    unsigned *h = &hist[(size_t)p * kBins];
    const uint64_t first = (key[0] >> (kBits * p)) & (kBins - 1);
    if (h[first] == (unsigned)n) continue;  // every key has this digit
    unsigned run = 0;
    for (int b = 0; b < kBins; ++b) { const unsigned c = h[b]; h[b] = run; run += c; }
    for (int k = 0; k < n; ++k) {
      const unsigned o = h[(key[k] >> (kBits * p)) & (kBins - 1)]++;
      key2[o] = key[k];
      idx2[o] = idx[k];
    }
    key.swap(key2);
    idx.swap(idx2);
  }
  for (int k = 1; k < n; ++k)
    if (d[idx[k - 1]] == d[idx[k]]) return false;  // a tie (+0 and -0 included)
  for (int k = 0; k < n; ++k) pm[l + k] = idx[k];
  return true;
}

void quicksort_xij(unsigned limit, double *d, int *i_, int *ib, int *ij, int *nb, int *ga, int *gb, int l, int r) {
  if (l >= r) return;
  std::vector<int> perm((size_t)r + 1);  // entries l .. r used
  int *pm = perm.data();
  // A subarray at depth nn holds at most n - nn values, so with n <= limit no
  // call reaches the recursion limit and the quicksort sorts d completely.
  if ((long)r - l + 1 <= (long)limit && sort_distinct(d, l, r, pm)) {
    std::vector<double> v((size_t)(r - l + 1));
    for (int k = l; k <= r; ++k) v[k - l] = d[pm[k]];
    for (int k = l; k <= r; ++k) d[k] = v[k - l];
  } else {
    for (int k = l; k <= r; ++k) perm[k] = k;
    struct Node { int l, r; unsigned nn; };
    std::vector<Node> st;
    st.push_back({l, r, 0});
    while (!st.empty()) {
      Node n = st.back();
      st.pop_back();
      if (n.l < n.r) {
        int j = partition_xij(d, pm, n.l, n.r);
        if (n.nn < limit) {
          st.push_back({j + 1, n.r, n.nn + 1});
          st.push_back({n.l, j - 1, n.nn + 1});
        }
      }
    }
  }
  std::vector<int> tmp((size_t)(r - l + 1));
  for (int *a : {i_, ib, ij, nb, ga, gb}) {
    if (!a) continue;
    for (int k = l; k <= r; ++k) tmp[k - l] = a[pm[k]];
    for (int k = l; k <= r; ++k) a[k] = tmp[k - l];
  }
}

// dQuickSort / dPartition, dir_c/Quicksort.c:43-81: ascending sort of the
// values d[stride*l] .. d[stride*r] with the first element as pivot (the
// order of equal values follows this partition), recursion depth limited as
// in the reference; an explicit stack instead of recursion.
void dquicksort_strided(unsigned limit, double *d, long stride, int l, int r) {
  struct Node { int l, r; unsigned nn; };
  std::vector<Node> st;
  st.push_back({l, r, 0});
  while (!st.empty()) {
    const Node n = st.back();
    st.pop_back();
    if (n.l >= n.r || n.nn >= limit) continue;
    const double pivot = d[stride * n.l];
    int i = n.l, j = n.r + 1;
    while (true) {
      do { i++; } while (i <= n.r && d[stride * i] <= pivot);
      do { j--; } while (d[stride * j] > pivot);
      if (i >= j) break;
      std::swap(d[stride * i], d[stride * j]);
    }
    std::swap(d[stride * n.l], d[stride * j]);
    st.push_back({j + 1, n.r, n.nn + 1});
    st.push_back({n.l, j - 1, n.nn + 1});
  }
}

}  // namespace lakbcc
