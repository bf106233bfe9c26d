// Host sorts of the elimination loop (dir_c/Quicksort.c), kept apart from the
// solve driver so that they build and test on their own.
#pragma once

namespace lakbcc {

// dQuickSort_xij (dir_c/Quicksort.c:83-141): d[l .. r] ascending, the index
// arrays (any of them null) permuted alongside, in the reference's order.
void quicksort_xij(unsigned limit, double *d, int *i_, int *ib, int *ij, int *nb, int *ga, int *gb, int l, int r);

// dQuickSort (dir_c/Quicksort.c:43-81): d[stride*l] .. d[stride*r] ascending.
void dquicksort_strided(unsigned limit, double *d, long stride, int l, int r);

// The permutation that sorts d[l .. r] ascending when those values are all
// distinct and none is NaN; false otherwise (pm untouched).
bool sort_distinct(const double *d, int l, int r, int *pm);

}  // namespace lakbcc
