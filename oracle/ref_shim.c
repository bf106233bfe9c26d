/* Test-infrastructure shim compiled together with the reference sources into
 * oracle/_ref/liblakref.so.  The reference program sets up its bump arena in
 * main() (dir_c/lakcluster_ver18.c:287-306); a shared library has no main, so
 * lakref_init() does the same set-up for callers that drive the reference's own
 * wrap_* kernels through ctypes (tests/golden/make_golden.py).
 * Only the test harness uses this file; the product never links it. */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <omp.h>

struct lakref_wkspace_point { struct lakref_wkspace_point *parent, *child; long long check; long long *point; };
extern unsigned char *wkspace, *wkspace_base;
extern long long wkspace_left, wkspace_used;
extern unsigned long long GLOBAL_memory_gb, GLOBAL_memory_mb, GLOBAL_memory_kb;
extern int GLOBAL_thread_count, GLOBAL_omp_type, GLOBAL_verbose, GLOBAL_2_cache_size;
extern void *wkspace_point_0, *wkspace_point_t;
extern void *wkspace_make_point(void);

static unsigned char *lakref_arena = NULL;

/* Allocate an arena of `mb` MiB and point the reference's allocator at it.
 * Calling it again discards everything allocated so far. */
int lakref_init(long long mb, int nthreads, int omp_on)
{
  if (lakref_arena) { free(lakref_arena); lakref_arena = NULL; }
  unsigned long long bytes = (unsigned long long)mb * 1048576ULL;
  lakref_arena = (unsigned char *)malloc(bytes + 64);
  if (!lakref_arena) return -1;
  wkspace = (unsigned char *)(((unsigned long)lakref_arena + 63) & ~63UL);
  wkspace_base = wkspace;
  wkspace_left = (long long)(bytes - (unsigned long long)(wkspace - lakref_arena));
  wkspace_used = 0;
  GLOBAL_memory_mb = (unsigned long long)mb; GLOBAL_memory_kb = GLOBAL_memory_mb * 1024ULL;
  GLOBAL_memory_gb = GLOBAL_memory_mb / 1024ULL;
  GLOBAL_thread_count = nthreads > 0 ? nthreads : 1;
  GLOBAL_omp_type = omp_on ? 1 : 0;
  GLOBAL_verbose = 0;
  GLOBAL_2_cache_size = 1048576; /* sysconf value used only to size Z-row blocks */
  if (nthreads > 0) omp_set_num_threads(nthreads);
  wkspace_point_0 = wkspace_make_point();
  wkspace_point_t = wkspace_point_0;
  return 0;
}

long long lakref_wkspace_left(void) { return wkspace_left; }
