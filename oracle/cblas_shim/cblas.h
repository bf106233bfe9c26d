/* Minimal stand-in for <cblas.h> used only to compile the reference sources
 * into the test oracle.  The reference calls cblas_dgemm from two routines
 * that are not on the bcc path (AnZt_mm.c:35-74, pca_driver.c:856); this
 * header gives them a plain triple loop so the monolith links without a BLAS.
 * Test infrastructure only: nothing in the product includes this file. */
#ifndef LAK_ORACLE_CBLAS_SHIM_H
#define LAK_ORACLE_CBLAS_SHIM_H
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };

static inline void cblas_dgemm(int order, int transa, int transb, int m, int n, int k,
                               double alpha, const double *a, int lda, const double *b, int ldb,
                               double beta, double *c, int ldc)
{
  (void)order; /* column-major only: the two callers pass CblasColMajor */
  for (int j = 0; j < n; j++) {
    for (int i = 0; i < m; i++) {
      double s = 0.0;
      for (int p = 0; p < k; p++) {
        double av = (transa == CblasTrans) ? a[p + (long)i * lda] : a[i + (long)p * lda];
        double bv = (transb == CblasTrans) ? b[j + (long)p * ldb] : b[p + (long)j * ldb];
        s += av * bv;
      }
      c[i + (long)j * ldc] = alpha * s + beta * c[i + (long)j * ldc];
    }
  }
}
#endif
