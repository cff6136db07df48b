/* The two CBLAS routines the reference's CPU FMM calls
 * (src/gromacs/rtfmm/mathfunc.cpp: dgemv and dgemm, row-major), forwarded to the
 * OpenBLAS that scipy bundles (exported as scipy_cblas_*).  TEST INFRASTRUCTURE
 * ONLY: it lets the reference's sources compile where no cblas.h is installed. */
#ifndef GBFMM_CBLAS_SUBSET_H
#define GBFMM_CBLAS_SUBSET_H
#ifdef __cplusplus
extern "C" {
#endif
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
void scipy_cblas_dgemv(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE trans, int m, int n, double alpha,
                       const double* a, int lda, const double* x, int incx, double beta, double* y, int incy);
void scipy_cblas_dgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb, int m, int n, int k,
                       double alpha, const double* a, int lda, const double* b, int ldb, double beta, double* c,
                       int ldc);
static inline void cblas_dgemv(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE trans, int m, int n, double alpha,
                               const double* a, int lda, const double* x, int incx, double beta, double* y, int incy)
{
    scipy_cblas_dgemv(order, trans, m, n, alpha, a, lda, x, incx, beta, y, incy);
}
static inline void cblas_dgemm(enum CBLAS_ORDER order, enum CBLAS_TRANSPOSE ta, enum CBLAS_TRANSPOSE tb, int m, int n,
                               int k, double alpha, const double* a, int lda, const double* b, int ldb, double beta,
                               double* c, int ldc)
{
    scipy_cblas_dgemm(order, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}
#ifdef __cplusplus
}
#endif
#endif
