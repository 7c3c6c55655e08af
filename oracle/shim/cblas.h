/* Minimal CBLAS declarations for building the reference's lib/*.cpp here.
 * Project-written; the definitions live in oracle/shim/blas_shim.cpp.
 * TEST INFRASTRUCTURE ONLY. */
#ifndef MAGPY_ORACLE_SHIM_CBLAS_H
#define MAGPY_ORACLE_SHIM_CBLAS_H
#ifdef __cplusplus
extern "C" {
#endif
enum CBLAS_ORDER { CblasRowMajor = 101, CblasColMajor = 102 };
enum CBLAS_TRANSPOSE { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 };
double cblas_dnrm2(const int n, const double *x, const int incx);
void cblas_dgemv(const enum CBLAS_ORDER order, const enum CBLAS_TRANSPOSE trans, const int m,
                 const int n, const double alpha, const double *a, const int lda,
                 const double *x, const int incx, const double beta, double *y, const int incy);
#ifdef __cplusplus
}
#endif
#endif
