/* Minimal LAPACKE declarations for building the reference's lib/*.cpp here.
 * Project-written; the definition lives in oracle/shim/blas_shim.cpp.
 * TEST INFRASTRUCTURE ONLY. */
#ifndef MAGPY_ORACLE_SHIM_LAPACKE_H
#define MAGPY_ORACLE_SHIM_LAPACKE_H
#ifdef __cplusplus
extern "C" {
#endif
typedef int lapack_int;
#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102
lapack_int LAPACKE_dgesv_work(int matrix_layout, lapack_int n, lapack_int nrhs, double *a,
                              lapack_int lda, lapack_int *ipiv, double *b, lapack_int ldb);
#ifdef __cplusplus
}
#endif
#endif
