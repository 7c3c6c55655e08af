// Project-written stand-ins for the three BLAS/LAPACK routines the
// reference calls (cblas_dnrm2, cblas_dgemv, LAPACKE_dgesv_work).  The
// reference links an unpinned OpenBLAS; these functions define the
// arithmetic of the reference build used here as the parity pin.  The
// oracle (oracle/sllg_oracle.cpp: oracle_nrm2, oracle_dgesv) and the CUDA
// path state exactly the same arithmetic.  TEST INFRASTRUCTURE ONLY.
#include <cmath>
#include <vector>
#include <algorithm>
#include "cblas.h"
#include "lapacke.h"

extern "C" {

double cblas_dnrm2(const int n, const double *x, const int incx)
{
    // squares summed inside consecutive triples, triples combined by a
    // pairwise tree over a power-of-two padded index
    int groups = (n + 2) / 3, p = 1;
    while (p < groups) p <<= 1;
    std::vector<double> q(p, 0.0);
    for (int g = 0; g < groups; g++) {
        double s = 0.0;
        for (int k = 3 * g; k < std::min(3 * g + 3, n); k++) s = s + x[k * incx] * x[k * incx];
        q[g] = s;
    }
    for (int stride = p / 2; stride >= 1; stride /= 2)
        for (int i = 0; i < stride; i++) q[i] = q[i] + q[i + stride];
    return std::sqrt(q[0]);
}

void cblas_dgemv(const enum CBLAS_ORDER order, const enum CBLAS_TRANSPOSE trans, const int m,
                 const int n, const double alpha, const double *a, const int lda,
                 const double *x, const int incx, const double beta, double *y, const int incy)
{
    // only the row-major, no-transpose form is used (stochastic_processes.cpp:23)
    (void)order; (void)trans;
    for (int i = 0; i < m; i++) {
        double s = 0.0;
        for (int j = 0; j < n; j++) s = s + a[i * lda + j] * x[j * incx];
        y[i * incy] = alpha * s + (beta == 0.0 ? 0.0 : beta * y[i * incy]);
    }
}

lapack_int LAPACKE_dgesv_work(int matrix_layout, lapack_int n, lapack_int nrhs, double *a,
                              lapack_int lda, lapack_int *ipiv, double *b, lapack_int ldb)
{
    // row-major, nrhs == 1 is the only form used (optimisation.cpp:134)
    (void)matrix_layout; (void)nrhs; (void)ldb;
    lapack_int info = 0;
    for (int k = 0; k < n; k++) {
        int p = k;
        double vmax = std::fabs(a[k * lda + k]);
        for (int i = k + 1; i < n; i++) {
            double v = std::fabs(a[i * lda + k]);
            if (v > vmax) { vmax = v; p = i; }
        }
        ipiv[k] = p + 1;
        if (a[p * lda + k] != 0.0) {
            if (p != k)
                for (int c = 0; c < n; c++) std::swap(a[k * lda + c], a[p * lda + c]);
            double pivot = a[k * lda + k];
            for (int i = k + 1; i < n; i++) {
                double l = a[i * lda + k] / pivot;
                a[i * lda + k] = l;
                for (int c = k + 1; c < n; c++) a[i * lda + c] = a[i * lda + c] - l * a[k * lda + c];
            }
        } else if (info == 0) {
            info = k + 1;
        }
    }
    if (info != 0) return info;
    for (int k = 0; k < n; k++)
        if (ipiv[k] - 1 != k) std::swap(b[k], b[ipiv[k] - 1]);
    for (int k = 0; k < n; k++)
        for (int i = k + 1; i < n; i++) b[i] = b[i] - b[k] * a[i * lda + k];
    for (int k = n - 1; k >= 0; k--) {
        b[k] = b[k] / a[k * lda + k];
        for (int i = 0; i < k; i++) b[i] = b[i] - b[k] * a[i * lda + k];
    }
    return 0;
}

}  // extern "C"
