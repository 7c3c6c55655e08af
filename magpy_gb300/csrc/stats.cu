// stats.cu -- ensemble statistics on the device, in FP64.
//
// ensemble magnetisation (magpy/results.py:61-75, 134-151):
//     M(t_s) = (1/E) sum_e sum_q m_c[s][e*N + q]
// with a fixed reduction tree per sample (run-to-run identical), and the
// energy dissipated over a window of samples (magpy/results.py:167-191):
//     E_loss = -mu0 * sum_i (M_{i+1} - M_i) (H_{i+1} + H_i) / 2,
// the trapezoid rule of integral H dM as numpy.trapezoid(H, M) states it.
#include <cstdint>
#include <cuda_runtime.h>
#include "plan.hpp"

namespace magpy {
namespace {

constexpr int STAT_THREADS = 256;

__global__ void ensemble_sum_kernel(const double *m, int64_t P, double inv_E, double *out)
{
    __shared__ double red[STAT_THREADS];
    const int64_t s = blockIdx.x;
    const double *row = m + s * P;
    double acc = 0.0;
    for (int64_t i = threadIdx.x; i < P; i += STAT_THREADS) acc += row[i];
    red[threadIdx.x] = acc;
    __syncthreads();
    for (int stride = STAT_THREADS / 2; stride >= 1; stride >>= 1) {
        if (threadIdx.x < stride) red[threadIdx.x] += red[threadIdx.x + stride];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[s] = red[0] * inv_E;
}

// one thread: the window is a few thousand samples at most
__global__ void trapezoid_kernel(const double *M, const double *H, int64_t lo, int64_t hi,
                                 double mu0, double *out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double acc = 0.0;
    for (int64_t i = lo; i + 1 <= hi; i++) acc += (M[i + 1] - M[i]) * (H[i + 1] + H[i]) / 2.0;
    *out = -mu0 * acc;
}

}  // namespace

cudaError_t launch_ensemble_mean(const double *m, int64_t S, int64_t P, int64_t E, double *out,
                                 cudaStream_t stream)
{
    if (S == 0 || E == 0) return cudaSuccess;
    ensemble_sum_kernel<<<(unsigned)S, STAT_THREADS, 0, stream>>>(m, P, 1.0 / (double)E, out);
    return cudaGetLastError();
}

cudaError_t launch_trapezoid(const double *M, const double *H, int64_t lo, int64_t hi, double mu0,
                             double *out, cudaStream_t stream)
{
    trapezoid_kernel<<<1, 32, 0, stream>>>(M, H, lo, hi, mu0, out);
    return cudaGetLastError();
}

}  // namespace magpy
