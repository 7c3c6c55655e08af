// geometry.cu -- seeded cluster geometry and initial conditions on the device.
//
// The reference builds cluster geometries on the host with numpy's global
// generator: easy axes uniform on the sphere (magpy/initial_conditions.py:4-37,
// uniform_random_axes), chains (magpy/geometry/coordinates.py,
// chain_coordinates) and hand-placed clusters.  For large batched ensembles
// with a different cluster per member this library draws them on the device
// from a counter-based generator (Philox-4x32-10 keyed by the member seed),
// so no host work scales with the ensemble:
//   * radii log-normal, r = median * exp(sigma z), z standard normal;
//   * easy axes uniform on the sphere (z uniform on [-1, 1], azimuth uniform),
//     the initial moments along the easy axes or independently uniform;
//   * locations: random packing in a sphere of radius R sized for a target
//     packing fraction phi of the exclusion spheres (R = r_x (N / phi)^(1/3),
//     r_x = spacing * mean(r) / 2), every pair at least spacing * (r_i + r_j) / 2
//     apart; or a straight chain along z with pitch spacing * mean(r).
// Packing: one CTA per member places particle i by drawing a round of
// candidates (one per thread) and taking the lowest-numbered valid one, so
// the result depends only on the seed; a member that finds no valid
// candidate in max_rounds rounds is reported and its remaining particles are
// left at NaN.
#include <cmath>
#include "common.cuh"
#include "plan.hpp"

namespace magpy {

namespace {

constexpr int GEO_THREADS = 256;
constexpr uint32_t TAG_RADIUS = 0x6e01u, TAG_AXIS = 0x6e02u, TAG_MOMENT = 0x6e03u,
                   TAG_PLACE = 0x6e04u;

// Uniform on (0, 1) from 53 bits of two words.
__device__ inline double u53(uint32_t hi, uint32_t lo)
{
    const uint64_t b = ((uint64_t)(hi >> 5) << 26) | (uint64_t)(lo >> 6);
    return ((double)b + 0.5) * 1.1102230246251565404e-16;  // 2^-53
}

__device__ inline U4 draw(uint64_t seed, uint32_t i, uint32_t j, uint32_t tag)
{
    return philox4x32_10(U4{i, j, tag, 0x9e01u}, (uint32_t)seed, (uint32_t)(seed >> 32));
}

__device__ inline void unit_vector(U4 r, double v[3])
{
    const double z = 2.0 * u53(r.x, r.y) - 1.0;
    const double ph = 6.283185307179586477 * u53(r.z, r.w);
    const double s = sqrt(fmax(0.0, 1.0 - z * z));
    v[0] = s * cos(ph);
    v[1] = s * sin(ph);
    v[2] = z;
}

__global__ void __launch_bounds__(GEO_THREADS)
    geometry_kernel(GeoArgs a)
{
    extern __shared__ double gsm[];
    const int n = a.n;
    double *pos = gsm;            // [n][3] accepted locations
    double *rad = gsm + 3 * n;    // [n] radii
    int *pick = (int *)(rad + n); // [1] lowest valid candidate of a round
    const int64_t e = blockIdx.x;
    const uint64_t seed = (uint64_t)a.seeds[e];
    const int tid = threadIdx.x;

    // radii, axes, moments: one particle per thread
    for (int i = tid; i < n; i += blockDim.x) {
        const U4 r = draw(seed, (uint32_t)i, 0u, TAG_RADIUS);
        const double z = sqrt(-2.0 * log(u53(r.x, r.y))) * cos(6.283185307179586477 * u53(r.z, r.w));
        const double ri = a.median_radius * exp(a.sigma * z);
        rad[i] = ri;
        double ax[3], m[3];
        unit_vector(draw(seed, (uint32_t)i, 0u, TAG_AXIS), ax);
        if (a.moments_random) unit_vector(draw(seed, (uint32_t)i, 0u, TAG_MOMENT), m);
        else { m[0] = ax[0]; m[1] = ax[1]; m[2] = ax[2]; }
        const int64_t g = e * n + i;
        a.radius[g] = ri;
        for (int c = 0; c < 3; c++) {
            a.axes[3 * g + c] = ax[c];
            a.m0[3 * g + c] = m[c];
        }
    }
    __syncthreads();
    // mean radius (fixed order: the same bits on every launch)
    __shared__ double s_mean;
    if (tid == 0) {
        double s = 0.0;
        for (int i = 0; i < n; i++) s += rad[i];
        s_mean = s / n;
    }
    __syncthreads();
    const double mean_r = s_mean;
    if (a.layout == 1) {  // chain along z
        for (int i = tid; i < n; i += blockDim.x) {
            const int64_t g = e * n + i;
            a.location[3 * g + 0] = 0.0;
            a.location[3 * g + 1] = 0.0;
            a.location[3 * g + 2] = a.spacing * mean_r * i;
        }
        if (tid == 0) a.status[e] = 0;
        return;
    }
    const double rx = 0.5 * a.spacing * mean_r;
    const double R = rx * cbrt((double)n / a.packing);
    int32_t status = 0;
    int placed = 0;
    for (int i = 0; i < n && status == 0; i++) {
        bool done = false;
        for (int64_t round = 0; round < a.max_rounds && !done; round++) {
            const U4 r = draw(seed, (uint32_t)i, (uint32_t)(round * GEO_THREADS + tid), TAG_PLACE);
            const U4 r2 = draw(seed, (uint32_t)i, (uint32_t)(round * GEO_THREADS + tid),
                               TAG_PLACE + 1u);
            const double c[3] = {R * (2.0 * u53(r.x, r.y) - 1.0), R * (2.0 * u53(r.z, r.w) - 1.0),
                                 R * (2.0 * u53(r2.x, r2.y) - 1.0)};
            bool ok = c[0] * c[0] + c[1] * c[1] + c[2] * c[2] <= R * R;
            for (int j = 0; j < i && ok; j++) {
                const double d0 = c[0] - pos[3 * j], d1 = c[1] - pos[3 * j + 1],
                             d2 = c[2] - pos[3 * j + 2];
                const double need = a.spacing * 0.5 * (rad[i] + rad[j]);
                ok = d0 * d0 + d1 * d1 + d2 * d2 >= need * need;
            }
            if (tid == 0) *pick = GEO_THREADS;
            __syncthreads();
            if (ok) atomicMin(pick, tid);
            __syncthreads();
            const int w = *pick;
            if (w < GEO_THREADS) {
                if (tid == w)
                    for (int k = 0; k < 3; k++) pos[3 * i + k] = c[k];
                done = true;
            }
            __syncthreads();
        }
        if (!done) status = 1;
        else placed = i + 1;
    }
    for (int i = tid; i < n; i += blockDim.x) {
        const int64_t g = e * n + i;
        for (int k = 0; k < 3; k++) a.location[3 * g + k] = i < placed ? pos[3 * i + k] : NAN;
    }
    if (tid == 0) a.status[e] = status;
}

}  // namespace

size_t geometry_smem_bytes(int n) { return (size_t)4 * n * sizeof(double) + 16; }

cudaError_t launch_geometry(const GeoArgs &a, cudaStream_t stream)
{
    if (a.E == 0) return cudaSuccess;
    const size_t smem = geometry_smem_bytes(a.n);
    if (smem > 48 * 1024) {
        cudaError_t err = cudaFuncSetAttribute(geometry_kernel,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)smem);
        if (err != cudaSuccess) return err;
    }
    geometry_kernel<<<(unsigned)a.E, GEO_THREADS, smem, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace magpy
