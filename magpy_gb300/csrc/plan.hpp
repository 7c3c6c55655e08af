// plan.hpp -- host/device description of one ensemble launch.
#pragma once
#include <cstdint>
#include <vector>
#include <cuda_runtime.h>
#include <cuda_fp16.h>
#include "common.cuh"

namespace magpy {

// Device pointers and sizes handed to the kernels (all particles of one launch
// have the same particle count n; members of other sizes go to other launches).
struct DevPlan {
    int64_t E = 0;          // members
    int64_t P = 0;          // particles in all members (E * n)
    int64_t S = 0;          // samples per member
    int32_t n = 0;          // particles per member
    int32_t use_implicit = 0;
    int32_t block_warps = 4; // warps per CTA when members are packed into warps (n <= 32)
    int32_t members_per_warp = 0; // members packed per warp (n <= 32); 0: as many as fit;
                                  // n > 32, mixed precision: members per CTA (1, 2 or 4)
    int32_t shared_cluster = 0;   // every member has the same cluster and parameters
    uint32_t wait_limit = 1u << 24; // polls of a tensor-core phase wait before the watchdog
                                    // status (the final drain keeps its own long bound)
    const MemberDev *members = nullptr;
    const double *m0 = nullptr;    // [3][P]
    const double *axes = nullptr;  // [3][P]
    const double *k_red = nullptr; // [P]
    const double *sr = nullptr;    // [P]
    const double *hj = nullptr;    // [9][P] field-Jacobian block as the reference reads it
    const double *out_scale = nullptr; // [E] Ms (SI output) or 1 (reduced output)
    const double *pt = nullptr;    // pair factors, per cluster [N][N] column-major
    const double *rt = nullptr;    // unit vectors, per cluster [3][N][N]
    const int64_t *sched = nullptr; // sample-step tables
    const double *noise = nullptr;  // injected increments or null
    double *mx = nullptr, *my = nullptr, *mz = nullptr; // [S][P]
    int32_t *status = nullptr;     // [E]
    int64_t *steps = nullptr;      // [E]
    // mixed-precision tables (built by mixed_prepare)
    const float *ftab = nullptr;   // [K][2] applied field per step, or null (constant field,
                                   // or the tensor-core kernels, which compute it)
    const float4 *pr = nullptr;    // pair table (r0, r1, r2, P) per cluster [N][N]
};

// Cache of device blocks (devpool.cu).  pool_free waits for the device unless
// the caller has just synchronised it (device_synced).
cudaError_t pool_alloc(void **ptr, size_t bytes);
void pool_free(void *ptr, bool device_synced = false);
void pool_trim(int device);

// Launchers (one translation unit each).
cudaError_t launch_fp64(const DevPlan &p, cudaStream_t stream);
cudaError_t launch_mixed(const DevPlan &p, cudaStream_t stream);
// Builds the FP32 pair table (from p.pt / p.rt, `clusters` tables of n*n)
// and the per-step field table for a launch whose members share one
// schedule (K steps) and one waveform; the caller frees *ftab and *pr.
cudaError_t mixed_prepare(const DevPlan &p, int64_t clusters, int64_t K, double dt, int shape,
                          double happ, double fapp, float **ftab, float4 **pr,
                          cudaStream_t stream);
// As mixed_prepare, into tables the caller provides (2K floats, clusters*n*n float4).
cudaError_t mixed_fill_tables(const DevPlan &p, int64_t clusters, int64_t K, double dt,
                              int shape, double happ, double fapp, float *ftab, float4 *pr,
                              cudaStream_t stream);
// Tensor-core dipolar path (sllg_tc.cu), members sharing one cluster, 2 <= n <= 64.
struct TcDims { int MP, KP; size_t split_elems; };
TcDims tc_dims(int n);
bool tc_supported(int n);
size_t tc_smem_bytes(int n);
cudaError_t tc_build_d(const double *pt, const double *rt, int n, __half **dhi, __half **dlo,
                       cudaStream_t stream);
cudaError_t tc_init_attributes();
cudaError_t launch_tc(const DevPlan &p, const __half *dhi, const __half *dlo,
                      cudaStream_t stream);
cudaError_t launch_tc_dipolar(const __half *dhi, const __half *dlo, int n, int64_t E,
                              const double *m, double *h, int *flag, size_t slack,
                              cudaStream_t stream);
// Tensor-core dipolar path for clusters of more than 64 particles
// (sllg_tcc.cu): a thread-block cluster of ceil(n / 42) CTAs per group of nb
// (32 or 64) members sharing one cluster; D (tcc_d_elems halves) built once,
// B buffers (tcc_b_elems halves) zeroed once when allocated.
bool tcc_supported(int n);            // Heun: 65 <= n <= 672
bool tcc_implicit_supported(int n);   // implicit midpoint: 2 <= n <= 672
size_t tcc_d_elems(int n);
size_t tcc_b_elems(int n, int64_t E, int nb);
cudaError_t tcc_build_d(const double *pt, const double *rt, int n, __half *d,
                        cudaStream_t stream);
// Kernel attributes (once per device) and the number of clusters of this n
// that can be resident at once (*max_clusters, may be NULL).
cudaError_t tcc_init(int n, int nb, int *max_clusters);
cudaError_t launch_tcc(const DevPlan &p, const __half *d, __half *b, int nb, cudaStream_t stream);
cudaError_t launch_tcc_dipolar(const __half *d, __half *b, int n, int64_t E, const double *m,
                               double *h, int *flag, cudaStream_t stream);
// Ensemble statistics (stats.cu).
cudaError_t launch_ensemble_mean(const double *m, int64_t S, int64_t P, int64_t E, double *out,
                                 cudaStream_t stream);
cudaError_t launch_trapezoid(const double *M, const double *H, int64_t lo, int64_t hi, double mu0,
                             double *out, cudaStream_t stream);
// Two-state master equation (dom.cu): one independent particle per thread.
constexpr int DOM_MAX_ATTEMPTS = 4096;      // rejected RK45 trials before a step gives up
constexpr int32_t DOM_ST_NONFINITE = 4;     // MAGPY_STATUS_NONFINITE
constexpr int32_t DOM_ST_STEP_LIMIT = 32;   // MAGPY_STATUS_STEP_LIMIT
struct DomMember {
    double v, k, T, ms, alpha;  // volume (m^3), K (J/m^3), T (K), Ms (A/m), damping
    double h, f;                // reduced field amplitude H0 / H_k, frequency (Hz)
    double hk;                  // H_k = 2 K / mu0 / Ms (output field scale)
    double p0, p1;              // initial probabilities
};
struct DomArgs {
    int64_t E = 0, N = 0;       // particles, samples per particle
    const DomMember *members = nullptr;
    const int64_t *order = nullptr;  // launch order of the particles, or null
    int32_t shape = 2;
    int64_t ncomp = 1;
    double time_step = 0, end_time = 0, sampling_time = 0;
    int64_t max_steps = 0;
    double *mz = nullptr, *field = nullptr, *time = nullptr;  // [E][N]
    int32_t *status = nullptr;
    int64_t *steps = nullptr;
};
cudaError_t launch_dom(const DomArgs &a, cudaStream_t stream);
// Seeded cluster geometry (geometry.cu): one CTA per member.
struct GeoArgs {
    int64_t E = 0;
    int32_t n = 0;
    int32_t layout = 0;          // 0: random packing in a sphere, 1: chain along z
    int32_t moments_random = 0;  // 0: moments along the easy axes, 1: uniform
    double median_radius = 0, sigma = 0, spacing = 0, packing = 0;
    int64_t max_rounds = 0;
    const int64_t *seeds = nullptr;  // [E]
    double *radius = nullptr, *axes = nullptr, *m0 = nullptr, *location = nullptr;
    int32_t *status = nullptr;       // [E]
};
size_t geometry_smem_bytes(int n);
cudaError_t launch_geometry(const GeoArgs &a, cudaStream_t stream);
// Pathwise adjoint (adjoint.cu): forward with checkpoints, backward sweep.
struct AdjointArgs {
    DevPlan p;            // members, particles, pair table (p.pr), schedule, samples
    const double *v_red;  // [P] reduced volumes
    const float *stab;    // [K][2] waveform values (sin or square sign), or null (constant)
    float happ, dt, sq, alpha, c;
    int64_t K;
    int C, interactions;
    float *ck, *seg;
    const double *wz;     // [S]
    double *grad;         // [5]
};
cudaError_t launch_adjoint(const AdjointArgs &a, bool backward, cudaStream_t stream);
cudaError_t launch_components(int64_t n, const double *m, const double *h, const double *hj,
                              const double *axis, const double *alpha, const double *sr,
                              double *drift, double *diffusion, double *drift_jac,
                              double *diff_jac, double *anis, cudaStream_t stream);
cudaError_t launch_wiener(uint64_t seed, int64_t n_particles, int64_t n_steps, double *out,
                          cudaStream_t stream);

}  // namespace magpy
