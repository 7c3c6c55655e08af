// capi.cu -- host side of the C-ABI (include/magpy_gpu.h).
//
// Turns the reference's inputs into a launch plan: the physical-to-reduced
// conversion of lib/simulation.cpp:476-583 (same formulas, same order of
// floating-point operations, so the reduced quantities are bit-identical
// to the reference's), the pair tables of the dipolar sum
// (lib/field.cpp:187-225), the field-Jacobian blocks of the implicit solve,
// and the sample/step schedule of lib/simulation.cpp:342-405.  Then it moves
// the data to the device, launches, and writes the results back in the
// reference's units.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <string>
#include <tuple>
#include <vector>
#include <algorithm>
#include <memory>
#include <mutex>
#include <new>
#include <stdexcept>
#include <cuda_runtime.h>

#include "../../include/magpy_gpu.h"
#include "plan.hpp"

namespace magpy {
namespace {

thread_local std::string g_err = "no error";

const double KB = 1.38064852e-23;     // include/constants.hpp:10-12
const double MU0 = 1.25663706e-6;
const double GYROMAG = 1.76086e11;

int fail(int code, const std::string &msg)
{
    g_err = msg;
    return code;
}

#define CUDA_TRY(expr)                                                                     \
    do {                                                                                   \
        cudaError_t err_ = (expr);                                                         \
        if (err_ != cudaSuccess)                                                           \
            return fail(err_ == cudaErrorMemoryAllocation ? MAGPY_ERR_OUT_OF_MEMORY        \
                                                          : MAGPY_ERR_CUDA,                \
                        std::string(#expr) + ": " + cudaGetErrorString(err_));             \
    } while (0)

// Reduced-unit description of one cluster: the arguments of the reduced
// simulation::full_dynamics (include/simulation.hpp:51-72).
struct Reduced {
    int64_t n = 0;
    std::vector<double> sr, k_red, v_red, axes, m0, unit, dist_mag;
    double k_av = 0, v_av = 0, alpha = 0, ms = 0, dt = 0, end = 0, happ = 0, fapp = 0;
    int32_t shape = MAGPY_FIELD_CONSTANT;
    // physical conversion (1 for reduced-unit calls)
    double H_k = 1.0, time_factor = 1.0, out_scale = 1.0;
};

// lib/simulation.cpp:498-583 and lib/distances.cpp:20-113
Reduced reduce_physical(int64_t n, const double *radius, const double *anisotropy,
                        const double *axes, const double *m0, const double *location,
                        double ms, double damping, double temperature, double time_step,
                        double end_time, int32_t shape, double amp, double freq)
{
    Reduced R;
    R.n = n;
    std::vector<double> volume(n);
    for (int64_t i = 0; i < n; i++)
        volume[i] = 4.0 / 3.0 * M_PI * radius[i] * radius[i] * radius[i];
    double vsum = 0.0;
    for (int64_t i = 0; i < n; i++) vsum += volume[i];
    const double average_volume = vsum / n;
    R.v_red.resize(n);
    for (int64_t i = 0; i < n; i++) R.v_red[i] = volume[i] / average_volume;
    double ksum = 0.0;
    for (int64_t i = 0; i < n; i++) ksum += anisotropy[i];
    const double average_anisotropy = ksum / n;
    R.k_red.resize(n);
    for (int64_t i = 0; i < n; i++) R.k_red[i] = anisotropy[i] / average_anisotropy;
    const double anisotropy_field = 2 * average_anisotropy / MU0 / ms;
    const double time_factor = GYROMAG * MU0 * anisotropy_field / (1 + damping * damping);
    R.sr.resize(n);
    for (int64_t i = 0; i < n; i++)
        R.sr[i] = std::sqrt(damping * KB * temperature / (average_anisotropy * volume[i]) /
                            (1 + damping * damping));
    // distances: vec[i][j] = p_j - p_i, magnitudes, unit vectors
    std::vector<double> vec(n * n * 3);
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < n; j++)
            for (int k = 0; k < 3; k++)
                vec[(i * n + j) * 3 + k] = location[j * 3 + k] - location[i * 3 + k];
    std::vector<double> mag(n * n);
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < n; j++) {
            const double *d = &vec[(i * n + j) * 3];
            double v = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            mag[i * n + j] = v;
            mag[j * n + i] = v;
        }
    R.unit.resize(n * n * 3);
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < n; j++)
            for (int k = 0; k < 3; k++)
                R.unit[(i * n + j) * 3 + k] = vec[(i * n + j) * 3 + k] / mag[i * n + j];
    const double scale = std::pow(average_volume, 1. / 3);
    R.dist_mag = mag;
    for (auto &v : R.dist_mag) v /= scale;
    R.axes.assign(axes, axes + 3 * n);
    R.m0.assign(m0, m0 + 3 * n);
    R.k_av = average_anisotropy;
    R.v_av = average_volume;
    R.alpha = damping;
    R.ms = ms;
    R.dt = time_step * time_factor;
    R.end = end_time * time_factor;
    R.happ = amp / anisotropy_field;
    R.fapp = freq / time_factor;
    R.shape = shape;
    R.H_k = anisotropy_field;
    R.time_factor = time_factor;
    R.out_scale = ms;
    return R;
}

// applied field in reduced units, lib/simulation.cpp:552-573
double field_fn(int32_t shape, double happ, double fapp, double t)
{
    if (shape == MAGPY_FIELD_CONSTANT) return happ;
    if (shape == MAGPY_FIELD_SINE) return happ * std::sin(2 * M_PI * fapp * t);
    return happ * (int(t * fapp * 2) % 2 ? -1 : 1);
}

// Sample/step schedule of lib/simulation.cpp:342-405: sched[s] = number of
// steps taken when sample s is recorded (sample s holds the state after
// sched[s]-1 steps).  Reproduces the reference's comparisons t <= s*Ts with
// t = step*dt in double arithmetic exactly.
int make_schedule(double dt, double end, int64_t S, std::vector<int64_t> &ks, int64_t &K)
{
    ks.assign(std::max<int64_t>(S, 1), 0);
    K = 0;
    if (S <= 1) return MAGPY_SUCCESS;
    if (!(dt > 0) || !std::isfinite(dt) || !(end >= 0) || !std::isfinite(end))
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "time_step must be > 0 and end_time >= 0, finite");
    if (S > (int64_t)0xffffffffLL)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "max_samples exceeds the 32-bit sample counter");
    const double Ts = end / (double)(S - 1);
    uint64_t k = 0;
    double t = 0.0;
    for (int64_t s = 1; s < S; s++) {
        const double thr = (double)(uint32_t)s * Ts;
        if (t <= thr) {
            const double est = thr / dt;
            if (!(est < 4294967294.0))
                return fail(MAGPY_ERR_INVALID_ARGUMENT,
                            "more than 2^32-1 steps: the reference's 32-bit step counter would wrap");
            uint64_t kk = (uint64_t)est;
            if (kk <= k) kk = k + 1;
            while (kk - 1 > k && (double)(uint32_t)(kk - 1) * dt > thr) kk--;
            while (!((double)(uint32_t)kk * dt > thr)) kk++;
            k = kk;
            t = (double)(uint32_t)k * dt;
        }
        ks[s] = (int64_t)k;
    }
    K = (int64_t)k;
    return MAGPY_SUCCESS;
}

// Device allocation from the block cache (devpool.cu).
struct DBuf {
    void *p = nullptr;
    DBuf() = default;
    DBuf(const DBuf &) = delete;
    DBuf &operator=(const DBuf &) = delete;
    // after the device was synchronised: back to the cache without waiting
    void release_synced() { pool_free(p, true); p = nullptr; }
    ~DBuf() { if (p) pool_free(p, false); }
};

// dst[r][e*n + q] = src[r][q] for rows r < rows, members e < E.
__global__ void expand_kernel(const double *src, int rows, int64_t n, int64_t E, double *dst)
{
    const int64_t P = E * n, total = (int64_t)rows * P;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < total;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / P, q = (i % P) % n;
        dst[i] = src[r * n + q];
    }
}

cudaError_t launch_expand(const double *src, int rows, int64_t n, int64_t E, double *dst,
                          cudaStream_t st)
{
    const int64_t total = (int64_t)rows * E * n;
    if (total == 0) return cudaSuccess;
    const int64_t blocks = std::min<int64_t>((total + 255) / 256, 152 * 16);
    expand_kernel<<<(unsigned)blocks, 256, 0, st>>>(src, rows, n, E, dst);
    return cudaGetLastError();
}

}  // namespace
}  // namespace magpy

// A reusable launch: device-resident inputs, tables and outputs of one
// uniform-size ensemble.
struct magpy_plan {
    magpy::DevPlan p;
    magpy::DBuf bufs[20];
    float *ftab = nullptr;
    float4 *pr = nullptr;
    __half *tc_d = nullptr;     // FP16 hi/lo dipolar matrix (tensor-core mode)
    __half *tcc_b = nullptr;    // B buffers of the cluster kernel (n > 64)
    size_t tcc_b_bytes = 0;
    int32_t tcc_last_nb = 0;    // members per cluster of the last run (0: none yet)
    int tcc_max_clusters[3] = {0, 0, 0};  // resident clusters of 32 / 64 / 40 members
    int32_t precision = 0;
    bool on_device = false;     // the caller's buffers are device pointers
    int64_t max_steps = 0;
    std::vector<double> times, fields;  // [E][S] host-side sample times and fields
    ~magpy_plan()
    {
        // a run may still be in flight on any stream: wait once, then hand
        // every buffer back to the cache
        cudaDeviceSynchronize();
        for (auto &b : bufs) b.release_synced();
        magpy::pool_free(ftab, true);
        magpy::pool_free(pr, true);
        magpy::pool_free(tc_d, true);
        magpy::pool_free(tcc_b, true);
    }
};

namespace magpy {
namespace {

template <class T>
int upload(DBuf &b, const std::vector<T> &v, cudaStream_t st, const T **out)
{
    if (v.empty()) { *out = nullptr; return MAGPY_SUCCESS; }
    CUDA_TRY(pool_alloc(&b.p, v.size() * sizeof(T)));
    CUDA_TRY(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, st));
    *out = (const T *)b.p;
    return MAGPY_SUCCESS;
}

// Builds a plan for members given in reduced form (all of size n).
// noise: host or device pointer ([E][noise_per_member]) or null.
int make_plan(const std::vector<const Reduced *> &members, const std::vector<uint64_t> &seeds,
              int32_t renorm, int32_t interactions, int32_t use_implicit, double eps,
              int64_t max_iter, int64_t S, int32_t precision, const double *noise,
              int64_t noise_per_member, bool on_device, bool keep_traj, cudaStream_t st,
              magpy_plan **out)
{
    const int64_t E = (int64_t)members.size();
    const int64_t n = E ? members[0]->n : 1;
    const int64_t P = E * n;
    if (max_iter <= 0) max_iter = 1000;
    std::unique_ptr<magpy_plan> plan(new magpy_plan());
    plan->precision = precision;
    plan->on_device = on_device;

    std::vector<MemberDev> md(E);
    // Members that all share one cluster (the common case) get their
    // per-particle arrays expanded on the device from one copy (expand_kernel)
    // instead of E copies built and uploaded here.
    bool shared = E > 0;
    for (int64_t e = 1; e < E && shared; e++) shared = members[e] == members[0];
    const int64_t Pb = shared ? n : P;  // rows built on the host
    std::vector<double> m0(3 * Pb), axes(3 * Pb), k_red(Pb), sr(Pb),
        hj(use_implicit ? 9 * Pb : 0), out_scale(E);
    std::vector<double> pt, rt;
    std::vector<int64_t> sched;
    std::map<const Reduced *, int64_t> cluster_of;
    std::map<std::pair<double, double>, int64_t> sched_of;
    plan->times.resize(E * S);
    plan->fields.resize(E * S);

    for (int64_t e = 0; e < E; e++) {
        const Reduced &R = *members[e];
        if (R.n != n) return fail(MAGPY_ERR_INVALID_ARGUMENT, "members differ in size");
        if (shared && e > 0) {
            // every member has member 0's reduced parameters: its record,
            // sample times and fields are member 0's but for its particle
            // offset, noise offset and seed
            md[e] = md[0];
            md[e].pbase = e * n;
            md[e].noise_off = e * noise_per_member;
            md[e].seed = seeds[e];
            out_scale[e] = out_scale[0];
            std::copy(plan->times.begin(), plan->times.begin() + S, plan->times.begin() + e * S);
            std::copy(plan->fields.begin(), plan->fields.begin() + S, plan->fields.begin() + e * S);
            continue;
        }
        MemberDev &d = md[e];
        d.dt = R.dt;
        d.sqrt_dt = std::sqrt(R.dt);
        d.alpha = R.alpha;
        d.happ = R.happ;
        d.fapp = R.fapp;
        d.Ah = std::sqrt(2 * 1000.0 * std::abs(std::log(R.dt)));  // integrators.cpp:599-600
        d.eps = eps;
        d.max_iter = max_iter;
        d.pbase = e * n;
        d.noise_off = e * noise_per_member;
        d.noise_len = noise ? noise_per_member : 0;
        d.seed = seeds[e];
        d.n = (int32_t)n;
        d.shape = R.shape;
        d.renorm = renorm;
        d.interactions = interactions;
        out_scale[e] = R.out_scale;
        const bool build = !shared || e == 0;
        for (int64_t q = 0; q < n && build; q++) {
            const int64_t g = e * n + q;
            for (int c = 0; c < 3; c++) {
                m0[c * Pb + g] = R.m0[3 * q + c];
                axes[c * Pb + g] = R.axes[3 * q + c];
            }
            k_red[g] = R.k_red[q];
            sr[g] = R.sr[q];
        }
        if (use_implicit && build) {
            // The reference hands llg::drift_jacobian the pointer hj + 3q into
            // the dense 3n x 3n anisotropy Jacobian (lib/llg.cpp:386) and
            // reads 9 consecutive doubles: flat indices 3q .. 3q+8.
            const int64_t n3 = 3 * n;
            for (int64_t q = 0; q < n; q++)
                for (int64_t k = 0; k < 9; k++) {
                    const int64_t f = 3 * q + k, r = f / n3, c = f % n3;
                    hj[k * Pb + e * n + q] =
                        (r / 3 == c / 3) ? R.k_red[r / 3] * R.axes[r] * R.axes[c] : 0.0;
                }
        }
        // pair tables, shared between members with the same cluster
        auto it = cluster_of.find(&R);
        if (it == cluster_of.end()) {
            const int64_t off = (int64_t)pt.size();
            if (interactions && n > 1) {
                const double pref = MU0 * R.ms * R.ms / 8.0 / M_PI / R.k_av;  // field.cpp:212-215
                pt.resize(off + n * n, 0.0);
                rt.resize(3 * (off + n * n), 0.0);
                for (int64_t q = 0; q < n; q++)
                    for (int64_t j = 0; j < n; j++) {
                        if (j == q) continue;
                        const double cube = std::pow(R.dist_mag[q * n + j], 3);  // simulation.cpp:262
                        pt[off + j * n + q] = pref * (R.v_red[j] / cube);
                        for (int c = 0; c < 3; c++)
                            rt[3 * off + (c * n + j) * n + q] = R.unit[(q * n + j) * 3 + c];
                    }
            }
            cluster_of[&R] = off;
            d.cluster_off = off;
        } else {
            d.cluster_off = it->second;
        }
        // sample schedule, shared between members with the same (dt, end)
        auto key = std::make_pair(R.dt, R.end);
        auto is = sched_of.find(key);
        if (is == sched_of.end()) {
            std::vector<int64_t> ks;
            int64_t K = 0;
            int rc = make_schedule(R.dt, R.end, S, ks, K);
            if (rc) return rc;
            d.sched_off = (int64_t)sched.size();
            sched.insert(sched.end(), ks.begin(), ks.end());
            sched_of[key] = d.sched_off;
        } else {
            d.sched_off = is->second;
        }
        const int64_t K = S > 1 ? sched[d.sched_off + S - 1] : 0;
        plan->max_steps = std::max(plan->max_steps, K);
        if (noise && K * 3 * n > noise_per_member)
            return fail(MAGPY_ERR_NOISE_TOO_SHORT,
                        "injected noise holds " + std::to_string(noise_per_member) +
                            " increments per member; the run needs " +
                            std::to_string(K * 3 * n));
        // sample times and fields, lib/simulation.cpp:209-219, 400-401, 614-616
        const double Ts = R.end / (double)(S - 1);
        for (int64_t s = 0; s < S; s++) {
            const double ts = (s == 0) ? 0.0 : (double)(uint32_t)s * Ts;
            plan->times[e * S + s] = ts / R.time_factor;
            plan->fields[e * S + s] = field_fn(R.shape, R.happ, R.fapp, ts) * R.H_k;
        }
    }
    if (precision == MAGPY_PRECISION_MIXED || precision == MAGPY_PRECISION_MIXED_TC)
        for (int64_t e = 1; e < E; e++)
            if (md[e].sched_off != md[0].sched_off || md[e].dt != md[0].dt ||
                md[e].shape != md[0].shape || md[e].happ != md[0].happ ||
                md[e].fapp != md[0].fapp)
                return fail(MAGPY_ERR_UNSUPPORTED,
                            "the mixed-precision kernel needs one time step and one applied-field "
                            "waveform per launch; split the ensemble");

    DevPlan &p = plan->p;
    DBuf *b = plan->bufs;
    p.E = E;
    p.P = P;
    p.S = S;
    p.n = (int32_t)n;
    p.use_implicit = use_implicit;
    p.shared_cluster = shared ? 1 : 0;
    int rc;
    if ((rc = upload(b[0], md, st, &p.members))) return rc;
    if (shared) {
        // one cluster's rows, then [rows][P] arrays filled on the device:
        // m0, axes (3 rows each), k_red, sr (1 each), hj (9, implicit only)
        const int rows = 8 + (use_implicit ? 9 : 0);
        std::vector<double> one((size_t)rows * n);
        for (int c = 0; c < 3; c++)
            for (int64_t q = 0; q < n; q++) {
                one[(size_t)c * n + q] = m0[c * n + q];
                one[(size_t)(3 + c) * n + q] = axes[c * n + q];
            }
        for (int64_t q = 0; q < n; q++) {
            one[(size_t)6 * n + q] = k_red[q];
            one[(size_t)7 * n + q] = sr[q];
        }
        if (use_implicit)
            for (int k = 0; k < 9; k++)
                for (int64_t q = 0; q < n; q++) one[(size_t)(8 + k) * n + q] = hj[k * n + q];
        DBuf src;
        const double *dsrc = nullptr;
        if ((rc = upload(src, one, st, &dsrc))) return rc;
        CUDA_TRY(pool_alloc(&b[1].p, (size_t)rows * P * sizeof(double)));
        double *dst = (double *)b[1].p;
        cudaError_t err = launch_expand(dsrc, rows, n, E, dst, st);
        if (err != cudaSuccess) return fail(MAGPY_ERR_CUDA, cudaGetErrorString(err));
        p.m0 = dst;
        p.axes = dst + 3 * P;
        p.k_red = dst + 6 * P;
        p.sr = dst + 7 * P;
        p.hj = use_implicit ? dst + 8 * P : nullptr;
        CUDA_TRY(cudaStreamSynchronize(st));  // `src` is released on return
    } else {
        if ((rc = upload(b[1], m0, st, &p.m0))) return rc;
        if ((rc = upload(b[2], axes, st, &p.axes))) return rc;
        if ((rc = upload(b[3], k_red, st, &p.k_red))) return rc;
        if ((rc = upload(b[4], sr, st, &p.sr))) return rc;
        if ((rc = upload(b[5], hj, st, &p.hj))) return rc;
    }
    if ((rc = upload(b[6], out_scale, st, &p.out_scale))) return rc;
    if ((rc = upload(b[7], pt, st, &p.pt))) return rc;
    if ((rc = upload(b[8], rt, st, &p.rt))) return rc;
    if ((rc = upload(b[9], sched, st, &p.sched))) return rc;
    if (noise && E > 0) {
        const size_t bytes = (size_t)E * noise_per_member * sizeof(double);
        CUDA_TRY(pool_alloc(&b[10].p, bytes));
        CUDA_TRY(cudaMemcpyAsync(b[10].p, noise, bytes,
                                 on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, st));
        p.noise = (const double *)b[10].p;
    }
    const size_t traj = (size_t)S * P;
    if (keep_traj && traj > 0) {
        CUDA_TRY(pool_alloc(&b[11].p, 3 * traj * sizeof(double)));
        p.mx = (double *)b[11].p;
        p.my = p.mx + traj;
        p.mz = p.my + traj;
    }
    if (E > 0) {
        CUDA_TRY(pool_alloc(&b[12].p, E * sizeof(int32_t)));
        CUDA_TRY(pool_alloc(&b[13].p, E * sizeof(int64_t)));
        p.status = (int32_t *)b[12].p;
        p.steps = (int64_t *)b[13].p;
    }
    // tensor cores: Heun below 65 particles on the single-CTA kernel, above on
    // the cluster kernel; the implicit solve on the cluster kernel for any size
    const bool tc_cluster = use_implicit ? tcc_implicit_supported((int)n)
                                         : (!tc_supported((int)n) && tcc_supported((int)n));
    if (precision == MAGPY_PRECISION_MIXED_TC) {
        if (!(interactions && n > 1 && (tc_cluster || tc_supported((int)n))))
            return fail(MAGPY_ERR_UNSUPPORTED,
                        "the tensor-core mode needs dipolar interactions and 2 <= n_particles <= 672");
        if (cluster_of.size() > 1)
            return fail(MAGPY_ERR_UNSUPPORTED,
                        "the tensor-core mode needs every member to share one geometry and one "
                        "set of material parameters");
    }
    if ((precision == MAGPY_PRECISION_MIXED || precision == MAGPY_PRECISION_MIXED_TC) && E > 0) {
        const int64_t clusters = pt.empty() ? 0 : (int64_t)pt.size() / (n * n);
        // the tensor-core kernels compute the applied field themselves (the
        // same FP64 expression, heun_field_f32): no per-step table, whose size
        // grows with the run (8 bytes a step)
        const int32_t table_shape =
            precision == MAGPY_PRECISION_MIXED_TC ? (int32_t)FIELD_CONSTANT : md[0].shape;
        cudaError_t err = mixed_prepare(p, clusters, plan->max_steps, md[0].dt, table_shape,
                                        md[0].happ, md[0].fapp, &plan->ftab, &plan->pr, st);
        if (err != cudaSuccess)
            return fail(MAGPY_ERR_CUDA, std::string("mixed tables: ") + cudaGetErrorString(err));
        p.ftab = plan->ftab;
        p.pr = plan->pr;
    }
    if (precision == MAGPY_PRECISION_MIXED_TC && E > 0 && !tc_cluster) {
        cudaError_t aerr = tc_init_attributes();
        if (aerr != cudaSuccess)
            return fail(MAGPY_ERR_CUDA, std::string("tensor-core kernel attributes: ") +
                                            cudaGetErrorString(aerr));
        __half *dlo = nullptr;
        cudaError_t err = tc_build_d(p.pt, p.rt, (int)n, &plan->tc_d, &dlo, st);
        if (err != cudaSuccess)
            return fail(MAGPY_ERR_CUDA, std::string("dipolar matrix: ") + cudaGetErrorString(err));
    } else if (precision == MAGPY_PRECISION_MIXED_TC && E > 0) {
        // clusters of more than 64 particles: D in the cluster kernel's
        // tile layout, and B buffers sized for either member count per cluster
        for (int nb : {32, 64, 40}) {
            cudaError_t aerr =
                tcc_init((int)n, nb, &plan->tcc_max_clusters[nb == 32 ? 0 : nb == 64 ? 1 : 2]);
            if (aerr != cudaSuccess)
                return fail(MAGPY_ERR_CUDA, std::string("cluster tensor-core kernel set-up: ") +
                                                cudaGetErrorString(aerr));
        }
        CUDA_TRY(pool_alloc((void **)&plan->tc_d, tcc_d_elems((int)n) * sizeof(__half)));
        cudaError_t err = tcc_build_d(p.pt, p.rt, (int)n, plan->tc_d, st);
        if (err != cudaSuccess)
            return fail(MAGPY_ERR_CUDA, std::string("dipolar matrix: ") + cudaGetErrorString(err));
        plan->tcc_b_bytes = std::max({tcc_b_elems((int)n, E, 32), tcc_b_elems((int)n, E, 40),
                                      tcc_b_elems((int)n, E, 48),
                                      tcc_b_elems((int)n, E, 64)}) *
                            sizeof(__half);
        CUDA_TRY(pool_alloc((void **)&plan->tcc_b, plan->tcc_b_bytes));
        CUDA_TRY(cudaMemsetAsync(plan->tcc_b, 0, plan->tcc_b_bytes, st));
    }
    CUDA_TRY(cudaStreamSynchronize(st));  // host tables are released on return
    *out = plan.release();
    return MAGPY_SUCCESS;
}

int run_plan(magpy_plan *plan, cudaStream_t st)
{
    cudaError_t le;
    if (plan->precision == MAGPY_PRECISION_MIXED_TC && !plan->p.use_implicit &&
        tc_supported(plan->p.n)) {
        const TcDims dims = tc_dims(plan->p.n);
        le = launch_tc(plan->p, plan->tc_d, plan->tc_d + dims.split_elems, st);
    } else if (plan->precision == MAGPY_PRECISION_MIXED_TC) {
        // members per cluster: as the launch shape asks (32, 40 or 64; 48
        // for Heun); else the count with the fewest waves of resident
        // clusters, then the fewest members (a wave takes time in proportion
        // to its clusters' members: at N = 512 an implicit step takes 0.184 ms
        // a wave with 32, 0.345 with 64; Heun at E = 1638 measured 64 / 48 /
        // 40 / 32: N = 84 134 / 123 / 98 / 92 ms per 1e4 steps, N = 125 145 /
        // 134 / 109 / 197 (32: two waves), and at N = 216, E = 1024 212 / 189
        // / 323 / 296 (40 and 32: two waves); every cluster form runs one CTA
        // per SM, so the resident count depends on the cluster size alone)
        const int32_t mpw = plan->p.members_per_warp;
        const bool imp = plan->p.use_implicit;
        int nb = 64;
        if (mpw == 32 || mpw == 40 || (mpw == 48 && !imp)) {
            nb = mpw;
        } else if (mpw != 64) {
            int64_t best = INT64_MAX;
            for (int m : {64, 48, 40, 32}) {
                if (m == 48 && imp) continue;  // no 48-member implicit form
                const int64_t res =
                    std::max(1, plan->tcc_max_clusters[m == 32 ? 0 : m == 40 ? 2 : 1]);
                const int64_t waves = ((plan->p.E + m - 1) / m + res - 1) / res;
                if (waves <= best) { best = waves; nb = m; }  // equal: fewer members
            }
        }
        // the B buffers were sized for every member count a launch may take
        if (tcc_b_elems((int)plan->p.n, plan->p.E, nb) * sizeof(__half) > plan->tcc_b_bytes)
            return fail(MAGPY_ERR_UNSUPPORTED, "cluster B buffer smaller than the " +
                                                   std::to_string(nb) + "-member layout");
        if (plan->tcc_last_nb != 0 && plan->tcc_last_nb != nb)
            // the other layout's words could land on positions this one
            // never writes: start from zero again
            CUDA_TRY(cudaMemsetAsync(plan->tcc_b, 0, plan->tcc_b_bytes, st));
        plan->tcc_last_nb = nb;
        le = launch_tcc(plan->p, plan->tc_d, plan->tcc_b, nb, st);
    } else if (plan->precision == MAGPY_PRECISION_MIXED && !plan->p.use_implicit) {
        le = launch_mixed(plan->p, st);
    } else {
        le = launch_fp64(plan->p, st);
    }
    if (le != cudaSuccess)
        return fail(MAGPY_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(le));
    return MAGPY_SUCCESS;
}

int copy_out(magpy_plan *plan, double *mx, double *my, double *mz, double *time_out,
             double *field_out, int32_t *status, int64_t *steps, cudaStream_t st)
{
    const DevPlan &p = plan->p;
    const bool dev = plan->on_device;
    const cudaMemcpyKind down = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const cudaMemcpyKind up = dev ? cudaMemcpyHostToDevice : cudaMemcpyHostToHost;
    const size_t traj = (size_t)p.S * p.P;
    if (mx && p.mx && traj) {
        CUDA_TRY(cudaMemcpyAsync(mx, p.mx, traj * sizeof(double), down, st));
        CUDA_TRY(cudaMemcpyAsync(my, p.my, traj * sizeof(double), down, st));
        CUDA_TRY(cudaMemcpyAsync(mz, p.mz, traj * sizeof(double), down, st));
    }
    if (status && p.E) CUDA_TRY(cudaMemcpyAsync(status, p.status, p.E * sizeof(int32_t), down, st));
    if (steps && p.E) CUDA_TRY(cudaMemcpyAsync(steps, p.steps, p.E * sizeof(int64_t), down, st));
    const size_t es = (size_t)p.E * p.S;
    if (dev) {
        if (time_out && es)
            CUDA_TRY(cudaMemcpyAsync(time_out, plan->times.data(), es * sizeof(double), up, st));
        if (field_out && es)
            CUDA_TRY(cudaMemcpyAsync(field_out, plan->fields.data(), es * sizeof(double), up, st));
    } else {
        // host to host: copied here while the device copies above are in flight
        if (time_out && es) std::memcpy(time_out, plan->times.data(), es * sizeof(double));
        if (field_out && es) std::memcpy(field_out, plan->fields.data(), es * sizeof(double));
    }
    CUDA_TRY(cudaStreamSynchronize(st));
    return MAGPY_SUCCESS;
}

bool finite_all(const double *a, int64_t n)
{
    for (int64_t i = 0; i < n; i++)
        if (!std::isfinite(a[i])) return false;
    return true;
}

}  // namespace
}  // namespace magpy

using namespace magpy;

extern "C" {

const char *magpy_last_error_string(void) { return g_err.c_str(); }

const char *magpy_version(void) { return "magpy-gb300 0.1 (sm_103a)"; }

int magpy_step_count(double time_step, double end_time, int64_t max_samples, int64_t *steps)
{
    if (!steps) return fail(MAGPY_ERR_INVALID_ARGUMENT, "steps is NULL");
    if (max_samples < 1) return fail(MAGPY_ERR_INVALID_ARGUMENT, "max_samples must be >= 1");
    std::vector<int64_t> ks;
    int64_t K = 0;
    int rc = make_schedule(time_step, end_time, max_samples, ks, K);
    if (rc) return rc;
    *steps = K;
    return MAGPY_SUCCESS;
}

static int plan_from_desc(const magpy_ensemble_desc *d, bool keep_traj, cudaStream_t st,
                          magpy_plan **out)
{
    if (!d || !out) return fail(MAGPY_ERR_INVALID_ARGUMENT, "desc or plan pointer is NULL");
    const int64_t E = d->n_members, n = d->n_particles, S = d->max_samples;
    if (E < 0 || n < 1 || n > 1024)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "need n_members >= 0 and 1 <= n_particles <= 1024");
    if (S < 1)
        return fail(MAGPY_ERR_INVALID_ARGUMENT,
                    "max_samples must be >= 1 (the reference's -1 never terminates, "
                    "lib/simulation.cpp:345-355)");
    if (!d->radius || !d->anisotropy || !d->anisotropy_axis || !d->magnetisation_direction ||
        !d->location || !d->seeds)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "a required input pointer is NULL");
    if (d->field_shape < 0 || d->field_shape > 2)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "field_shape must be SINE, SQUARE or CONSTANT "
                                                "(the reference throws std::invalid_argument)");
    if (d->precision != MAGPY_PRECISION_FP64 && d->precision != MAGPY_PRECISION_MIXED &&
        d->precision != MAGPY_PRECISION_MIXED_TC)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "unknown precision");
    if (d->precision == MAGPY_PRECISION_MIXED_TC &&
        !(d->interactions && n > 1 &&
          (d->use_implicit ? tcc_implicit_supported((int)n)
                           : (tc_supported((int)n) || tcc_supported((int)n)))))
        return fail(MAGPY_ERR_UNSUPPORTED,
                    "the tensor-core mode needs dipolar interactions and 2 <= n_particles <= 672");
    if (d->noise && d->noise_per_member < 0)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "noise_per_member < 0");
    const bool dev = d->buffers_on_device != 0;
    const int64_t rows = d->per_member_geometry ? E * n : n;

    // geometry and per-member scalars are planned on the host
    std::vector<double> radius(rows), anis(rows), axes(3 * rows), m0(3 * rows), loc(3 * rows);
    std::vector<int64_t> seeds(E);
    std::vector<double> pm[5];
    const double *pm_src[5] = {d->magnetisation_per_member, d->damping_per_member,
                               d->temperature_per_member, d->field_amplitude_per_member,
                               d->field_frequency_per_member};
    auto fetch = [&](void *dst, const void *src, size_t bytes) -> int {
        if (bytes == 0) return MAGPY_SUCCESS;
        if (dev) CUDA_TRY(cudaMemcpy(dst, src, bytes, cudaMemcpyDeviceToHost));
        else std::memcpy(dst, src, bytes);
        return MAGPY_SUCCESS;
    };
    int rc;
    if ((rc = fetch(radius.data(), d->radius, rows * sizeof(double)))) return rc;
    if ((rc = fetch(anis.data(), d->anisotropy, rows * sizeof(double)))) return rc;
    if ((rc = fetch(axes.data(), d->anisotropy_axis, 3 * rows * sizeof(double)))) return rc;
    if ((rc = fetch(m0.data(), d->magnetisation_direction, 3 * rows * sizeof(double)))) return rc;
    if ((rc = fetch(loc.data(), d->location, 3 * rows * sizeof(double)))) return rc;
    if ((rc = fetch(seeds.data(), d->seeds, E * sizeof(int64_t)))) return rc;
    for (int k = 0; k < 5; k++)
        if (pm_src[k]) {
            pm[k].resize(E);
            if ((rc = fetch(pm[k].data(), pm_src[k], E * sizeof(double)))) return rc;
        }
    if (!finite_all(radius.data(), rows) || !finite_all(anis.data(), rows) ||
        !finite_all(loc.data(), 3 * rows))
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "radius, anisotropy and location must be finite");

    // reduce each distinct (geometry, scalars) once
    using Key = std::tuple<int64_t, double, double, double, double, double>;
    std::map<Key, Reduced> cache;
    std::vector<const Reduced *> mem(E);
    std::vector<uint64_t> useeds(E);
    auto prev = cache.end();  // the previous member's entry (runs of equal keys skip the lookup)
    Key prev_key;
    for (int64_t e = 0; e < E; e++) {
        const double ms = pm[0].empty() ? d->magnetisation : pm[0][e];
        const double al = pm[1].empty() ? d->damping : pm[1][e];
        const double T = pm[2].empty() ? d->temperature : pm[2][e];
        const double H0 = pm[3].empty() ? d->field_amplitude : pm[3][e];
        const double f = pm[4].empty() ? d->field_frequency : pm[4][e];
        const int64_t gid = d->per_member_geometry ? e : 0;
        const Key key = std::make_tuple(gid, ms, al, T, H0, f);
        auto it = (prev != cache.end() && key == prev_key) ? prev : cache.find(key);
        if (it == cache.end()) {
            const int64_t r0 = gid * n;
            it = cache.emplace(key, reduce_physical(n, &radius[r0], &anis[r0], &axes[3 * r0],
                                                    &m0[3 * r0], &loc[3 * r0], ms, al, T,
                                                    d->time_step, d->end_time, d->field_shape,
                                                    H0, f)).first;
        }
        mem[e] = &it->second;
        useeds[e] = (uint64_t)seeds[e];
        prev = it;
        prev_key = key;
    }
    return make_plan(mem, useeds, d->renorm, d->interactions, d->use_implicit, d->eps,
                     d->max_iter, S, d->precision, d->noise, d->noise_per_member, dev, keep_traj,
                     st, out);
}

int magpy_ensemble_dynamics(const magpy_ensemble_desc *d, magpy_ensemble_out *o, void *stream)
{
    if (!d || !o) return fail(MAGPY_ERR_INVALID_ARGUMENT, "desc or out is NULL");
    cudaStream_t st = (cudaStream_t)stream;
    magpy_plan *plan = nullptr;
    int rc = plan_from_desc(d, o->mx != nullptr, st, &plan);
    if (rc) return rc;
    std::unique_ptr<magpy_plan> owner(plan);
    if ((rc = run_plan(plan, st))) return rc;
    return copy_out(plan, o->mx, o->my, o->mz, o->time, o->field, o->status, o->steps, st);
}

int magpy_plan_create(const magpy_ensemble_desc *desc, magpy_plan **plan, void *stream)
{
    return plan_from_desc(desc, true, (cudaStream_t)stream, plan);
}

int magpy_plan_run(magpy_plan *plan, void *stream)
{
    if (!plan) return fail(MAGPY_ERR_INVALID_ARGUMENT, "plan is NULL");
    return run_plan(plan, (cudaStream_t)stream);
}

int magpy_plan_device_outputs(magpy_plan *plan, double **mx, double **my, double **mz,
                              int32_t **status, int64_t **steps)
{
    if (!plan) return fail(MAGPY_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (mx) *mx = plan->p.mx;
    if (my) *my = plan->p.my;
    if (mz) *mz = plan->p.mz;
    if (status) *status = plan->p.status;
    if (steps) *steps = plan->p.steps;
    return MAGPY_SUCCESS;
}

int magpy_plan_copy_out(magpy_plan *plan, magpy_ensemble_out *o, void *stream)
{
    if (!plan || !o) return fail(MAGPY_ERR_INVALID_ARGUMENT, "plan or out is NULL");
    return copy_out(plan, o->mx, o->my, o->mz, o->time, o->field, o->status, o->steps,
                    (cudaStream_t)stream);
}

int magpy_plan_shape(const magpy_plan *plan, int64_t *n_members, int64_t *n_particles,
                     int64_t *n_samples, int64_t *max_steps)
{
    if (!plan) return fail(MAGPY_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (n_members) *n_members = plan->p.E;
    if (n_particles) *n_particles = plan->p.n;
    if (n_samples) *n_samples = plan->p.S;
    if (max_steps) *max_steps = plan->max_steps;
    return MAGPY_SUCCESS;
}

int magpy_plan_ensemble_magnetisation(magpy_plan *plan, int32_t direction, double *out,
                                      void *stream)
{
    if (!plan || !out) return fail(MAGPY_ERR_INVALID_ARGUMENT, "plan or out is NULL");
    if (direction < 0 || direction > 2)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "direction must be 0, 1 or 2");
    const DevPlan &p = plan->p;
    if (!p.mx) return fail(MAGPY_ERR_INVALID_ARGUMENT, "the plan keeps no trajectories");
    cudaStream_t st = (cudaStream_t)stream;
    const double *m = direction == 0 ? p.mx : direction == 1 ? p.my : p.mz;
    DBuf b;
    CUDA_TRY(pool_alloc(&b.p, (p.S > 0 ? p.S : 1) * sizeof(double)));
    cudaError_t err = launch_ensemble_mean(m, p.S, p.P, p.E, (double *)b.p, st);
    if (err != cudaSuccess) return fail(MAGPY_ERR_CUDA, cudaGetErrorString(err));
    CUDA_TRY(cudaMemcpyAsync(out, b.p, p.S * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return MAGPY_SUCCESS;
}

int magpy_plan_energy_dissipated(magpy_plan *plan, double start_time, double end_time,
                                 double *out, void *stream)
{
    if (!plan || !out) return fail(MAGPY_ERR_INVALID_ARGUMENT, "plan or out is NULL");
    const DevPlan &p = plan->p;
    if (!p.mz) return fail(MAGPY_ERR_INVALID_ARGUMENT, "the plan keeps no trajectories");
    if (p.E == 0 || p.S == 0) { *out = 0.0; return MAGPY_SUCCESS; }
    cudaStream_t st = (cudaStream_t)stream;
    // the mask (time >= start) & (time <= end) selects a contiguous range of
    // the monotone sample times of member 0
    const double *t = plan->times.data();
    int64_t lo = 0, hi = p.S - 1;
    while (lo < p.S && !std::isnan(start_time) && !(t[lo] >= start_time)) lo++;
    while (hi >= 0 && !std::isnan(end_time) && !(t[hi] <= end_time)) hi--;
    if (hi <= lo) { *out = 0.0; return MAGPY_SUCCESS; }
    DBuf b;
    CUDA_TRY(pool_alloc(&b.p, (2 * p.S + 1) * sizeof(double)));
    double *M = (double *)b.p, *H = M + p.S, *res = H + p.S;
    cudaError_t err = launch_ensemble_mean(p.mz, p.S, p.P, p.E, M, st);
    if (err != cudaSuccess) return fail(MAGPY_ERR_CUDA, cudaGetErrorString(err));
    CUDA_TRY(cudaMemcpyAsync(H, plan->fields.data(), p.S * sizeof(double), cudaMemcpyHostToDevice,
                             st));
    err = launch_trapezoid(M, H, lo, hi, MU0, res, st);
    if (err != cudaSuccess) return fail(MAGPY_ERR_CUDA, cudaGetErrorString(err));
    CUDA_TRY(cudaMemcpyAsync(out, res, sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return MAGPY_SUCCESS;
}

int magpy_plan_set_launch(magpy_plan *plan, int32_t block_warps, int32_t members_per_warp)
{
    if (!plan) return fail(MAGPY_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (block_warps < 1 || block_warps > 32 || members_per_warp < 0 ||
        (members_per_warp > 32 && members_per_warp != 40 && members_per_warp != 48 &&
         members_per_warp != 64))
        return fail(MAGPY_ERR_INVALID_ARGUMENT,
                    "block_warps in 1..32, members_per_warp in 0..32, 40, 48 or 64");
    plan->p.block_warps = block_warps;
    plan->p.members_per_warp = members_per_warp;
    return MAGPY_SUCCESS;
}

int magpy_plan_set_wait_limit(magpy_plan *plan, int64_t polls)
{
    if (!plan) return fail(MAGPY_ERR_INVALID_ARGUMENT, "plan is NULL");
    if (polls < 0 || polls > (int64_t)UINT32_MAX)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "polls must be in 0..2^32-1");
    plan->p.wait_limit = (uint32_t)polls;
    return MAGPY_SUCCESS;
}

int magpy_plan_destroy(magpy_plan *plan)
{
    delete plan;
    return MAGPY_SUCCESS;
}

int magpy_dom_dynamics(const magpy_dom_desc *d, double *mz, double *field, double *time,
                       int32_t *status, int64_t *steps, void *stream)
{
    if (!d) return fail(MAGPY_ERR_INVALID_ARGUMENT, "descriptor is NULL");
    const int64_t E = d->n_particles;
    if (E < 0) return fail(MAGPY_ERR_INVALID_ARGUMENT, "n_particles must be >= 0");
    if (E > 0 && (!d->volume || !d->anisotropy || !d->temperature || !d->magnetisation ||
                  !d->damping || !d->initial_probabilities || !d->field_amplitude ||
                  !d->field_frequency))
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "every per-particle array is required");
    if (!(d->time_step > 0) || !std::isfinite(d->time_step) || !(d->end_time > 0) ||
        !std::isfinite(d->end_time))
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "time_step and end_time must be > 0, finite");
    if (d->field_shape < 0 || d->field_shape > 3)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "field_shape must be 0..3");
    if (d->field_shape == MAGPY_FIELD_SQUARE_FOURIER &&
        (d->field_n_components < 1 || d->field_n_components > 100000))
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "field_n_components must be in 1..100000");
    int64_t N;
    if (d->max_samples == -1) {
        // simulation.cpp:710-712: int(end_time / time_step) + 1
        const double r = d->end_time / d->time_step;
        if (!(r < 2147483646.0))
            return fail(MAGPY_ERR_INVALID_ARGUMENT, "max_samples = -1 needs end/dt < 2^31 - 1");
        N = (int64_t)(int)r + 1;
    } else if (d->max_samples >= 1 && d->max_samples <= 2147483647) {
        N = d->max_samples;  // the reference passes it as an int
    } else {
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "max_samples must be -1 or 1 .. 2^31-1");
    }
    if (d->max_steps < 0) return fail(MAGPY_ERR_INVALID_ARGUMENT, "max_steps must be >= 0");
    if (E == 0) return MAGPY_SUCCESS;
    if (!mz && !field && !time && !status && !steps) return MAGPY_SUCCESS;

    std::vector<DomMember> hm(E);
    std::vector<std::pair<double, int64_t>> key(E);
    for (int64_t e = 0; e < E; e++) {
        DomMember &m = hm[e];
        m.v = d->volume[e];
        m.k = d->anisotropy[e];
        m.T = d->temperature[e];
        m.ms = d->magnetisation[e];
        m.alpha = d->damping[e];
        m.hk = 2.0 * m.k / MU0 / m.ms;     // core.pyx:226
        m.h = d->field_amplitude[e] / m.hk; // core.pyx:227
        m.f = d->field_frequency[e];
        m.p0 = d->initial_probabilities[2 * e];
        m.p1 = d->initial_probabilities[2 * e + 1];
        // launch order: by the zero-field relaxation rate, the main driver of
        // the step count, fastest (most steps) first, so that a warp's
        // particles take similar step counts and the heavy warps start first
        const double sigma = m.k * m.v / KB / m.T;
        const double taun = m.v * m.ms * (1 + m.alpha * m.alpha) / 2.0 / GYROMAG / m.alpha / KB /
                            m.T;
        const double lr = -sigma + 1.5 * std::log(sigma) - std::log(taun * std::sqrt(M_PI));
        key[e] = {std::isfinite(lr) ? -lr : 1e300, e};
    }
    std::sort(key.begin(), key.end());
    std::vector<int64_t> order(E);
    for (int64_t e = 0; e < E; e++) order[e] = key[e].second;

    cudaStream_t st = (cudaStream_t)stream;
    const size_t EN = (size_t)E * (size_t)N;
    DBuf bm, bo, bz, bf, bt, bs, bk;
    CUDA_TRY(pool_alloc(&bm.p, E * sizeof(DomMember)));
    CUDA_TRY(pool_alloc(&bo.p, E * sizeof(int64_t)));
    CUDA_TRY(pool_alloc(&bz.p, EN * sizeof(double)));
    CUDA_TRY(pool_alloc(&bf.p, EN * sizeof(double)));
    CUDA_TRY(pool_alloc(&bt.p, EN * sizeof(double)));
    CUDA_TRY(pool_alloc(&bs.p, E * sizeof(int32_t)));
    CUDA_TRY(pool_alloc(&bk.p, E * sizeof(int64_t)));
    CUDA_TRY(cudaMemcpyAsync(bm.p, hm.data(), E * sizeof(DomMember), cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemcpyAsync(bo.p, order.data(), E * sizeof(int64_t), cudaMemcpyHostToDevice,
                             st));
    DomArgs a;
    a.E = E;
    a.N = N;
    a.members = (const DomMember *)bm.p;
    a.order = (const int64_t *)bo.p;
    a.shape = d->field_shape;
    a.ncomp = d->field_n_components;
    a.time_step = d->time_step;
    a.end_time = d->end_time;
    a.sampling_time = d->end_time / (double)(N - 1);  // simulation.cpp:713
    a.max_steps = d->max_steps > 0 ? d->max_steps : 100000000;
    a.mz = (double *)bz.p;
    a.field = (double *)bf.p;
    a.time = (double *)bt.p;
    a.status = (int32_t *)bs.p;
    a.steps = (int64_t *)bk.p;
    CUDA_TRY(launch_dom(a, st));
    const cudaMemcpyKind down = cudaMemcpyDeviceToHost;
    if (mz) CUDA_TRY(cudaMemcpyAsync(mz, bz.p, EN * sizeof(double), down, st));
    if (field) CUDA_TRY(cudaMemcpyAsync(field, bf.p, EN * sizeof(double), down, st));
    if (time) CUDA_TRY(cudaMemcpyAsync(time, bt.p, EN * sizeof(double), down, st));
    if (status) CUDA_TRY(cudaMemcpyAsync(status, bs.p, E * sizeof(int32_t), down, st));
    if (steps) CUDA_TRY(cudaMemcpyAsync(steps, bk.p, E * sizeof(int64_t), down, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return MAGPY_SUCCESS;
}

int magpy_generate_clusters(const magpy_geometry_desc *d, double *radius, double *axes,
                            double *m0, double *location, int32_t *status, void *stream)
{
    if (!d) return fail(MAGPY_ERR_INVALID_ARGUMENT, "descriptor is NULL");
    const int64_t E = d->n_members, n = d->n_particles;
    if (E < 0 || n < 1 || n > 1024)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "need n_members >= 0 and 1 <= n_particles <= 1024");
    if (d->layout != MAGPY_LAYOUT_SPHERE && d->layout != MAGPY_LAYOUT_CHAIN)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "layout must be SPHERE or CHAIN");
    if (!(d->median_radius > 0) || !(d->sigma_log_radius >= 0) || !(d->spacing >= 0) ||
        !std::isfinite(d->median_radius) || !std::isfinite(d->sigma_log_radius) ||
        !std::isfinite(d->spacing))
        return fail(MAGPY_ERR_INVALID_ARGUMENT,
                    "median_radius > 0, sigma_log_radius >= 0, spacing >= 0, all finite");
    if (d->layout == MAGPY_LAYOUT_SPHERE &&
        !(d->packing_fraction > 0 && d->packing_fraction <= 0.6))
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "packing_fraction must be in (0, 0.6]");
    if (d->max_rounds < 0 || d->max_rounds > 16384)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "max_rounds must be in 0..16384");
    if (E == 0) return MAGPY_SUCCESS;
    if (!d->seeds || !radius || !axes || !m0 || !location)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "seeds and the four outputs are required");
    cudaStream_t st = (cudaStream_t)stream;
    const bool dev = d->buffers_on_device != 0;
    const size_t P = (size_t)E * n;
    DBuf bs, br, ba, bm, bl, bst;
    GeoArgs a;
    a.E = E;
    a.n = (int32_t)n;
    a.layout = d->layout;
    a.moments_random = d->moments ? 1 : 0;
    a.median_radius = d->median_radius;
    a.sigma = d->sigma_log_radius;
    a.spacing = d->spacing;
    a.packing = d->packing_fraction;
    a.max_rounds = d->max_rounds > 0 ? d->max_rounds : 4096;
    if (dev) {
        a.seeds = d->seeds;
        a.radius = radius; a.axes = axes; a.m0 = m0; a.location = location;
    } else {
        CUDA_TRY(pool_alloc(&bs.p, E * sizeof(int64_t)));
        CUDA_TRY(pool_alloc(&br.p, P * sizeof(double)));
        CUDA_TRY(pool_alloc(&ba.p, 3 * P * sizeof(double)));
        CUDA_TRY(pool_alloc(&bm.p, 3 * P * sizeof(double)));
        CUDA_TRY(pool_alloc(&bl.p, 3 * P * sizeof(double)));
        CUDA_TRY(cudaMemcpyAsync(bs.p, d->seeds, E * sizeof(int64_t), cudaMemcpyHostToDevice, st));
        a.seeds = (const int64_t *)bs.p;
        a.radius = (double *)br.p; a.axes = (double *)ba.p; a.m0 = (double *)bm.p;
        a.location = (double *)bl.p;
    }
    if (dev && status) {
        a.status = status;
    } else {
        CUDA_TRY(pool_alloc(&bst.p, E * sizeof(int32_t)));
        a.status = (int32_t *)bst.p;
    }
    cudaError_t err = launch_geometry(a, st);
    if (err != cudaSuccess) return fail(MAGPY_ERR_CUDA, cudaGetErrorString(err));
    if (!dev) {
        const cudaMemcpyKind down = cudaMemcpyDeviceToHost;
        CUDA_TRY(cudaMemcpyAsync(radius, br.p, P * sizeof(double), down, st));
        CUDA_TRY(cudaMemcpyAsync(axes, ba.p, 3 * P * sizeof(double), down, st));
        CUDA_TRY(cudaMemcpyAsync(m0, bm.p, 3 * P * sizeof(double), down, st));
        CUDA_TRY(cudaMemcpyAsync(location, bl.p, 3 * P * sizeof(double), down, st));
    }
    if (status && !(dev && status == a.status))
        CUDA_TRY(cudaMemcpyAsync(status, a.status, E * sizeof(int32_t),
                                 dev ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return MAGPY_SUCCESS;
}

// One raw array of doubles per file, as io::write_array (include/io.hpp:13-27).
static int write_doubles(const std::string &name, const double *a, int64_t n)
{
    FILE *f = std::fopen(name.c_str(), "wb");
    if (!f) return fail(MAGPY_ERR_IO, "cannot open " + name + " for writing");
    const size_t w = n > 0 ? std::fwrite(a, sizeof(double), (size_t)n, f) : 0;
    const bool ok = (std::fclose(f) == 0) && w == (size_t)(n > 0 ? n : 0);
    return ok ? MAGPY_SUCCESS : fail(MAGPY_ERR_IO, "short write to " + name);
}

int magpy_save_results(const char *prefix, const double *mx, const double *my, const double *mz,
                       const double *field, const double *time, int64_t n_samples)
{
    if (!prefix || n_samples < 0 || (n_samples > 0 && (!mx || !my || !mz || !field || !time)))
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "prefix and five arrays of n_samples >= 0");
    const std::string p(prefix);
    const std::pair<const char *, const double *> parts[5] = {
        {".mx", mx}, {".my", my}, {".mz", mz}, {".field", field}, {".time", time}};
    for (const auto &pt : parts) {
        const int rc = write_doubles(p + pt.first, pt.second, n_samples);
        if (rc != MAGPY_SUCCESS) return rc;
    }
    return MAGPY_SUCCESS;
}

int magpy_plan_save_results(magpy_plan *plan, const char *prefix, int64_t member_begin,
                            int64_t member_end, void *stream)
{
    if (!plan || !prefix) return fail(MAGPY_ERR_INVALID_ARGUMENT, "plan or prefix is NULL");
    const DevPlan &p = plan->p;
    if (!p.mx) return fail(MAGPY_ERR_INVALID_ARGUMENT, "the plan keeps no trajectories");
    if (member_begin < 0 || member_end > p.E || member_begin > member_end)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "member range outside [0, n_members]");
    const int64_t n = p.n, S = p.S, cols = (member_end - member_begin) * n;
    if (cols == 0 || S == 0) return MAGPY_SUCCESS;
    cudaStream_t st = (cudaStream_t)stream;
    // the members' columns of the [S][P] trajectories, one strided copy per component
    std::vector<double> host((size_t)3 * S * cols);
    const double *src[3] = {p.mx, p.my, p.mz};
    for (int c = 0; c < 3; c++)
        CUDA_TRY(cudaMemcpy2DAsync(host.data() + (size_t)c * S * cols, cols * sizeof(double),
                                   src[c] + member_begin * n, p.P * sizeof(double),
                                   cols * sizeof(double), S, cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    std::vector<double> m3((size_t)3 * S);
    for (int64_t e = member_begin; e < member_end; e++) {
        const double *tm = plan->times.data() + e * S, *fd = plan->fields.data() + e * S;
        for (int64_t i = 0; i < n; i++) {
            const int64_t col = (e - member_begin) * n + i;
            for (int c = 0; c < 3; c++)
                for (int64_t s = 0; s < S; s++)
                    m3[c * S + s] = host[((size_t)c * S + s) * cols + col];
            const std::string name = std::string(prefix) + "_" + std::to_string(e) + "_" +
                                     std::to_string(i);
            const int rc = magpy_save_results(name.c_str(), m3.data(), m3.data() + S,
                                              m3.data() + 2 * S, fd, tm, S);
            if (rc != MAGPY_SUCCESS) return rc;
        }
    }
    return MAGPY_SUCCESS;
}

// Reorder [S][n] sample-major device output into the reference's [n][S].
static void to_particle_major(const std::vector<double> &src, int64_t n, int64_t S, double *dst)
{
    for (int64_t q = 0; q < n; q++)
        for (int64_t s = 0; s < S; s++) dst[q * S + s] = src[s * n + q];
}

int magpy_full_dynamics(int64_t n_particles, const double *radius, const double *anisotropy,
                        const double *anisotropy_axis, const double *magnetisation_direction,
                        const double *location, double magnetisation, double damping,
                        double temperature, int32_t renorm, int32_t interactions,
                        int32_t use_implicit, double eps, double time_step, double end_time,
                        int64_t max_samples, int64_t seed, int32_t field_shape,
                        double field_amplitude, double field_frequency, const double *noise,
                        int64_t noise_len, int32_t precision, double *mx, double *my,
                        double *mz, double *field, double *time, int32_t *status)
{
    if (n_particles < 1 || max_samples < 1)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "need n_particles >= 1 and max_samples >= 1");
    magpy_ensemble_desc d{};
    d.n_members = 1;
    d.n_particles = n_particles;
    d.radius = radius;
    d.anisotropy = anisotropy;
    d.anisotropy_axis = anisotropy_axis;
    d.magnetisation_direction = magnetisation_direction;
    d.location = location;
    d.magnetisation = magnetisation;
    d.damping = damping;
    d.temperature = temperature;
    d.field_amplitude = field_amplitude;
    d.field_frequency = field_frequency;
    d.field_shape = field_shape;
    d.renorm = renorm;
    d.interactions = interactions;
    d.use_implicit = use_implicit;
    d.eps = eps;
    d.max_iter = 1000;
    d.time_step = time_step;
    d.end_time = end_time;
    d.max_samples = max_samples;
    d.seeds = &seed;
    d.noise = noise;
    d.noise_per_member = noise_len;
    d.precision = precision;
    const int64_t tr = n_particles * max_samples;
    std::vector<double> bx(tr), by(tr), bz(tr);
    int32_t st = 0;
    magpy_ensemble_out o{bx.data(), by.data(), bz.data(), time, field, &st, nullptr};
    int rc = magpy_ensemble_dynamics(&d, &o, nullptr);
    if (rc) return rc;
    to_particle_major(bx, n_particles, max_samples, mx);
    to_particle_major(by, n_particles, max_samples, my);
    to_particle_major(bz, n_particles, max_samples, mz);
    if (status) *status = st;
    return MAGPY_SUCCESS;
}

int magpy_full_dynamics_reduced(
    int64_t n, const double *thermal_field_strengths, const double *reduced_anisotropy_constants,
    const double *reduced_particle_volumes, const double *anisotropy_unit_axes,
    const double *initial_magnetisations, const double *interparticle_unit_distances,
    const double *interparticle_reduced_distance_magnitudes, int32_t field_shape,
    double reduced_field_amplitude, double reduced_field_frequency, double average_anisotropy,
    double average_volume, double damping_constant, double saturation_magnetisation,
    double time_step, double end_time, const double *noise, int64_t noise_len, int32_t renorm,
    int32_t interactions, int32_t use_implicit, double eps, int64_t max_iter,
    int64_t max_samples, int32_t precision, double *mx, double *my, double *mz, double *field,
    double *time, int32_t *status, int64_t *steps)
{
    if (n < 1 || n > 1024 || max_samples < 1)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "need 1 <= n <= 1024 and max_samples >= 1");
    if (field_shape < 0 || field_shape > 2)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "bad field_shape");
    Reduced R;
    R.n = n;
    R.sr.assign(thermal_field_strengths, thermal_field_strengths + n);
    R.k_red.assign(reduced_anisotropy_constants, reduced_anisotropy_constants + n);
    R.v_red.assign(reduced_particle_volumes, reduced_particle_volumes + n);
    R.axes.assign(anisotropy_unit_axes, anisotropy_unit_axes + 3 * n);
    R.m0.assign(initial_magnetisations, initial_magnetisations + 3 * n);
    R.unit.assign(interparticle_unit_distances, interparticle_unit_distances + 3 * n * n);
    R.dist_mag.assign(interparticle_reduced_distance_magnitudes,
                      interparticle_reduced_distance_magnitudes + n * n);
    R.k_av = average_anisotropy;
    R.v_av = average_volume;
    R.alpha = damping_constant;
    R.ms = saturation_magnetisation;
    R.dt = time_step;
    R.end = end_time;
    R.happ = reduced_field_amplitude;
    R.fapp = reduced_field_frequency;
    R.shape = field_shape;
    std::vector<const Reduced *> mem{&R};
    std::vector<uint64_t> seeds{0};
    const int64_t tr = n * max_samples;
    std::vector<double> bx(tr), by(tr), bz(tr);
    int32_t st = 0;
    int64_t k = 0;
    magpy_plan *plan = nullptr;
    int rc = make_plan(mem, seeds, renorm, interactions, use_implicit, eps, max_iter, max_samples,
                       precision, noise, noise_len, false, true, nullptr, &plan);
    if (rc) return rc;
    std::unique_ptr<magpy_plan> owner(plan);
    if ((rc = run_plan(plan, nullptr))) return rc;
    if ((rc = copy_out(plan, bx.data(), by.data(), bz.data(), time, field, &st, &k, nullptr)))
        return rc;
    to_particle_major(bx, n, max_samples, mx);
    to_particle_major(by, n, max_samples, my);
    to_particle_major(bz, n, max_samples, mz);
    if (status) *status = st;
    if (steps) *steps = k;
    return MAGPY_SUCCESS;
}

int magpy_llg_components(int64_t n, const double *m, const double *h, const double *hj,
                         const double *axis, const double *alpha, const double *sr,
                         double *drift, double *diffusion, double *drift_jac,
                         double *diff_jac, double *anis)
{
    if (n < 0) return fail(MAGPY_ERR_INVALID_ARGUMENT, "n < 0");
    if (n == 0) return MAGPY_SUCCESS;
    // inputs m,h,hj,axis (3+3+9+3 per state), alpha, sr; outputs 3+9+9+27+3
    const size_t in_n = 18 * n + 2 * n, out_n = 51 * n;
    std::vector<double> hin(in_n, 0.0);
    auto put = [&](size_t off, const double *src, size_t cnt) {
        if (src) std::memcpy(&hin[off], src, cnt * sizeof(double));
    };
    put(0, m, 3 * n);
    put(3 * n, h, 3 * n);
    put(6 * n, hj, 9 * n);
    put(15 * n, axis, 3 * n);
    put(18 * n, alpha, n);
    put(19 * n, sr, n);
    DBuf bi, bo;
    CUDA_TRY(pool_alloc(&bi.p, in_n * sizeof(double)));
    CUDA_TRY(pool_alloc(&bo.p, out_n * sizeof(double)));
    CUDA_TRY(cudaMemcpy(bi.p, hin.data(), in_n * sizeof(double), cudaMemcpyHostToDevice));
    const double *di = (const double *)bi.p;
    double *dO = (double *)bo.p;
    cudaError_t le = launch_components(n, di, di + 3 * n, di + 6 * n, di + 15 * n, di + 18 * n,
                                       di + 19 * n, dO, dO + 3 * n, dO + 12 * n, dO + 21 * n,
                                       dO + 48 * n, nullptr);
    if (le != cudaSuccess) return fail(MAGPY_ERR_CUDA, cudaGetErrorString(le));
    std::vector<double> hout(out_n);
    CUDA_TRY(cudaMemcpy(hout.data(), bo.p, out_n * sizeof(double), cudaMemcpyDeviceToHost));
    auto get = [&](double *dst, size_t off, size_t cnt) {
        if (dst) std::memcpy(dst, &hout[off], cnt * sizeof(double));
    };
    get(drift, 0, 3 * n);
    get(diffusion, 3 * n, 9 * n);
    get(drift_jac, 12 * n, 9 * n);
    get(diff_jac, 21 * n, 27 * n);
    get(anis, 48 * n, 3 * n);
    return MAGPY_SUCCESS;
}

int magpy_wiener_increments(int64_t seed, int64_t n_particles, int64_t n_steps, double *out)
{
    if (n_particles < 1 || n_steps < 0 || !out)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "bad arguments");
    const size_t cnt = (size_t)n_steps * 3 * n_particles;
    if (cnt == 0) return MAGPY_SUCCESS;
    DBuf b;
    CUDA_TRY(pool_alloc(&b.p, cnt * sizeof(double)));
    cudaError_t le = launch_wiener((uint64_t)seed, n_particles, n_steps, (double *)b.p, nullptr);
    if (le != cudaSuccess) return fail(MAGPY_ERR_CUDA, cudaGetErrorString(le));
    CUDA_TRY(cudaMemcpy(out, b.p, cnt * sizeof(double), cudaMemcpyDeviceToHost));
    return MAGPY_SUCCESS;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Batches of uneven cluster sizes: one plan per group, one CUDA graph.
// ---------------------------------------------------------------------------
struct magpy_batch {
    std::vector<magpy_plan *> plans;
    std::vector<int32_t> precision, block_warps, members_per_warp;
    std::vector<double> tuned_ms;
    std::vector<cudaStream_t> streams;
    std::vector<cudaEvent_t> events;
    cudaStream_t capture = nullptr;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    ~magpy_batch()
    {
        if (exec) cudaGraphExecDestroy(exec);
        if (graph) cudaGraphDestroy(graph);
        for (auto e : events) cudaEventDestroy(e);
        for (auto s : streams) cudaStreamDestroy(s);
        if (capture) cudaStreamDestroy(capture);
        for (auto p : plans) delete p;
    }
};

namespace {

struct TuneKey {
    int64_t n, E;
    int32_t precision, interactions, per_member_geometry, use_implicit;
    bool operator<(const TuneKey &o) const
    {
        return std::tie(n, E, precision, interactions, per_member_geometry, use_implicit) <
               std::tie(o.n, o.E, o.precision, o.interactions, o.per_member_geometry,
                        o.use_implicit);
    }
};
std::mutex g_tune_mu;
std::map<TuneKey, std::tuple<int32_t, int32_t, int32_t, double>> g_tune_cache;

// Time one configuration of a group on a short window of its own ensemble.
int tune_time(const magpy_ensemble_desc &d0, int32_t precision, int32_t bw, int32_t mpw,
              cudaStream_t st, double *ms_per_step)
{
    magpy_ensemble_desc d = d0;
    d.precision = precision;
    d.max_samples = 2;
    d.noise = nullptr;  // timing only: the in-kernel generator stands in
    const int64_t window = 64;
    d.end_time = d.time_step * window;
    magpy_plan *plan = nullptr;
    int rc = plan_from_desc(&d, true, st, &plan);
    if (rc) return rc;
    std::unique_ptr<magpy_plan> owner(plan);
    plan->p.block_warps = bw;
    plan->p.members_per_warp = mpw;
    cudaEvent_t a, b;
    CUDA_TRY(cudaEventCreate(&a));
    CUDA_TRY(cudaEventCreate(&b));
    float best = 1e30f;
    for (int it = 0; it < 3 && rc == 0; it++) {
        cudaEventRecord(a, st);
        rc = run_plan(plan, st);
        cudaEventRecord(b, st);
        cudaEventSynchronize(b);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, a, b);
        if (it > 0) best = std::min(best, ms);  // the first run warms up
    }
    cudaEventDestroy(a);
    cudaEventDestroy(b);
    if (rc) return rc;
    *ms_per_step = (double)best / (double)std::max<int64_t>(plan->max_steps, 1);
    return MAGPY_SUCCESS;
}

}  // namespace

extern "C" int magpy_batch_create(const magpy_ensemble_desc *groups, int64_t n_groups,
                                  int32_t autotune, magpy_batch **out, void *stream)
{
    if (!groups || !out || n_groups < 1)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "need groups, n_groups >= 1 and an out pointer");
    cudaStream_t st = (cudaStream_t)stream;
    std::unique_ptr<magpy_batch> B(new magpy_batch());
    for (int64_t g = 0; g < n_groups; g++) {
        const magpy_ensemble_desc &d = groups[g];
        int32_t prec = d.precision, bw = 4, mpw = 0;
        double ms = 0.0;
        // the implicit solve has one kernel per precision: only its launch shape is tuned
        const bool mixed = !d.use_implicit && (d.precision == MAGPY_PRECISION_MIXED ||
                                               d.precision == MAGPY_PRECISION_MIXED_TC);
        if (autotune && d.n_members > 0 && !d.buffers_on_device) {
            const TuneKey key{d.n_particles, d.n_members, mixed ? -1 : d.precision,
                              d.interactions, d.per_member_geometry, d.use_implicit ? 1 : 0};
            bool cached = false;
            {
                std::lock_guard<std::mutex> lock(g_tune_mu);
                auto it = g_tune_cache.find(key);
                if (it != g_tune_cache.end()) {
                    std::tie(prec, bw, mpw, ms) = it->second;
                    cached = true;
                }
            }
            if (!cached) {
                std::vector<int32_t> precs{d.precision};
                if (mixed) {
                    precs = {MAGPY_PRECISION_MIXED};
                    if (d.interactions && !d.per_member_geometry &&
                        (tc_supported((int)d.n_particles) || tcc_supported((int)d.n_particles)))
                        precs.push_back(MAGPY_PRECISION_MIXED_TC);
                }
                // launch shapes of the warp-packed kernels: warps per CTA and
                // members per warp (full packing, a quarter of it, one)
                std::vector<std::pair<int32_t, int32_t>> shapes{{4, 0}};
                if (d.n_particles <= 32) {
                    const int32_t full = (int32_t)(32 / d.n_particles);
                    std::vector<int32_t> mpws{0};
                    if (full >= 4) mpws.push_back(full / 4);
                    if (full > 1) mpws.push_back(1);
                    shapes.clear();
                    for (int32_t w : {1, 2, 4, 8})
                        for (int32_t m : mpws) shapes.push_back({w, m});
                }
                // clusters of more than 32 particles in mixed precision: 1, 2
                // or 4 members per CTA (members sharing a cluster)
                std::vector<std::pair<int32_t, int32_t>> big{{4, 0}};
                if (d.n_particles > 32 && !d.per_member_geometry) big = {{4, 0}, {4, 2}, {4, 4}};
                // tensor cores: clusters of more than 64 particles run 64 or
                // 32 members per thread-block cluster (members_per_warp 0 / 32)
                std::vector<std::pair<int32_t, int32_t>> tcs{{4, 0}};
                if (tcc_supported((int)d.n_particles)) tcs = {{4, 64}, {4, 48}, {4, 40}, {4, 32}};
                double best = 1e30;
                for (int32_t pc : precs)
                    for (auto sh : (pc == MAGPY_PRECISION_MIXED_TC
                                        ? tcs
                                        : (pc == MAGPY_PRECISION_MIXED && d.n_particles > 32)
                                              ? big
                                              : shapes)) {
                        double t = 0.0;
                        int rc = tune_time(d, pc, sh.first, sh.second, st, &t);
                        if (rc == MAGPY_ERR_UNSUPPORTED) continue;  // e.g. parameters differ
                        if (rc) return rc;
                        if (t < best) { best = t; prec = pc; bw = sh.first; mpw = sh.second; }
                    }
                ms = best;
                std::lock_guard<std::mutex> lock(g_tune_mu);
                g_tune_cache[key] = std::make_tuple(prec, bw, mpw, ms);
            }
        }
        magpy_ensemble_desc dd = d;
        dd.precision = prec;
        magpy_plan *plan = nullptr;
        int rc = plan_from_desc(&dd, true, st, &plan);
        if (rc) return rc;
        plan->p.block_warps = bw;
        plan->p.members_per_warp = mpw;
        B->plans.push_back(plan);
        B->precision.push_back(prec);
        B->block_warps.push_back(bw);
        B->members_per_warp.push_back(mpw);
        B->tuned_ms.push_back(ms);
    }
    // one graph: fork from the capture stream into a stream per group, join back.
    // The groups' streams get scheduling priorities by the group's time alone,
    // longest first (the graph runs with its nodes' priorities), so that the
    // group on the critical path takes its SMs before the shorter ones fill
    // the rest.
    CUDA_TRY(cudaStreamCreateWithFlags(&B->capture, cudaStreamNonBlocking));
    cudaEvent_t fork;
    CUDA_TRY(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming));
    B->events.push_back(fork);
    int least_prio = 0, greatest_prio = 0;
    CUDA_TRY(cudaDeviceGetStreamPriorityRange(&least_prio, &greatest_prio));
    std::vector<int64_t> by_time(n_groups);
    for (int64_t g = 0; g < n_groups; g++) by_time[g] = g;
    std::stable_sort(by_time.begin(), by_time.end(), [&](int64_t a, int64_t b) {
        return B->tuned_ms[a] > B->tuned_ms[b];
    });
    std::vector<int> prio(n_groups, least_prio);
    for (int64_t r = 0; r < n_groups; r++)  // greatest_prio is numerically the lowest
        prio[by_time[r]] = std::min(least_prio, greatest_prio + (int)r);
    for (int64_t g = 0; g < n_groups; g++) {
        cudaStream_t s;
        cudaEvent_t e;
        CUDA_TRY(cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, prio[g]));
        CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        B->streams.push_back(s);
        B->events.push_back(e);
    }
    // capture every group's launch as a parallel branch of one graph
    auto capture = [&]() -> int {
        if (B->exec) { cudaGraphExecDestroy(B->exec); B->exec = nullptr; }
        if (B->graph) { cudaGraphDestroy(B->graph); B->graph = nullptr; }
        CUDA_TRY(cudaStreamBeginCapture(B->capture, cudaStreamCaptureModeThreadLocal));
        int rc = MAGPY_SUCCESS;
        cudaEventRecord(fork, B->capture);
        for (int64_t g = 0; g < n_groups && rc == MAGPY_SUCCESS; g++) {
            cudaStreamWaitEvent(B->streams[g], fork, 0);
            rc = run_plan(B->plans[g], B->streams[g]);
            cudaEventRecord(B->events[g + 1], B->streams[g]);
            cudaStreamWaitEvent(B->capture, B->events[g + 1], 0);
        }
        cudaGraph_t graph = nullptr;
        cudaError_t ce = cudaStreamEndCapture(B->capture, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        if (ce != cudaSuccess)
            return fail(MAGPY_ERR_CUDA, std::string("graph capture: ") + cudaGetErrorString(ce));
        B->graph = graph;
        CUDA_TRY(cudaGraphInstantiate(&B->exec, B->graph, cudaGraphInstantiateFlagUseNodePriority));
        return MAGPY_SUCCESS;
    };
    int rc = capture();
    if (rc) return rc;
    // Groups on the cluster tensor-core kernel: members per cluster decide
    // how many SMs the group holds, and so how much room the groups running
    // beside it get; the count is chosen by timing the whole graph.
    if (autotune) {
        cudaEvent_t a, b;
        CUDA_TRY(cudaEventCreate(&a));
        CUDA_TRY(cudaEventCreate(&b));
        auto time_graph = [&](float *ms) -> int {
            float best = 1e30f;
            for (int it = 0; it < 3; it++) {
                CUDA_TRY(cudaEventRecord(a, st));
                CUDA_TRY(cudaGraphLaunch(B->exec, st));
                CUDA_TRY(cudaEventRecord(b, st));
                CUDA_TRY(cudaEventSynchronize(b));
                float t = 0.f;
                cudaEventElapsedTime(&t, a, b);
                if (it > 0) best = std::min(best, t);  // the first launch warms up
            }
            *ms = best;
            return MAGPY_SUCCESS;
        };
        for (int64_t g = 0; g < n_groups && rc == MAGPY_SUCCESS; g++) {
            magpy_plan *pl = B->plans[g];
            if (B->precision[g] != MAGPY_PRECISION_MIXED_TC || pl->p.use_implicit ||
                !tcc_supported(pl->p.n) || tc_supported(pl->p.n))
                continue;
            int32_t best_nb = B->members_per_warp[g];
            float best_ms = 1e30f;
            for (int32_t nb : {64, 48, 40, 32}) {
                pl->p.members_per_warp = nb;
                if (pl->tcc_last_nb != nb) {  // no memset node in the captured graph
                    CUDA_TRY(cudaMemsetAsync(pl->tcc_b, 0, pl->tcc_b_bytes, st));
                    pl->tcc_last_nb = nb;
                }
                float ms = 0.f;
                if ((rc = capture()) || (rc = time_graph(&ms))) break;
                if (ms < best_ms) { best_ms = ms; best_nb = nb; }
            }
            if (rc) break;
            pl->p.members_per_warp = best_nb;
            B->members_per_warp[g] = best_nb;
            if (pl->tcc_last_nb != best_nb) {
                CUDA_TRY(cudaMemsetAsync(pl->tcc_b, 0, pl->tcc_b_bytes, st));
                pl->tcc_last_nb = best_nb;
            }
            rc = capture();
        }
        // Groups that chose the CUDA-core kernel alone but could run on the
        // single-CTA tensor-core kernel: alone, a kernel spread over every SM
        // wins, while beside the other groups the SM time it takes counts;
        // the kernel is kept that makes the whole graph faster.
        float graph_ms = 0.f;
        if (rc == MAGPY_SUCCESS) rc = time_graph(&graph_ms);
        for (int64_t g = 0; g < n_groups && rc == MAGPY_SUCCESS; g++) {
            const magpy_ensemble_desc &d = groups[g];
            if (B->precision[g] != MAGPY_PRECISION_MIXED || d.use_implicit || !d.interactions ||
                d.per_member_geometry || d.buffers_on_device || d.n_members < 1 ||
                !tc_supported((int)d.n_particles))
                continue;
            magpy_ensemble_desc dd = d;
            dd.precision = MAGPY_PRECISION_MIXED_TC;
            magpy_plan *alt = nullptr;
            const int arc = plan_from_desc(&dd, true, st, &alt);
            if (arc == MAGPY_ERR_UNSUPPORTED) continue;  // e.g. parameters differ
            if (arc) { rc = arc; break; }
            alt->p.block_warps = 4;
            alt->p.members_per_warp = 0;
            magpy_plan *old = B->plans[g];
            B->plans[g] = alt;
            float ms = 0.f;
            if ((rc = capture()) == MAGPY_SUCCESS) rc = time_graph(&ms);
            if (rc == MAGPY_SUCCESS && ms < graph_ms) {
                graph_ms = ms;
                delete old;
                B->precision[g] = MAGPY_PRECISION_MIXED_TC;
                B->block_warps[g] = 4;
                B->members_per_warp[g] = 0;
            } else {
                B->plans[g] = old;
                delete alt;
            }
        }
        if (rc == MAGPY_SUCCESS) rc = capture();
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        CUDA_TRY(cudaStreamSynchronize(st));
        if (rc) return rc;
    }
    *out = B.release();
    return MAGPY_SUCCESS;
}

extern "C" int magpy_batch_run(magpy_batch *b, void *stream)
{
    if (!b || !b->exec) return fail(MAGPY_ERR_INVALID_ARGUMENT, "batch is NULL");
    CUDA_TRY(cudaGraphLaunch(b->exec, (cudaStream_t)stream));
    return MAGPY_SUCCESS;
}

extern "C" int magpy_batch_group_plan(magpy_batch *b, int64_t g, magpy_plan **plan)
{
    if (!b || !plan || g < 0 || g >= (int64_t)b->plans.size())
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "bad batch or group");
    *plan = b->plans[g];
    return MAGPY_SUCCESS;
}

extern "C" int magpy_batch_group_choice(const magpy_batch *b, int64_t g, int32_t *precision,
                                        int32_t *block_warps, int32_t *members_per_warp,
                                        double *ms_per_step)
{
    if (!b || g < 0 || g >= (int64_t)b->plans.size())
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "bad batch or group");
    if (precision) *precision = b->precision[g];
    if (block_warps) *block_warps = b->block_warps[g];
    if (members_per_warp) *members_per_warp = b->members_per_warp[g];
    if (ms_per_step) *ms_per_step = b->tuned_ms[g];
    return MAGPY_SUCCESS;
}

extern "C" int magpy_batch_destroy(magpy_batch *b)
{
    delete b;
    return MAGPY_SUCCESS;
}

// ---------------------------------------------------------------------------
// Pathwise adjoint of the Heun step (adjoint.cu).
// ---------------------------------------------------------------------------
struct magpy_adjoint {
    magpy_plan *plan = nullptr;
    magpy::AdjointArgs a;
    void *bufs[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    double Kbar = 0, alpha = 0, H0 = 0, H_k = 0, dt_red = 0, sq = 0, happ = 0, c = 0, Ms = 0;
    int64_t E = 0, S = 0;
    ~magpy_adjoint()
    {
        cudaDeviceSynchronize();
        for (void *b : bufs) magpy::pool_free(b, true);
        delete plan;
    }
};

extern "C" int magpy_adjoint_create(const magpy_ensemble_desc *d, int64_t checkpoint_every,
                                    magpy_adjoint **out, void *stream)
{
    using namespace magpy;
    if (!d || !out) return fail(MAGPY_ERR_INVALID_ARGUMENT, "desc or out is NULL");
    if (d->use_implicit || d->renorm || d->noise || d->buffers_on_device)
        return fail(MAGPY_ERR_UNSUPPORTED,
                    "the adjoint covers the Heun path without renormalisation, with the "
                    "in-kernel increments and host inputs");
    if (d->per_member_geometry || d->magnetisation_per_member || d->damping_per_member ||
        d->temperature_per_member || d->field_amplitude_per_member ||
        d->field_frequency_per_member)
        return fail(MAGPY_ERR_UNSUPPORTED, "the adjoint needs members that share all parameters");
    if (checkpoint_every < 1) return fail(MAGPY_ERR_INVALID_ARGUMENT, "checkpoint_every < 1");
    if (d->n_particles > 512)
        return fail(MAGPY_ERR_UNSUPPORTED, "the adjoint supports clusters of up to 512 particles");
    cudaStream_t st = (cudaStream_t)stream;
    magpy_ensemble_desc dd = *d;
    dd.precision = MAGPY_PRECISION_MIXED;
    std::unique_ptr<magpy_adjoint> A(new magpy_adjoint());
    int rc = plan_from_desc(&dd, true, st, &A->plan);
    if (rc) return rc;
    const int64_t n = d->n_particles, E = d->n_members, P = E * n;
    const Reduced R = reduce_physical(n, d->radius, d->anisotropy, d->anisotropy_axis,
                                      d->magnetisation_direction, d->location, d->magnetisation,
                                      d->damping, d->temperature, d->time_step, d->end_time,
                                      d->field_shape, d->field_amplitude, d->field_frequency);
    const int64_t K = A->plan->max_steps, C = checkpoint_every;
    A->Kbar = R.k_av;
    A->alpha = R.alpha;
    A->H0 = d->field_amplitude;
    A->H_k = R.H_k;
    A->dt_red = R.dt;
    A->sq = std::sqrt(R.dt);
    A->happ = R.happ;
    A->c = MU0 * R.ms * R.ms / 8.0 / M_PI / R.k_av;  // lib/field.cpp:212-215
    A->Ms = R.ms;
    A->E = E;
    A->S = d->max_samples;
    std::vector<double> vred(P);
    for (int64_t e = 0; e < E; e++)
        for (int64_t q = 0; q < n; q++) vred[e * n + q] = R.v_red[q];
    const size_t nck = (size_t)(K / C + 1);
    CUDA_TRY(pool_alloc(&A->bufs[0], P * sizeof(double)));
    CUDA_TRY(cudaMemcpy(A->bufs[0], vred.data(), P * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(pool_alloc(&A->bufs[1], nck * 6 * P * sizeof(float)));
    CUDA_TRY(pool_alloc(&A->bufs[2], (size_t)std::min(C, std::max<int64_t>(K, 1)) * 3 * P * sizeof(float)));
    CUDA_TRY(pool_alloc(&A->bufs[3], std::max<int64_t>(A->S, 1) * sizeof(double)));
    CUDA_TRY(pool_alloc(&A->bufs[4], 5 * sizeof(double)));
    if (R.shape != MAGPY_FIELD_CONSTANT && K > 0) {
        CUDA_TRY(pool_alloc(&A->bufs[5], 2 * K * sizeof(float)));
        cudaError_t err = mixed_fill_tables(A->plan->p, 0, K, R.dt, R.shape, 1.0, R.fapp,
                                            (float *)A->bufs[5], nullptr, st);
        if (err != cudaSuccess) return fail(MAGPY_ERR_CUDA, cudaGetErrorString(err));
    }
    AdjointArgs &a = A->a;
    a.p = A->plan->p;
    a.v_red = (const double *)A->bufs[0];
    a.ck = (float *)A->bufs[1];
    a.seg = (float *)A->bufs[2];
    a.wz = (const double *)A->bufs[3];
    a.grad = (double *)A->bufs[4];
    a.stab = (const float *)A->bufs[5];
    a.happ = (float)R.happ;
    a.dt = (float)R.dt;
    a.sq = (float)A->sq;
    a.alpha = (float)R.alpha;
    a.c = (float)A->c;
    a.K = K;
    a.C = (int)C;
    a.interactions = (d->interactions && n > 1) ? 1 : 0;
    if (a.interactions && !a.p.pr)
        return fail(MAGPY_ERR_CUDA, "pair table missing");
    CUDA_TRY(cudaStreamSynchronize(st));
    *out = A.release();
    return MAGPY_SUCCESS;
}

extern "C" int magpy_adjoint_forward(magpy_adjoint *A, void *stream)
{
    using namespace magpy;
    if (!A) return fail(MAGPY_ERR_INVALID_ARGUMENT, "adjoint is NULL");
    cudaError_t err = launch_adjoint(A->a, false, (cudaStream_t)stream);
    if (err != cudaSuccess) return fail(MAGPY_ERR_CUDA, cudaGetErrorString(err));
    CUDA_TRY(cudaStreamSynchronize((cudaStream_t)stream));
    return MAGPY_SUCCESS;
}

extern "C" int magpy_adjoint_plan(magpy_adjoint *A, magpy_plan **plan)
{
    if (!A || !plan) return fail(MAGPY_ERR_INVALID_ARGUMENT, "NULL argument");
    *plan = A->plan;
    return MAGPY_SUCCESS;
}

extern "C" int magpy_adjoint_backward(magpy_adjoint *A, const double *dJ_dM, double *grad_theta,
                                      double *grad_reduced, void *stream)
{
    using namespace magpy;
    if (!A || !dJ_dM) return fail(MAGPY_ERR_INVALID_ARGUMENT, "NULL argument");
    cudaStream_t st = (cudaStream_t)stream;
    std::vector<double> wz(std::max<int64_t>(A->S, 1));
    for (int64_t s = 0; s < A->S; s++) wz[s] = dJ_dM[s] * A->Ms / (double)A->E;
    CUDA_TRY(cudaMemcpyAsync((void *)A->a.wz, wz.data(), A->S * sizeof(double),
                             cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaMemsetAsync(A->a.grad, 0, 5 * sizeof(double), st));
    cudaError_t err = launch_adjoint(A->a, true, st);
    if (err != cudaSuccess) return fail(MAGPY_ERR_CUDA, cudaGetErrorString(err));
    double G[5];
    CUDA_TRY(cudaMemcpyAsync(G, A->a.grad, 5 * sizeof(double), cudaMemcpyDeviceToHost, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    if (grad_reduced)
        for (int i = 0; i < 5; i++) grad_reduced[i] = G[i];
    // chain rule from (dt, sqrt(dt) with the common sr scale, alpha, happ, c)
    // to (mean anisotropy K, damping alpha, field amplitude H0); see
    // lib/simulation.cpp:519-549 for how each reduced quantity is formed
    const double K = A->Kbar, al = A->alpha, sq = A->sq, dt = A->dt_red;
    const double Gh = G[0], Gw = G[1], Ga = G[2], Gha = G[3], Gc = G[4];
    const double q = 1 + al * al;
    if (grad_theta) {
        // dt_red and sqrt(dt) sr: dt scales with K, sqrt(dt) sr does not depend on K
        grad_theta[0] = Gh * dt / K - Gha * A->happ / K - Gc * A->c / K;
        grad_theta[1] = Gh * dt * (-2 * al / q) + Gw * sq * (0.5 / al - 2 * al / q) + Ga;
        grad_theta[2] = Gha / A->H_k;
    }
    return MAGPY_SUCCESS;
}

extern "C" int magpy_adjoint_destroy(magpy_adjoint *A)
{
    delete A;
    return MAGPY_SUCCESS;
}

extern "C" int magpy_dipolar_field_tc(int64_t n, int64_t n_members, double ms, double k_av,
                                      const double *v_reduced, const double *unit_distances,
                                      const double *distance_cubes, const double *mag,
                                      double *field)
{
    using namespace magpy;
    if (n < 2 || n_members < 0 || !(tc_supported((int)n) || tcc_supported((int)n)))
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "need 2 <= n <= 672 and n_members >= 0");
    if (!v_reduced || !unit_distances || !distance_cubes || !mag || !field)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "a pointer is NULL");
    if (n_members == 0) return MAGPY_SUCCESS;
    // pair tables as the integrator builds them (lib/field.cpp:212-225)
    const double pref = MU0 * ms * ms / 8.0 / M_PI / k_av;
    std::vector<double> pt(n * n, 0.0), rt(3 * n * n, 0.0);
    for (int64_t q = 0; q < n; q++)
        for (int64_t j = 0; j < n; j++) {
            if (j == q) continue;
            pt[j * n + q] = pref * (v_reduced[j] / distance_cubes[q * n + j]);
            for (int c = 0; c < 3; c++)
                rt[(c * n + j) * n + q] = unit_distances[(q * n + j) * 3 + c];
        }
    const size_t st_bytes = (size_t)n_members * n * 3 * sizeof(double);
    DBuf b_pt, b_rt, b_m, b_h, b_flag;
    CUDA_TRY(pool_alloc(&b_pt.p, pt.size() * sizeof(double)));
    CUDA_TRY(pool_alloc(&b_rt.p, rt.size() * sizeof(double)));
    CUDA_TRY(pool_alloc(&b_m.p, st_bytes));
    CUDA_TRY(pool_alloc(&b_h.p, st_bytes));
    CUDA_TRY(pool_alloc(&b_flag.p, sizeof(int)));
    CUDA_TRY(cudaMemcpy(b_pt.p, pt.data(), pt.size() * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(b_rt.p, rt.data(), rt.size() * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(b_m.p, mag, st_bytes, cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemset(b_flag.p, 0, sizeof(int)));
    cudaError_t err;
    DBuf b_d, b_b;
    if (tc_supported((int)n)) {
        __half *dhi = nullptr, *dlo = nullptr;
        err = tc_build_d((const double *)b_pt.p, (const double *)b_rt.p, (int)n, &dhi, &dlo,
                         nullptr);
        b_d.p = dhi;
        if (err != cudaSuccess) return fail(MAGPY_ERR_CUDA, cudaGetErrorString(err));
        // spare shared memory beyond the layout keeps every operand address
        // inside the CTA's allocation
        const size_t need = tc_smem_bytes((int)n), cap = 232448;
        const size_t slack = need + 65536 <= cap ? 65536 : cap - need;
        err = launch_tc_dipolar(dhi, dlo, (int)n, n_members, (const double *)b_m.p,
                                (double *)b_h.p, (int *)b_flag.p, slack, nullptr);
    } else {
        // clusters of more than 64 particles: the cluster kernel's tiles
        err = tcc_init((int)n, 32, nullptr);
        if (err != cudaSuccess) return fail(MAGPY_ERR_CUDA, cudaGetErrorString(err));
        CUDA_TRY(pool_alloc(&b_d.p, tcc_d_elems((int)n) * sizeof(__half)));
        const size_t bb = tcc_b_elems((int)n, n_members, 32) * sizeof(__half);
        CUDA_TRY(pool_alloc(&b_b.p, bb));
        CUDA_TRY(cudaMemset(b_b.p, 0, bb));
        err = tcc_build_d((const double *)b_pt.p, (const double *)b_rt.p, (int)n,
                          (__half *)b_d.p, nullptr);
        if (err == cudaSuccess)
            err = launch_tcc_dipolar((const __half *)b_d.p, (__half *)b_b.p, (int)n, n_members,
                                     (const double *)b_m.p, (double *)b_h.p, (int *)b_flag.p,
                                     nullptr);
    }
    if (err != cudaSuccess) return fail(MAGPY_ERR_CUDA, cudaGetErrorString(err));
    std::vector<double> h(n_members * n * 3);
    int flag = 0;
    CUDA_TRY(cudaMemcpy(h.data(), b_h.p, st_bytes, cudaMemcpyDeviceToHost));
    CUDA_TRY(cudaMemcpy(&flag, b_flag.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (flag) return fail(MAGPY_ERR_CUDA, "tensor-core completion wait timed out");
    for (size_t i = 0; i < h.size(); i++) field[i] += h[i];
    return MAGPY_SUCCESS;
}

// ---------------------------------------------------------------------------
// Entry point that allocates no device memory.
//
// Some callers cannot let a library call cudaMalloc or cudaFree: a host
// framework that owns the GPU's memory through its own pool and budget (a
// stray allocation outside that pool can push it into out-of-memory), and
// latency-critical loops, where cudaFree (and at times cudaMalloc) waits for
// the whole device to go idle.  For them, every device-side table the
// mixed-precision kernel needs -- member parameters, per-particle arrays,
// pair tables, sample schedule, field table -- is laid out in one static
// device array of MAGPY_NOALLOC_SCRATCH_BYTES that each GPU loading this
// library holds until the process exits.  Inputs and outputs stay the
// caller's (device pointers).
// ---------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_noalloc_scratch[MAGPY_NOALLOC_SCRATCH_BYTES];

namespace {
// Looks up the device address of the static scratch array with the caller's
// device (and context) current.  The name g_noalloc_scratch is only a
// host-side stand-in and must never be handed to a kernel.  The lookup is
// repeated on every call rather than cached: a cached address would outlive
// a cudaDeviceReset or belong to another context than the caller's current
// one.
int noalloc_scratch(unsigned char **out)
{
    void *ptr = nullptr;
    cudaError_t err = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
    if (err != cudaSuccess || !ptr)
        return fail(MAGPY_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") +
                                        cudaGetErrorString(err));
    *out = (unsigned char *)ptr;
    return MAGPY_SUCCESS;
}

size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
}  // namespace

namespace {
int noalloc_run(const magpy_ensemble_desc *d, magpy_ensemble_out *o, void *stream);
}

extern "C" int magpy_ensemble_dynamics_noalloc(const magpy_ensemble_desc *d,
                                               magpy_ensemble_out *o, void *stream)
{
    // host-side staging vectors may fail to allocate; no exception may cross
    // the C boundary
    try {
        return noalloc_run(d, o, stream);
    } catch (const std::bad_alloc &) {
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "host memory for staging the ensemble's tables "
                                                "could not be allocated");
    } catch (const std::exception &ex) {
        return fail(MAGPY_ERR_CUDA, std::string("no-allocation entry point: ") + ex.what());
    }
}

namespace {
int noalloc_run(const magpy_ensemble_desc *d, magpy_ensemble_out *o, void *stream)
{
    using namespace magpy;
    if (!d || !o) return fail(MAGPY_ERR_INVALID_ARGUMENT, "desc or out is NULL");
    if (!d->buffers_on_device)
        return fail(MAGPY_ERR_INVALID_ARGUMENT,
                    "the no-allocation entry point takes device buffers only "
                    "(buffers_on_device = 1)");
    if (d->precision != MAGPY_PRECISION_MIXED || d->use_implicit)
        return fail(MAGPY_ERR_UNSUPPORTED,
                    "the no-allocation entry point runs the mixed-precision Heun kernel only");
    const int64_t E = d->n_members, n = d->n_particles, S = d->max_samples;
    if (E < 1 || n < 1 || n > 1024 || S < 1)
        return fail(MAGPY_ERR_INVALID_ARGUMENT,
                    "need n_members >= 1, 1 <= n_particles <= 1024, max_samples >= 1");
    if (!d->radius || !d->anisotropy || !d->anisotropy_axis || !d->magnetisation_direction ||
        !d->location || !d->seeds)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "a required input pointer is NULL");
    if (d->field_shape < 0 || d->field_shape > 2)
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "bad field_shape");
    // the kernel writes the three trajectory components together
    if (!((o->mx && o->my && o->mz) || (!o->mx && !o->my && !o->mz)))
        return fail(MAGPY_ERR_INVALID_ARGUMENT,
                    "out->mx, out->my and out->mz must be all set or all NULL");
    // bounds by division first, so that no product below can wrap
    constexpr size_t LIMIT = (size_t)MAGPY_NOALLOC_SCRATCH_BYTES;
    if ((size_t)E > LIMIT / sizeof(MemberDev) || (size_t)S > LIMIT / sizeof(int64_t) ||
        (size_t)E * (size_t)n > LIMIT / (8 * sizeof(double)))
        return fail(MAGPY_ERR_INVALID_ARGUMENT,
                    "ensemble of " + std::to_string(E) + " members x " + std::to_string(n) +
                        " particles x " + std::to_string(S) +
                        " samples exceeds the no-allocation entry point's device scratch of " +
                        std::to_string(LIMIT) +
                        " bytes (MAGPY_NOALLOC_SCRATCH_BYTES); split the ensemble");
    const int64_t P = E * n;
    // the part of the footprint known before reading any input
    const size_t base_need = align256(E * sizeof(MemberDev)) + align256(8 * P * sizeof(double)) +
                             align256(E * sizeof(double)) + align256(S * sizeof(int64_t));
    if (base_need > (size_t)MAGPY_NOALLOC_SCRATCH_BYTES)
        return fail(MAGPY_ERR_INVALID_ARGUMENT,
                    "ensemble needs " + std::to_string(base_need) +
                        " bytes of device scratch; the no-allocation entry point has " +
                        std::to_string((size_t)MAGPY_NOALLOC_SCRATCH_BYTES) +
                        " (MAGPY_NOALLOC_SCRATCH_BYTES); split the ensemble");

    // read the inputs and reduce each distinct (geometry, scalars) once
    const int64_t rows = d->per_member_geometry ? E * n : n;
    std::vector<double> radius(rows), anis(rows), axes(3 * rows), m0(3 * rows), loc(3 * rows);
    std::vector<int64_t> seeds(E);
    std::vector<double> pm[5];
    const double *pm_src[5] = {d->magnetisation_per_member, d->damping_per_member,
                               d->temperature_per_member, d->field_amplitude_per_member,
                               d->field_frequency_per_member};
    cudaStream_t st = (cudaStream_t)stream;
    // the inputs are read on the caller's stream, after whatever work the
    // caller queued there to produce them
    const cudaMemcpyKind down = cudaMemcpyDeviceToHost;
    CUDA_TRY(cudaMemcpyAsync(radius.data(), d->radius, rows * sizeof(double), down, st));
    CUDA_TRY(cudaMemcpyAsync(anis.data(), d->anisotropy, rows * sizeof(double), down, st));
    CUDA_TRY(cudaMemcpyAsync(axes.data(), d->anisotropy_axis, 3 * rows * sizeof(double), down, st));
    CUDA_TRY(cudaMemcpyAsync(m0.data(), d->magnetisation_direction, 3 * rows * sizeof(double), down,
                             st));
    CUDA_TRY(cudaMemcpyAsync(loc.data(), d->location, 3 * rows * sizeof(double), down, st));
    CUDA_TRY(cudaMemcpyAsync(seeds.data(), d->seeds, E * sizeof(int64_t), down, st));
    for (int k = 0; k < 5; k++)
        if (pm_src[k]) {
            pm[k].resize(E);
            CUDA_TRY(cudaMemcpyAsync(pm[k].data(), pm_src[k], E * sizeof(double), down, st));
        }
    CUDA_TRY(cudaStreamSynchronize(st));
    if (!finite_all(radius.data(), rows) || !finite_all(anis.data(), rows) ||
        !finite_all(loc.data(), 3 * rows))
        return fail(MAGPY_ERR_INVALID_ARGUMENT, "radius, anisotropy and location must be finite");
    std::map<std::tuple<int64_t, double, double, double, double, double>, Reduced> cache;
    std::vector<const Reduced *> mem(E);
    for (int64_t e = 0; e < E; e++) {
        const double ms = pm[0].empty() ? d->magnetisation : pm[0][e];
        const double al = pm[1].empty() ? d->damping : pm[1][e];
        const double T = pm[2].empty() ? d->temperature : pm[2][e];
        const double H0 = pm[3].empty() ? d->field_amplitude : pm[3][e];
        const double f = pm[4].empty() ? d->field_frequency : pm[4][e];
        const int64_t gid = d->per_member_geometry ? e : 0;
        auto key = std::make_tuple(gid, ms, al, T, H0, f);
        auto it = cache.find(key);
        if (it == cache.end()) {
            const int64_t r0 = gid * n;
            it = cache.emplace(key, reduce_physical(n, &radius[r0], &anis[r0], &axes[3 * r0],
                                                    &m0[3 * r0], &loc[3 * r0], ms, al, T,
                                                    d->time_step, d->end_time, d->field_shape,
                                                    H0, f)).first;
        }
        mem[e] = &it->second;
    }
    // one schedule and one waveform per launch of the mixed kernel
    const Reduced &R0 = *mem[0];
    for (int64_t e = 1; e < E; e++)
        if (mem[e]->dt != R0.dt || mem[e]->end != R0.end || mem[e]->shape != R0.shape ||
            mem[e]->happ != R0.happ || mem[e]->fapp != R0.fapp)
            return fail(MAGPY_ERR_UNSUPPORTED,
                        "the mixed-precision kernel needs one time step and one applied-field "
                        "waveform per launch; split the ensemble");
    std::vector<int64_t> sched;
    int64_t K = 0;
    int rc = make_schedule(R0.dt, R0.end, S, sched, K);
    if (rc) return rc;
    if (d->noise && K * 3 * n > d->noise_per_member)
        return fail(MAGPY_ERR_NOISE_TOO_SHORT, "injected noise is shorter than the run");

    // clusters: one pair table per distinct reduced cluster
    std::map<const Reduced *, int64_t> cluster_of;
    for (int64_t e = 0; e < E; e++)
        if (!cluster_of.count(mem[e])) {
            const int64_t c = (int64_t)cluster_of.size();
            cluster_of[mem[e]] = c;
        }
    const bool pairs = d->interactions && n > 1;
    const int64_t clusters = pairs ? (int64_t)cluster_of.size() : 0;

    // scratch layout (256-byte aligned regions)
    size_t cur = 0;
    auto take = [&](size_t bytes) { size_t off = align256(cur); cur = off + bytes; return off; };
    const size_t o_mem = take(E * sizeof(MemberDev));
    const size_t o_m0 = take(3 * P * sizeof(double)), o_ax = take(3 * P * sizeof(double));
    const size_t o_k = take(P * sizeof(double)), o_sr = take(P * sizeof(double));
    const size_t o_scale = take(E * sizeof(double));
    const size_t o_pt = take(clusters * n * n * sizeof(double));
    const size_t o_rt = take(3 * clusters * n * n * sizeof(double));
    const size_t o_sched = take(S * sizeof(int64_t));
    const size_t staged = cur;  // everything above is built on the host
    const size_t o_pr = take(clusters * n * n * sizeof(float4));
    const bool table = R0.shape != MAGPY_FIELD_CONSTANT && K > 0;
    const size_t o_ftab = take(table ? 2 * K * sizeof(float) : 0);
    if (cur > (size_t)MAGPY_NOALLOC_SCRATCH_BYTES)
        return fail(MAGPY_ERR_INVALID_ARGUMENT,
                    "ensemble needs " + std::to_string(cur) +
                        " bytes of device scratch; the no-allocation entry point has " +
                        std::to_string((size_t)MAGPY_NOALLOC_SCRATCH_BYTES) +
                        " (MAGPY_NOALLOC_SCRATCH_BYTES); split the ensemble or shorten the run");

    std::vector<unsigned char> stage(staged, 0);
    MemberDev *md = (MemberDev *)&stage[o_mem];
    double *hm0 = (double *)&stage[o_m0], *hax = (double *)&stage[o_ax];
    double *hk = (double *)&stage[o_k], *hsr = (double *)&stage[o_sr];
    double *hscale = (double *)&stage[o_scale];
    double *hpt = (double *)&stage[o_pt], *hrt = (double *)&stage[o_rt];
    std::memcpy(&stage[o_sched], sched.data(), S * sizeof(int64_t));
    std::vector<double> times(E * S), fields(E * S);
    for (int64_t e = 0; e < E; e++) {
        const Reduced &R = *mem[e];
        MemberDev &m = md[e];
        m.dt = R.dt;
        m.sqrt_dt = std::sqrt(R.dt);
        m.alpha = R.alpha;
        m.happ = R.happ;
        m.fapp = R.fapp;
        m.Ah = std::sqrt(2 * 1000.0 * std::abs(std::log(R.dt)));
        m.eps = d->eps;
        m.max_iter = d->max_iter > 0 ? d->max_iter : 1000;
        m.pbase = e * n;
        m.noise_off = e * d->noise_per_member;
        m.noise_len = d->noise ? d->noise_per_member : 0;
        m.seed = (uint64_t)seeds[e];
        m.sched_off = 0;
        m.cluster_off = pairs ? cluster_of[&R] * n * n : 0;
        m.n = (int32_t)n;
        m.shape = R.shape;
        m.renorm = d->renorm;
        m.interactions = d->interactions;
        hscale[e] = R.out_scale;
        for (int64_t q = 0; q < n; q++) {
            const int64_t g = e * n + q;
            for (int c = 0; c < 3; c++) {
                hm0[c * P + g] = R.m0[3 * q + c];
                hax[c * P + g] = R.axes[3 * q + c];
            }
            hk[g] = R.k_red[q];
            hsr[g] = R.sr[q];
        }
        const double Ts = R.end / (double)(S - 1);
        for (int64_t s = 0; s < S; s++) {
            const double ts = (s == 0) ? 0.0 : (double)(uint32_t)s * Ts;
            times[e * S + s] = ts / R.time_factor;
            fields[e * S + s] = field_fn(R.shape, R.happ, R.fapp, ts) * R.H_k;
        }
    }
    if (pairs)
        for (auto &kv : cluster_of) {
            const Reduced &R = *kv.first;
            const int64_t off = kv.second * n * n;
            const double pref = MU0 * R.ms * R.ms / 8.0 / M_PI / R.k_av;
            for (int64_t q = 0; q < n; q++)
                for (int64_t j = 0; j < n; j++) {
                    if (j == q) continue;  // the diagonal stays zero (stage is zero-filled)
                    const double cube = std::pow(R.dist_mag[q * n + j], 3);
                    hpt[off + j * n + q] = pref * (R.v_red[j] / cube);
                    for (int c = 0; c < 3; c++)
                        hrt[3 * off + (c * n + j) * n + q] = R.unit[(q * n + j) * 3 + c];
                }
        }

    unsigned char *scratch = nullptr;
    if ((rc = noalloc_scratch(&scratch))) return rc;
    // every region the kernel reads is rewritten here, so nothing depends on
    // what an earlier call left in the array
    CUDA_TRY(cudaMemcpyAsync(scratch, stage.data(), staged, cudaMemcpyHostToDevice, st));
    DevPlan p;
    p.E = E;
    p.P = P;
    p.S = S;
    p.n = (int32_t)n;
    p.use_implicit = 0;
    p.members = (const MemberDev *)(scratch + o_mem);
    p.m0 = (const double *)(scratch + o_m0);
    p.axes = (const double *)(scratch + o_ax);
    p.k_red = (const double *)(scratch + o_k);
    p.sr = (const double *)(scratch + o_sr);
    p.out_scale = (const double *)(scratch + o_scale);
    p.pt = pairs ? (const double *)(scratch + o_pt) : nullptr;
    p.rt = pairs ? (const double *)(scratch + o_rt) : nullptr;
    p.sched = (const int64_t *)(scratch + o_sched);
    p.noise = d->noise;
    p.mx = o->mx;
    p.my = o->my;
    p.mz = o->mz;
    p.status = o->status;
    p.steps = o->steps;
    float *ftab = table ? (float *)(scratch + o_ftab) : nullptr;
    float4 *pr = pairs ? (float4 *)(scratch + o_pr) : nullptr;
    cudaError_t err = mixed_fill_tables(p, clusters, K, R0.dt, R0.shape, R0.happ, R0.fapp, ftab,
                                        pr, st);
    if (err != cudaSuccess)
        return fail(MAGPY_ERR_CUDA, std::string("table kernels: ") + cudaGetErrorString(err));
    p.ftab = ftab;
    p.pr = pr;
    err = launch_mixed(p, st);
    if (err != cudaSuccess)
        return fail(MAGPY_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(err));
    if (o->time)
        CUDA_TRY(cudaMemcpyAsync(o->time, times.data(), E * S * sizeof(double),
                                 cudaMemcpyHostToDevice, st));
    if (o->field)
        CUDA_TRY(cudaMemcpyAsync(o->field, fields.data(), E * S * sizeof(double),
                                 cudaMemcpyHostToDevice, st));
    CUDA_TRY(cudaStreamSynchronize(st));
    return MAGPY_SUCCESS;
}
}  // namespace
