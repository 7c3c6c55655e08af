// dom.cu -- two-state master equation ("discrete orientation model") for a
// batch of independent particles, one thread per particle.
//
// Path restated: magpy/core.pyx:205-278 simulate_dom ->
// simulation::dom_ensemble_dynamics (lib/simulation.cpp:659-767) ->
// integrator::rk45 (lib/integrators.cpp:152-251) -> dom::master_equation_with_update
// (lib/dom.cpp:79-97) -> dom::transition_matrix (lib/dom.cpp:33-59) and the
// 2x2 product of stochastic::master_equation (lib/stochastic_processes.cpp:18-25).
//
// FP64 throughout, compiled without FMA contraction, in the reference's
// operation order; per-particle constants of the transition matrix (sigma,
// tau_N, its sqrt(pi)/sigma^1.5 factor) are computed once per particle, which
// yields the same values as recomputing them inside every evaluation.  The
// device's exp/pow/sin differ from the host libm by a few ulp, so results
// agree with the reference to rounding, not bit for bit.
//
// The reference's retry loop and sampling loop have no bound; here each step
// gives up after MAX_ATTEMPTS rejected trials and each particle after
// max_steps steps, with a status bit, so a NaN never turns into a spin.
#include <cmath>
#include "common.cuh"
#include "plan.hpp"

namespace magpy {

namespace {

constexpr double KB_D = 1.38064852e-23;  // include/constants.hpp:10-12
constexpr double GYRO_D = 1.76086e11;
// One warp per CTA: the step counts of particles differ by orders of
// magnitude, so the launch (heaviest warps first) leaves the balancing of
// the SMs' FP64 pipes to the CTA scheduler.
constexpr int DOM_THREADS = 32;

struct DomParams {
    double hpre;   // (tau_N sqrt(pi)) / sigma^1.5
    double sigma;  // K V / kB / T
    double h, f;   // reduced field amplitude, frequency (Hz)
};

__device__ inline double dom_field(int shape, double t, double h, double f, int64_t ncomp)
{
    switch (shape) {
    case 2: return h;                                          // field.cpp:23-26
    case 0: return h * sin(2 * M_PI * f * t);                  // field.cpp:37-40
    case 1: return h * (int(t * f * 2) % 2 ? -1 : 1);          // field.cpp:51-54
    case 3: {                                                  // field.cpp:67-79
        double field = 0;
        for (unsigned int k = 1; k < (unsigned int)ncomp + 1; k++)
            field += sin(2 * M_PI * (2 * k - 1) * f * t) / (2 * k - 1);
        field *= 4 / M_PI * h;
        return field;
    }
    default: return NAN;
    }
}

// dp/dt = W(h(t)) p with W = [[-r2, r1], [r2, -r1]]: lib/dom.cpp:33-59, 79-97.
__device__ inline void dom_derivs(double d[2], const double x[2], double t, const DomParams &q,
                                  int shape, int64_t ncomp)
{
    const double h = dom_field(shape, t, q.h, q.f, ncomp);
    const double e1 = q.sigma * (1 - h) * (1 - h);
    const double e2 = q.sigma * (1 + h) * (1 + h);
    const double pref = q.hpre / (1 - h * h);
    const double r1 = 1.0 / pref * (1 - h) * exp(-e1);
    const double r2 = 1.0 / pref * (1 + h) * exp(-e2);
    // row-major 2x2 product, summed as the project's dgemv shim sums it
    double s0 = 0.0, s1 = 0.0;
    s0 = s0 + (-r2) * x[0];
    s0 = s0 + r1 * x[1];
    s1 = s1 + r2 * x[0];
    s1 = s1 + (-r1) * x[1];
    d[0] = 1.0 * s0 + 0.0;
    d[1] = 1.0 * s1 + 0.0;
}

// Cash-Karp RK45 step (lib/integrators.cpp:152-251; coefficients: J. R. Cash,
// A. H. Karp, ACM TOMS 16 (1990) 201-222).  Returns false when MAX_ATTEMPTS
// trials were rejected.
__device__ inline bool dom_rk45(double next[2], double *h_ptr, double *t_ptr, const double cur[2],
                                double tol, const DomParams &q, int shape, int64_t ncomp)
{
    const double c11 = 0.2, c21 = 3.0 / 40.0, c22 = 9.0 / 40.0, c31 = 3.0 / 10.0,
                 c32 = -9.0 / 10.0, c33 = 6.0 / 5.0, c41 = -11.0 / 54.0, c42 = 2.5,
                 c43 = -70.0 / 27.0, c44 = 35.0 / 27.0, c51 = 1631.0 / 55296.0,
                 c52 = 175.0 / 512.0, c53 = 575.0 / 13824.0, c54 = 44275.0 / 110592.0,
                 c55 = 253.0 / 4096.0;
    const double hc1 = 0.2, hc2 = 0.3, hc3 = 0.6, hc4 = 1.0, hc5 = 7.0 / 8.0;
    const double x11 = 37.0 / 378.0, x13 = 250.0 / 621.0, x14 = 125.0 / 594.0,
                 x16 = 512.0 / 1771.0;
    const double x21 = 2825.0 / 27648.0, x23 = 18575.0 / 48384.0, x24 = 13525.0 / 55296.0,
                 x25 = 277.0 / 14336.0, x26 = 0.25;
    double k1[2], k2[2], k3[2], k4[2], k5[2], k6[2], tmp[2];
    double err = 0.0, h = *h_ptr;
    const double t = *t_ptr;
    bool ok = false;
    for (int attempt = 0; attempt < DOM_MAX_ATTEMPTS && !ok; attempt++) {
        dom_derivs(k1, cur, t, q, shape, ncomp);
        for (int i = 0; i < 2; i++) next[i] = k1[i] * h * c11 + cur[i];
        dom_derivs(k2, next, t + h * hc1, q, shape, ncomp);
        for (int i = 0; i < 2; i++) next[i] = cur[i] + h * (c21 * k1[i] + c22 * k2[i]);
        dom_derivs(k3, next, t + h * hc2, q, shape, ncomp);
        for (int i = 0; i < 2; i++)
            next[i] = cur[i] + h * (c31 * k1[i] + c32 * k2[i] + c33 * k3[i]);
        dom_derivs(k4, next, t + h * hc3, q, shape, ncomp);
        for (int i = 0; i < 2; i++)
            next[i] = cur[i] + h * (c41 * k1[i] + c42 * k2[i] + c43 * k3[i] + c44 * k4[i]);
        dom_derivs(k5, next, t + h * hc4, q, shape, ncomp);
        for (int i = 0; i < 2; i++)
            next[i] = cur[i] +
                      h * (c51 * k1[i] + c52 * k2[i] + c53 * k3[i] + c54 * k4[i] + c55 * k5[i]);
        dom_derivs(k6, next, t + h * hc5, q, shape, ncomp);
        for (int i = 0; i < 2; i++)
            tmp[i] = cur[i] + h * (x11 * k1[i] + x13 * k3[i] + x14 * k4[i] + x16 * k6[i]);
        for (int i = 0; i < 2; i++)
            next[i] = cur[i] +
                      h * (x21 * k1[i] + x23 * k3[i] + x24 * k4[i] + x25 * k5[i] + x26 * k6[i]);
        // std::pow(x, 2) compiles to x * x in the reference build (exact), and
        // std::pow(x, 0.5) of a non-negative finite x is within half an ulp of
        // the correctly rounded sqrt, which the device computes exactly
        err = 0;
        double mag = 0;
        for (int i = 0; i < 2; i++) mag += cur[i] * cur[i];
        mag = sqrt(mag);
        for (int i = 0; i < 2; i++) {
            const double d = tmp[i] - next[i];
            err += d * d;
        }
        err = sqrt(err);
        err /= (2.0 * tol * (1 + mag));
        if (err < 1.0) {
            ok = true;
        } else {
            double hf = 0.84 * pow(err, -0.2);
            hf = fabs(hf) < 0.1 ? 0.1 : hf;
            h *= hf;
        }
    }
    if (!ok) return false;
    *t_ptr = t + h;
    double hf = err == 0.0 ? 5.0 : 0.84 * pow(err, -0.2);
    hf = hf > 5 ? 5.0 : hf;
    *h_ptr = hf * h;
    return true;
}

// One thread per particle; `order` lists particles by expected step count,
// largest first, so that the threads of a warp take similar numbers of steps.
__global__ void __launch_bounds__(DOM_THREADS)
    dom_kernel(DomArgs a)
{
    const int64_t w = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (w >= a.E) return;
    const int64_t e = a.order ? a.order[w] : w;
    const DomMember m = a.members[e];
    const double sigma = m.k * m.v / KB_D / m.T;
    const double taun = m.v * m.ms * (1 + m.alpha * m.alpha) / 2.0 / GYRO_D / m.alpha / KB_D / m.T;
    const DomParams q{taun * sqrt(M_PI) / pow(sigma, 1.5), sigma, m.h, m.f};
    const int shape = a.shape;
    const int64_t N = a.N, nc = a.ncomp;
    double *mz = a.mz + e * N, *fld = a.field + e * N, *tm = a.time + e * N;
    double last[2], next[2] = {m.p0, m.p1};
    mz[0] = next[0] - next[1];
    tm[0] = 0;
    fld[0] = dom_field(shape, 0, q.h, q.f, nc) * m.hk;
    double t = 0, t_last = 0;
    const double max_dt = a.end_time / 1000.0;
    double dt = 0.01 * a.time_step;
    const double eps = a.time_step;
    const double Ts = a.sampling_time;
    int64_t step = 0;
    int32_t status = 0;
    int64_t sample = 1;
    for (; sample < N && status == 0; sample++) {
        while (t <= sample * Ts) {
            last[0] = next[0];
            last[1] = next[1];
            t_last = t;
            if (step >= a.max_steps) { status = DOM_ST_STEP_LIMIT; break; }
            step++;
            if (!dom_rk45(next, &dt, &t, last, eps, q, shape, nc)) {
                status = DOM_ST_STEP_LIMIT;
                break;
            }
            if (!isfinite(t) || !isfinite(dt)) { status = DOM_ST_NONFINITE; break; }
            dt = dt > max_dt ? max_dt : dt;
        }
        if (status != 0) break;
        const double mz_last = last[0] - last[1];
        const double mz_next = next[0] - next[1];
        const double t_sample = sample * Ts;
        const double beta = (mz_next - mz_last) / (t - t_last);  // first-order hold
        mz[sample] = mz_last + beta * (t_sample - t_last);
        tm[sample] = t_sample;
        fld[sample] = dom_field(shape, t_sample, q.h, q.f, nc) * m.hk;
    }
    for (; sample < N; sample++) {
        const double t_sample = sample * Ts;
        mz[sample] = NAN;
        tm[sample] = t_sample;
        fld[sample] = dom_field(shape, t_sample, q.h, q.f, nc) * m.hk;
    }
    a.status[e] = status;
    a.steps[e] = step;
}

}  // namespace

cudaError_t launch_dom(const DomArgs &a, cudaStream_t stream)
{
    if (a.E == 0) return cudaSuccess;
    const int64_t blocks = (a.E + DOM_THREADS - 1) / DOM_THREADS;
    dom_kernel<<<(unsigned)blocks, DOM_THREADS, 0, stream>>>(a);
    return cudaGetLastError();
}

}  // namespace magpy
