// dom_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement (FP64) of magpy's two-state master-equation path (the
// "discrete orientation model", DOModel): magpy/model.py:211-295 ->
// magpy/core.pyx:205-278 simulate_dom -> simulation::dom_ensemble_dynamics
// (lib/simulation.cpp:659-767) -> integrator::rk45 (lib/integrators.cpp:
// 152-251) -> dom::master_equation_with_update (lib/dom.cpp:79-97) ->
// dom::transition_matrix (lib/dom.cpp:33-59) and stochastic::master_equation
// (lib/stochastic_processes.cpp:18-25, a 2x2 dgemv).
//
// The checker for magpy_gb300/csrc/dom.cu; only tests/, smoke() and the CPU
// legs of bench.py load it.  Pinned bit for bit against the reference's own
// lib/*.cpp (oracle/_ref) and against the rk45 / master-equation / transition
// matrix known answers of test/tests.cpp.
//
// Same operation order as the reference everywhere.  The one deliberate
// difference: the reference's rk45 retry loop and sampling loop are
// unbounded (a NaN error estimate never ends the retry loop); here both are
// bounded (max_attempts retries per step, max_steps steps per member) and
// the member stops with a status bit, as on the GPU.

#include <cmath>
#include <cstdint>
#include <cstring>

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

static const double KB_ = 1.38064852e-23;  // include/constants.hpp:10-12
static const double MU0_ = 1.25663706e-6;
static const double GYRO_ = 1.76086e11;

enum { DOM_SINE = 0, DOM_SQUARE = 1, DOM_CONSTANT = 2, DOM_SQUARE_FOURIER = 3 };
enum { DOM_OK = 0, DOM_NONFINITE = 4, DOM_STEP_LIMIT = 32 };

// Waveforms bound by magpy/core.pyx:231-248 (lib/field.cpp:23-81).
double oracle_dom_field(int shape, double t, double h, double f, int64_t n_components)
{
    switch (shape) {
    case DOM_CONSTANT: return h;                                       // field.cpp:23-26
    case DOM_SINE: return h * std::sin(2 * M_PI * f * t);              // field.cpp:37-40
    case DOM_SQUARE: return h * (int(t * f * 2) % 2 ? -1 : 1);         // field.cpp:51-54
    case DOM_SQUARE_FOURIER: {                                         // field.cpp:67-79
        double field = 0;
        for (unsigned int k = 1; k < (unsigned int)n_components + 1; k++)
            field += std::sin(2 * M_PI * (2 * k - 1) * f * t) / (2 * k - 1);
        field *= 4 / M_PI * h;
        return field;
    }
    default: return NAN;
    }
}

// y = W x for a row-major n x n W, as the project's cblas_dgemv shim
// computes it (alpha = 1, beta = 0): lib/stochastic_processes.cpp:18-25.
void oracle_master_equation(double *y, const double *W, const double *x, int64_t n)
{
    for (int64_t i = 0; i < n; i++) {
        double s = 0.0;
        for (int64_t j = 0; j < n; j++) s = s + W[i * n + j] * x[j];
        y[i] = 1.0 * s + 0.0;
    }
}

typedef void (*ode_cb)(double *dx, const double *x, double t, void *ctx);

// Cash-Karp embedded Runge-Kutta 4(5) step with adaptive step size:
// lib/integrators.cpp:152-251.  The coefficients are the published Cash-Karp
// table (J. R. Cash, A. H. Karp, ACM TOMS 16 (1990) 201-222), as in
// include/integrators.hpp:127-160.  Returns 0, or DOM_STEP_LIMIT when
// max_attempts trials were rejected (the reference retries forever).
int oracle_rk45(double *next, double *tmp, double *k1, double *k2, double *k3, double *k4,
                double *k5, double *k6, double *h_ptr, double *t_ptr, const double *cur,
                ode_cb derivs, void *ctx, int64_t n, double tol, int64_t max_attempts)
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
    bool ok = false;
    double err = 0.0;
    double h = *h_ptr;
    const double t = *t_ptr;
    int64_t attempts = 0;
    while (!ok) {
        if (attempts++ >= max_attempts) return DOM_STEP_LIMIT;
        derivs(k1, cur, t, ctx);
        for (int64_t i = 0; i < n; i++) next[i] = k1[i] * h * c11 + cur[i];
        derivs(k2, next, t + h * hc1, ctx);
        for (int64_t i = 0; i < n; i++) next[i] = cur[i] + h * (c21 * k1[i] + c22 * k2[i]);
        derivs(k3, next, t + h * hc2, ctx);
        for (int64_t i = 0; i < n; i++)
            next[i] = cur[i] + h * (c31 * k1[i] + c32 * k2[i] + c33 * k3[i]);
        derivs(k4, next, t + h * hc3, ctx);
        for (int64_t i = 0; i < n; i++)
            next[i] = cur[i] + h * (c41 * k1[i] + c42 * k2[i] + c43 * k3[i] + c44 * k4[i]);
        derivs(k5, next, t + h * hc4, ctx);
        for (int64_t i = 0; i < n; i++)
            next[i] = cur[i] +
                      h * (c51 * k1[i] + c52 * k2[i] + c53 * k3[i] + c54 * k4[i] + c55 * k5[i]);
        derivs(k6, next, t + h * hc5, ctx);
        for (int64_t i = 0; i < n; i++)
            tmp[i] = cur[i] + h * (x11 * k1[i] + x13 * k3[i] + x14 * k4[i] + x16 * k6[i]);
        for (int64_t i = 0; i < n; i++)
            next[i] = cur[i] +
                      h * (x21 * k1[i] + x23 * k3[i] + x24 * k4[i] + x25 * k5[i] + x26 * k6[i]);
        err = 0;
        double mag = 0;
        for (int64_t i = 0; i < n; i++) mag += cur[i] * cur[i];
        mag = std::pow(mag, 0.5);
        for (int64_t i = 0; i < n; i++) err += std::pow(std::abs(tmp[i] - next[i]), 2);
        err = std::pow(err, 0.5);
        err /= ((double)n * tol * (1 + mag));
        if (err < 1.0) {
            ok = true;
        } else {
            double hf = 0.84 * std::pow(err, -0.2);
            hf = std::abs(hf) < 0.1 ? 0.1 : hf;
            h *= hf;
        }
    }
    *t_ptr = t + h;
    double hf = err == 0.0 ? 5.0 : 0.84 * std::pow(err, -0.2);
    hf = hf > 5 ? 5.0 : hf;
    *h_ptr = hf * h;
    return 0;
}

// Néel-Brown transition matrix: lib/dom.cpp:33-59 (same association).
static void dom_W(double *W, double k, double v, double T, double h, double ms, double alpha)
{
    double sigma = k * v / KB_ / T;
    double taun = v * ms * (1 + alpha * alpha) / 2.0 / GYRO_ / alpha / KB_ / T;
    double e1 = sigma * (1 - h) * (1 - h);
    double e2 = sigma * (1 + h) * (1 + h);
    double pref = taun * std::sqrt(M_PI) / std::pow(sigma, 1.5) / (1 - h * h);
    double r1 = 1.0 / pref * (1 - h) * std::exp(-e1);
    double r2 = 1.0 / pref * (1 + h) * std::exp(-e2);
    W[0] = -r2; W[1] = r1; W[2] = r2; W[3] = -r1;
}

struct DomCtx {
    double k, v, T, ms, alpha, h, f;
    int shape;
    int64_t ncomp;
};

// dom::master_equation_with_update: lib/dom.cpp:79-97.
static void dom_derivs(double *d, const double *x, double t, void *c)
{
    const DomCtx *p = (const DomCtx *)c;
    double W[4];
    dom_W(W, p->k, p->v, p->T, oracle_dom_field(p->shape, t, p->h, p->f, p->ncomp), p->ms,
          p->alpha);
    oracle_master_equation(d, W, x, 2);
}

// simulation::dom_ensemble_dynamics: lib/simulation.cpp:659-767, reduced
// field amplitude h, physical time.  Outputs [N_samples]: mz (p_up - p_down
// with first-order hold), reduced field, time.  max_samples = -1 samples
// every integration step of length time_step (int(end/dt)+1 samples).
int oracle_dom_dynamics(double volume, double anisotropy, double temperature, double ms,
                        double alpha, int32_t shape, double h_red, double f, int64_t ncomp,
                        const double *p0, double time_step, double end_time,
                        int64_t max_samples, int64_t max_steps, int64_t max_attempts,
                        double *mz, double *field, double *time, int64_t *steps_out)
{
    DomCtx c{anisotropy, volume, temperature, ms, alpha, h_red, f, shape, ncomp};
    double last[2], next[2] = {p0[0], p0[1]};
    double k1[2], k2[2], k3[2], k4[2], k5[2], k6[2], tmp[2];
    const int64_t N = max_samples == -1 ? (int64_t)int(end_time / time_step) + 1 : max_samples;
    const double sampling_time = end_time / (N - 1);
    mz[0] = next[0] - next[1];
    time[0] = 0;
    field[0] = oracle_dom_field(shape, 0, h_red, f, ncomp);
    double t = 0, t_last = 0;
    const double max_dt = end_time / 1000.0;
    double dt = 0.01 * time_step;
    const double eps = time_step;
    int64_t step = 0;
    int status = DOM_OK;
    int64_t sample = 1;
    for (; sample < N && status == DOM_OK; sample++) {
        while (t <= sample * sampling_time) {
            last[0] = next[0];
            last[1] = next[1];
            t_last = t;
            if (step >= max_steps) { status = DOM_STEP_LIMIT; break; }
            step++;
            const int rc = oracle_rk45(next, tmp, k1, k2, k3, k4, k5, k6, &dt, &t, last,
                                       dom_derivs, &c, 2, eps, max_attempts);
            if (rc != 0 || !std::isfinite(t) || !std::isfinite(dt)) {
                status = rc != 0 ? rc : DOM_NONFINITE;
                break;
            }
            dt = dt > max_dt ? max_dt : dt;
        }
        if (status != DOM_OK) break;
        const double mz_last = last[0] - last[1];
        const double mz_next = next[0] - next[1];
        const double t_sample = sample * sampling_time;
        const double beta = (mz_next - mz_last) / (t - t_last);
        mz[sample] = mz_last + beta * (t_sample - t_last);
        time[sample] = t_sample;
        field[sample] = oracle_dom_field(shape, t_sample, h_red, f, ncomp);
    }
    for (; sample < N; sample++) {  // a stopped member: the rest of its samples are NaN
        const double t_sample = sample * sampling_time;
        mz[sample] = NAN;
        time[sample] = t_sample;
        field[sample] = oracle_dom_field(shape, t_sample, h_red, f, ncomp);
    }
    if (steps_out) *steps_out = step;
    return status;
}

// magpy/core.pyx:205-278 simulate_dom for a batch of independent particles
// (one OpenMP task each): physical field amplitude, output field in A/m.
// Per-member arrays [E]; p0 [E][2]; outputs [E][N].
int oracle_dom_batch(int64_t E, const double *volume, const double *anisotropy,
                     const double *temperature, const double *ms, const double *alpha,
                     const double *p0, int32_t shape, const double *amplitude,
                     const double *frequency, int64_t ncomp, double time_step, double end_time,
                     int64_t max_samples, int64_t max_steps, int64_t max_attempts,
                     int32_t n_threads, double *mz, double *field, double *time,
                     int32_t *status, int64_t *steps)
{
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
    const int64_t N = max_samples == -1 ? (int64_t)int(end_time / time_step) + 1 : max_samples;
#pragma omp parallel for schedule(dynamic)
    for (int64_t e = 0; e < E; e++) {
        const double hk = 2.0 * anisotropy[e] / MU0_ / ms[e];  // core.pyx:226
        const double h_red = amplitude[e] / hk;                  // core.pyx:227
        status[e] = oracle_dom_dynamics(volume[e], anisotropy[e], temperature[e], ms[e],
                                        alpha[e], shape, h_red, frequency[e], ncomp,
                                        p0 + 2 * e, time_step, end_time, max_samples,
                                        max_steps, max_attempts, mz + e * N, field + e * N,
                                        time + e * N, steps ? steps + e : nullptr);
        for (int64_t s = 0; s < N; s++) field[e * N + s] *= hk;  // core.pyx:269
    }
    return 0;
}

// test/tests.cpp rk45 known answers use this ODE: dx0 = x1 t, dx1 = -x0 - 5
static void tests_ode(double *dx, const double *x, double t, void *)
{
    dx[0] = x[1] * t;
    dx[1] = -x[0] - 5;
}

int oracle_rk45_tests_ode(double *x2, double *k_all, double *h, double *t, const double *x1,
                          double tol)
{
    double tmp[2];
    return oracle_rk45(x2, tmp, k_all, k_all + 2, k_all + 4, k_all + 6, k_all + 8, k_all + 10,
                       h, t, x1, tests_ode, nullptr, 2, tol, 1 << 20);
}

}  // extern "C"
