// ref_harness.cpp -- TEST INFRASTRUCTURE ONLY.
//
// A C-ABI harness around the reference's own C++ (lib/*.cpp, compiled from
// the reference checkout by oracle/Makefile into oracle/_ref/).  It lets the
// tests and the golden-fixture generator call the unmodified reference:
//   * the reduced-unit simulation::full_dynamics (lib/simulation.cpp:132)
//     with injected Wiener increments through RngArray (lib/rng.cpp:67-94);
//   * the physical-unit simulation::full_dynamics (lib/simulation.cpp:476)
//     with its own RngMtNorm noise, per member under OpenMP (the reference
//     CPU baseline; the reference itself fans out with joblib processes);
//   * the component functions pinned by test/tests.cpp.
// Built only where the reference sources exist; never shipped or linked by
// the product.

#include <cstdint>
#include <cstring>
#include <vector>
#include <array>
#include <functional>
#include <stdexcept>
#include <cmath>
#include <omp.h>

#include "simulation.hpp"
#include "llg.hpp"
#include "field.hpp"
#include "integrators.hpp"
#include "optimisation.hpp"
#include "rng.hpp"
#include "dom.hpp"
#include "distances.hpp"

using d3v = std::array<double, 3>;

static std::vector<d3v> to_d3(const double *a, int64_t n)
{
    std::vector<d3v> v(n);
    for (int64_t i = 0; i < n; i++)
        for (int k = 0; k < 3; k++) v[i][k] = a[3 * i + k];
    return v;
}

static field::options shape_of(int32_t s)
{
    return s == 0 ? field::SINE : s == 1 ? field::SQUARE : field::CONSTANT;
}

extern "C" {

// Reduced-unit driver with injected noise.  Arguments mirror
// oracle_reduced_t field by field.  Returns 0, or 8 when RngArray ran out.
int ref_full_dynamics_reduced(int64_t n, const double *sr, const double *k_red,
                              const double *v_red, const double *axes, const double *m0,
                              const double *unit_dist, const double *dist_mag,
                              int32_t field_shape, double happ, double fapp, double k_av,
                              double v_av, double alpha, double ms, double dt, double end_time,
                              int32_t renorm, int32_t interactions, int32_t use_implicit,
                              double eps, int64_t max_samples, const double *noise,
                              int64_t noise_len, double *mx, double *my, double *mz,
                              double *fieldv, double *timev)
{
    std::vector<double> vsr(sr, sr + n), vk(k_red, k_red + n), vv(v_red, v_red + n);
    std::vector<std::vector<d3v>> ud(n, std::vector<d3v>(n));
    std::vector<std::vector<double>> dm(n, std::vector<double>(n));
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < n; j++) {
            for (int k = 0; k < 3; k++) ud[i][j][k] = unit_dist[(i * n + j) * 3 + k];
            dm[i][j] = dist_mag[i * n + j];
        }
    std::function<double(const double)> f;
    if (field_shape == 2) f = [happ](const double) { return happ; };
    else if (field_shape == 0) f = [happ, fapp](const double t) { return field::sinusoidal(t, happ, fapp); };
    else f = [happ, fapp](const double t) { return field::square(t, happ, fapp); };
    RngArray rng(noise, (size_t)noise_len);
    try {
        auto res = simulation::full_dynamics(vsr, vk, vv, to_d3(axes, n), to_d3(m0, n), ud, dm, f,
                                             k_av, v_av, alpha, ms, dt, end_time, rng, renorm,
                                             interactions, use_implicit, eps, (int)max_samples);
        for (int64_t q = 0; q < n; q++)
            for (int64_t s = 0; s < max_samples; s++) {
                mx[q * max_samples + s] = res[q].mx[s];
                my[q * max_samples + s] = res[q].my[s];
                mz[q * max_samples + s] = res[q].mz[s];
                if (q == 0) { fieldv[s] = res[q].field[s]; timev[s] = res[q].time[s]; }
            }
    } catch (const std::out_of_range &) {
        return 8;
    }
    return 0;
}

// Physical-unit driver (RngMtNorm noise from the seed), one cluster.
int ref_full_dynamics(int64_t n, const double *radius, const double *anisotropy,
                      const double *axes, const double *m0, const double *location, double ms,
                      double damping, double temperature, int32_t renorm, int32_t interactions,
                      int32_t use_implicit, double eps, double time_step, double end_time,
                      int64_t max_samples, int64_t seed, int32_t field_shape, double amp,
                      double freq, double *mx, double *my, double *mz, double *fieldv,
                      double *timev)
{
    std::vector<double> r(radius, radius + n), k(anisotropy, anisotropy + n);
    auto res = simulation::full_dynamics(r, k, to_d3(axes, n), to_d3(m0, n), to_d3(location, n),
                                         ms, damping, temperature, renorm, interactions,
                                         use_implicit, eps, time_step, end_time,
                                         (size_t)max_samples, (long)seed, shape_of(field_shape),
                                         amp, freq);
    for (int64_t q = 0; q < n; q++)
        for (int64_t s = 0; s < max_samples; s++) {
            mx[q * max_samples + s] = res[q].mx[s];
            my[q * max_samples + s] = res[q].my[s];
            mz[q * max_samples + s] = res[q].mz[s];
            if (q == 0) { fieldv[s] = res[q].field[s]; timev[s] = res[q].time[s]; }
        }
    return 0;
}

// Members sharing one geometry, run under OpenMP (dynamic schedule);
// outputs [E][n][S] (pass NULL to discard trajectories).
int ref_ensemble(int64_t E, int64_t n, const double *radius, const double *anisotropy,
                 const double *axes, const double *m0, const double *location, double ms,
                 double damping, double temperature, int32_t renorm, int32_t interactions,
                 int32_t use_implicit, double eps, double time_step, double end_time,
                 int64_t max_samples, const int64_t *seeds, int32_t field_shape, double amp,
                 double freq, int32_t n_threads, double *mx, double *my, double *mz)
{
    if (n_threads > 0) omp_set_num_threads(n_threads);
    const int64_t S = max_samples;
#pragma omp parallel
    {
        std::vector<double> bx(n * S), by(n * S), bz(n * S), f(S), t(S);
#pragma omp for schedule(dynamic)
        for (int64_t e = 0; e < E; e++) {
            ref_full_dynamics(n, radius, anisotropy, axes, m0, location, ms, damping,
                              temperature, renorm, interactions, use_implicit, eps, time_step,
                              end_time, max_samples, seeds[e], field_shape, amp, freq,
                              bx.data(), by.data(), bz.data(), f.data(), t.data());
            if (mx) {
                std::memcpy(mx + e * n * S, bx.data(), n * S * sizeof(double));
                std::memcpy(my + e * n * S, by.data(), n * S * sizeof(double));
                std::memcpy(mz + e * n * S, bz.data(), n * S * sizeof(double));
            }
        }
    }
    return 0;
}

// ---- component functions (test/tests.cpp goldens) ----
void ref_llg_drift(double *d, const double *m, double alpha, const double *h)
{ llg::drift(d, m, 0.0, alpha, h); }
void ref_llg_diffusion(double *b, const double *m, double sr, double alpha)
{ llg::diffusion(b, m, 0.0, sr, alpha); }
void ref_llg_drift_jacobian(double *j, const double *m, double alpha, const double *h,
                            const double *hj)
{ llg::drift_jacobian(j, m, 0.0, alpha, h, hj); }
void ref_llg_diffusion_jacobian(double *j, const double *m, double sr, double alpha)
{ llg::diffusion_jacobian(j, m, 0.0, sr, alpha); }
void ref_multi_add_dipolar(double *field, double ms, double k_av, const double *v_red,
                           const double *mag, const double *dists, const double *dist_cubes,
                           int64_t n)
{ field::multi_add_dipolar(field, ms, k_av, v_red, mag, dists, dist_cubes, (size_t)n); }
void ref_mt_norm(uint64_t seed, double stddev, int64_t count, double *out)
{
    RngMtNorm rng(seed, stddev);
    for (int64_t i = 0; i < count; i++) out[i] = rng.get();
}
void ref_save_results(const char *prefix, const double *mx, const double *my, const double *mz,
                      const double *field, const double *time, int64_t n)
{
    simulation::results r((size_t)n);
    for (int64_t i = 0; i < n; i++) {
        r.mx[i] = mx[i]; r.my[i] = my[i]; r.mz[i] = mz[i];
        r.field[i] = field[i]; r.time[i] = time[i];
    }
    simulation::save_results(prefix, r);
}
// simulation::dom_ensemble_dynamics (lib/simulation.cpp:659-767) with the
// reduced field bound as magpy/core.pyx:231-248 binds it; outputs [N].
int ref_dom_dynamics(double volume, double anisotropy, double temperature, double ms,
                     double alpha, int32_t shape, double h_red, double f, int64_t ncomp,
                     const double *p0, double time_step, double end_time, int64_t max_samples,
                     double *mz, double *field, double *time)
{
    std::function<double(double)> fn;
    switch (shape) {
    case 0: fn = [=](double t) { return field::sinusoidal(t, h_red, f); }; break;
    case 1: fn = [=](double t) { return field::square(t, h_red, f); }; break;
    case 2: fn = [=](double t) { return field::constant(t, h_red); }; break;
    case 3: fn = [=](double t) { return field::square_fourier(t, h_red, f, (size_t)ncomp); };
        break;
    default: return -1;
    }
    std::array<double, 2> ip{p0[0], p0[1]};
    simulation::results r = simulation::dom_ensemble_dynamics(
        volume, anisotropy, temperature, ms, alpha, fn, ip, time_step, end_time,
        (int)max_samples);
    for (size_t i = 0; i < r.N; i++) {
        mz[i] = r.mz[i]; field[i] = r.field[i]; time[i] = r.time[i];
    }
    return 0;
}
// integrator::rk45 on the ODE of the rk45 tests in test/tests.cpp.
void ref_rk45_tests_ode(double *x2, double *k_all, double *h, double *t, const double *x1,
                        double tol)
{
    auto ode = [](double *dx, const double *x, const double tt) {
        dx[0] = x[1] * tt;
        dx[1] = -x[0] - 5;
    };
    double tmp[2];
    integrator::rk45(x2, tmp, k_all, k_all + 2, k_all + 4, k_all + 6, k_all + 8, k_all + 10, h,
                     t, x1, ode, 2, tol);
}
void ref_dom_transition_matrix(double *W, double k, double v, double T, double h, double ms,
                               double alpha)
{ dom::transition_matrix(W, k, v, T, h, ms, alpha); }

}  // extern "C"
