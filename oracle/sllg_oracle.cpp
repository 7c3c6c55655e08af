// sllg_oracle.cpp -- TEST INFRASTRUCTURE ONLY.
//
// CPU restatement (FP64) of magpy's stochastic Landau-Lifshitz-Gilbert
// ensemble path, used as the checker for the CUDA implementation in
// magpy_gb300/csrc.  Only tests/, __graft_entry__.smoke() and the CPU
// baseline legs of bench.py may load this library.  Nothing in the product
// path links or calls it.
//
// Parity pin: the restatement is checked bit-for-bit against the reference
// itself (lib/*.cpp compiled by oracle/Makefile into oracle/_ref, driven
// through oracle/ref_harness.cpp) and against the golden values of the
// reference's unit tests (test/tests.cpp) -- see tests/test_oracle_*.py.
//
// Build: g++ -O2 -ffp-contract=off (no FMA contraction, so every product and
// sum rounds exactly as written, on x86-64 and on aarch64 alike).
//
// Each function cites the reference file:line it restates.  The arithmetic
// is kept in the same order as the reference (same association of every
// sum and product) because the CUDA FP64 path is required to reproduce it
// exactly.  Where the reference multiplies by structurally-zero blocks of a
// dense 3N x 3N matrix, the restatement skips them: adding an exact zero
// never changes an IEEE double (except the sign of a zero), so the block
// form gives the same bits as the dense loops.

#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>
#include <vector>
#include <algorithm>
#include <stdexcept>

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" {

// ---------------------------------------------------------------------------
// Constants: include/constants.hpp:10-12
// ---------------------------------------------------------------------------
static const double KB = 1.38064852e-23;
static const double MU0 = 1.25663706e-6;
static const double GYROMAG = 1.76086e11;

double oracle_const_kb() { return KB; }
double oracle_const_mu0() { return MU0; }
double oracle_const_gyromag() { return GYROMAG; }

// Status bits (per member), shared meaning with the CUDA path.
enum {
    ORACLE_OK = 0,
    ORACLE_NEWTON_MAXITER = 1,   // optimisation.hpp:22-33 MAX_ITERATIONS_ERR
    ORACLE_SINGULAR = 2,         // LAPACK_ERR (dgesv info > 0)
    ORACLE_NONFINITE = 4,
    ORACLE_NOISE_EXHAUSTED = 8,  // RngArray out_of_range, rng.cpp:84-94
};

enum { FIELD_SINE = 0, FIELD_SQUARE = 1, FIELD_CONSTANT = 2 };  // field.hpp options

// ---------------------------------------------------------------------------
// Field waveforms: lib/field.cpp:23-54
// ---------------------------------------------------------------------------
double oracle_field_value(int shape, double t, double h, double f)
{
    switch (shape) {
    case FIELD_CONSTANT: return h;                                  // field.cpp:23
    case FIELD_SINE: return h * std::sin(2 * M_PI * f * t);         // field.cpp:37-40
    case FIELD_SQUARE: return h * (int(t * f * 2) % 2 ? -1 : 1);    // field.cpp:51-54
    default: return NAN;
    }
}

// ---------------------------------------------------------------------------
// LLG drift: lib/llg.cpp:14-29
// ---------------------------------------------------------------------------
void oracle_llg_drift(double *d, const double *m, double alpha, const double *h)
{
    d[0] = m[2] * h[1] - m[1] * h[2]
        + alpha * (h[0] * (m[1] * m[1] + m[2] * m[2]) - m[0] * (m[1] * h[1] + m[2] * h[2]));
    d[1] = m[0] * h[2] - m[2] * h[0]
        + alpha * (h[1] * (m[0] * m[0] + m[2] * m[2]) - m[1] * (m[0] * h[0] + m[2] * h[2]));
    d[2] = m[1] * h[0] - m[0] * h[1]
        + alpha * (h[2] * (m[0] * m[0] + m[1] * m[1]) - m[2] * (m[0] * h[0] + m[1] * h[1]));
}

// LLG diffusion (3x3, row-major): lib/llg.cpp:92-106
void oracle_llg_diffusion(double *b, const double *m, double sr, double alpha)
{
    b[0] = alpha * sr * (m[1] * m[1] + m[2] * m[2]);
    b[1] = sr * (m[2] - alpha * m[0] * m[1]);
    b[2] = -sr * (m[1] + alpha * m[0] * m[2]);
    b[3] = -sr * (m[2] + alpha * m[0] * m[1]);
    b[4] = alpha * sr * (m[0] * m[0] + m[2] * m[2]);
    b[5] = sr * (m[0] - alpha * m[1] * m[2]);
    b[6] = sr * (m[1] - alpha * m[0] * m[2]);
    b[7] = -sr * (m[0] + alpha * m[1] * m[2]);
    b[8] = alpha * sr * (m[0] * m[0] + m[1] * m[1]);
}

// Drift Jacobian: lib/llg.cpp:68-81 (hj is a 3x3 row-major block)
void oracle_llg_drift_jacobian(double *j, const double *m, double a, const double *h,
                               const double *hj)
{
    j[0] =  m[2]*hj[3] - m[1]*hj[6] + a*( -m[1]*h[1] - m[2]*h[2] + ( m[1]*m[1] + m[2]*m[2] )*hj[0] - m[0]*( m[1]*hj[3] + m[2]*hj[6] ) );
    j[1] = -h[2] + m[2]*hj[4] - m[1]*hj[7] + a*( 2*m[1]*h[0] + ( m[1]*m[1] + m[2]*m[2] )*hj[1] - m[0]*( h[1] + m[1]*hj[4] + m[2]*hj[7] ) );
    j[2] =  h[1] + m[2]*hj[5] - m[1]*hj[8] + a*( 2*m[2]*h[0] + ( m[1]*m[1] + m[2]*m[2] )*hj[2] - m[0]*( h[2] + m[1]*hj[5] + m[2]*hj[8] ) );
    j[3] =  h[2] - m[2]*hj[0] + m[0]*hj[6] + a*( 2*m[0]*h[1] + ( m[0]*m[0] + m[2]*m[2] )*hj[3] - m[1]*( h[0] + m[0]*hj[0] + m[2]*hj[6] ) );
    j[4] = -m[2]*hj[1] + m[0]*hj[7] + a*( -m[0]*h[0] - m[2]*h[2] + ( m[0]*m[0] + m[2]*m[2] )*hj[4] - m[1]*( m[0]*hj[1] + m[2]*hj[7] ) );
    j[5] = -h[0] - m[2]*hj[2] + m[0]*hj[8] + a*( 2*m[2]*h[1] + ( m[0]*m[0] + m[2]*m[2] )*hj[5] - m[1]*( h[2] + m[0]*hj[2] + m[2]*hj[8] ) );
    j[6] = -h[1] + m[1]*hj[0] - m[0]*hj[3] + a*( 2*m[0]*h[2] + ( m[0]*m[0] + m[1]*m[1] )*hj[6] - m[2]*( h[0] + m[0]*hj[0] + m[1]*hj[3] ) );
    j[7] =  h[0] + m[1]*hj[1] - m[0]*hj[4] + a*( 2*m[1]*h[2] + ( m[0]*m[0] + m[1]*m[1] )*hj[7] - m[2]*( h[1] + m[0]*hj[1] + m[1]*hj[4] ) );
    j[8] =  m[1]*hj[2] - m[0]*hj[5] + a*( -m[0]*h[0] - m[1]*h[1] + ( m[0]*m[0] + m[1]*m[1] )*hj[8] - m[2]*( m[0]*hj[2] + m[1]*hj[5] ) );
}

// Diffusion Jacobian (3x3x3, index 9*row + 3*wiener + deriv):
// lib/llg.cpp:118-158.  Entries [4] and [25] reproduce the reference as
// written (they use m[2] where the analytic derivative has m[0] and m[1]).
void oracle_llg_diffusion_jacobian(double *j, const double *m, double sr, double alpha)
{
    j[0] = 0;
    j[1] = 2 * alpha * sr * m[1];
    j[2] = 2 * alpha * sr * m[2];
    j[3] = -alpha * sr * m[1];
    j[4] = -alpha * sr * m[2];
    j[5] = sr;
    j[6] = -alpha * sr * m[2];
    j[7] = -sr;
    j[8] = -alpha * sr * m[0];
    j[9] = -alpha * sr * m[1];
    j[10] = -alpha * sr * m[0];
    j[11] = -sr;
    j[12] = 2 * alpha * sr * m[0];
    j[13] = 0;
    j[14] = 2 * alpha * sr * m[2];
    j[15] = sr;
    j[16] = -alpha * sr * m[2];
    j[17] = -alpha * sr * m[1];
    j[18] = -alpha * sr * m[2];
    j[19] = sr;
    j[20] = -alpha * sr * m[0];
    j[21] = -sr;
    j[22] = -alpha * sr * m[2];
    j[23] = -alpha * sr * m[1];
    j[24] = 2 * alpha * sr * m[0];
    j[25] = 2 * alpha * sr * m[2];
    j[26] = 0;
}

// Uniaxial anisotropy of one particle: lib/field.cpp:97-105
void oracle_uniaxial_anisotropy(double *h, const double *m, const double *axis)
{
    double dot = m[0] * axis[0] + m[1] * axis[1] + m[2] * axis[2];
    h[0] = dot * axis[0];
    h[1] = dot * axis[1];
    h[2] = dot * axis[2];
}

// Uniaxial anisotropy Jacobian: lib/field.cpp:143-149
void oracle_uniaxial_anisotropy_jacobian(double *j, const double *axis)
{
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++)
            j[r * 3 + c] = axis[r] * axis[c];
}

// Dense (3N x 3N) anisotropy field Jacobian: lib/field.cpp:159-174
void oracle_multi_add_uniaxial_anisotropy_jacobian(double *jac, const double *axes,
                                                   const double *k_red, int64_t n)
{
    const int64_t n3 = 3 * n;
    for (int64_t i = 0; i < n3; i++)
        for (int64_t j = 0; j < n3; j++)
            if (i / 3 == j / 3)
                jac[i * n3 + j] = k_red[i / 3] * axes[i] * axes[j];
}

// Dipolar prefactor: lib/field.cpp:212-215
double oracle_dipolar_prefactor(double ms, double k_av)
{
    return MU0 * ms * ms / 8.0 / M_PI / k_av;
}

// One pair term: lib/field.cpp:217-225
void oracle_dipolar_p2p(double *out, double vj, double rij3, const double *mj,
                        const double *dist, double prefactor)
{
    double dot = mj[0] * dist[0] + mj[1] * dist[1] + mj[2] * dist[2];
    double term_1 = vj / rij3;
    for (int c = 0; c < 3; c++)
        out[c] += prefactor * term_1 * (3 * dot * dist[c] - mj[c]);
}

// Pair sum: lib/field.cpp:187-203
void oracle_multi_add_dipolar(double *field, double ms, double k_av, const double *v_red,
                              const double *mag, const double *dists,
                              const double *dist_cubes, int64_t n)
{
    double pref = oracle_dipolar_prefactor(ms, k_av);
    for (int64_t i = 0; i < n; i++) {
        for (int64_t j = 0; j < i; j++)
            oracle_dipolar_p2p(field + i * 3, v_red[j], dist_cubes[i * n + j], mag + j * 3,
                               dists + i * n * 3 + j * 3, pref);
        for (int64_t j = i + 1; j < n; j++)
            oracle_dipolar_p2p(field + i * 3, v_red[j], dist_cubes[i * n + j], mag + j * 3,
                               dists + i * n * 3 + j * 3, pref);
    }
}

// Pairwise geometry: lib/distances.cpp:20-113.
// vec[i][j] = p_j - p_i; mag[i][j] = |vec[i][j]|; unit = vec / mag.
void oracle_pairwise_geometry(const double *points, int64_t n, double *vec, double *mag,
                              double *unit)
{
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < n; j++)
            for (int k = 0; k < 3; k++)
                vec[(i * n + j) * 3 + k] = points[j * 3 + k] - points[i * 3 + k];
    // distances.cpp:68-74 writes [i][j] and [j][i] from vec[i][j]; the last
    // write to [i][j] comes from vec[j][i] when j < i, whose norm is equal.
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < n; j++) {
            const double *d = vec + (i * n + j) * 3;
            double v = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
            mag[i * n + j] = v;
            mag[j * n + i] = v;
        }
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < n; j++)
            for (int k = 0; k < 3; k++)
                unit[(i * n + j) * 3 + k] = vec[(i * n + j) * 3 + k] / mag[i * n + j];
}

// ---------------------------------------------------------------------------
// BLAS/LAPACK arithmetic used on the path.  The reference links an unpinned
// OpenBLAS (environment.yml:6); the project's own shim (oracle/shim) defines
// the arithmetic that the reference build here uses, and these functions
// state the same arithmetic.
// ---------------------------------------------------------------------------

// dnrm2: squares summed sequentially inside consecutive triples, triples
// combined by a pairwise tree over a power-of-two padded index.
double oracle_nrm2(const double *x, int64_t n)
{
    int64_t groups = (n + 2) / 3;
    int64_t p = 1;
    while (p < groups) p <<= 1;
    std::vector<double> q(p, 0.0);
    for (int64_t g = 0; g < groups; g++) {
        double s = 0.0;
        for (int64_t k = 3 * g; k < std::min<int64_t>(3 * g + 3, n); k++)
            s = s + x[k] * x[k];
        q[g] = s;
    }
    for (int64_t stride = p / 2; stride >= 1; stride /= 2)
        for (int64_t i = 0; i < stride; i++)
            q[i] = q[i] + q[i + stride];
    return std::sqrt(q[0]);
}

// dgesv (row-major, one right-hand side): right-looking LU with partial
// pivoting (first index of the largest |a| wins), division multipliers,
// forward substitution in increasing order, column-oriented back
// substitution.  Returns info: 0 ok, k>0 when U(k,k) is exactly zero (b is
// then left unchanged, as LAPACK does).
int64_t oracle_dgesv(int64_t n, double *a, double *b)
{
    std::vector<int64_t> piv(n);
    int64_t info = 0;
    for (int64_t k = 0; k < n; k++) {
        int64_t p = k;
        double vmax = std::fabs(a[k * n + k]);
        for (int64_t i = k + 1; i < n; i++) {
            double v = std::fabs(a[i * n + k]);
            if (v > vmax) { vmax = v; p = i; }
        }
        piv[k] = p;
        if (a[p * n + k] != 0.0) {
            if (p != k)
                for (int64_t c = 0; c < n; c++) std::swap(a[k * n + c], a[p * n + c]);
            double pivot = a[k * n + k];
            for (int64_t i = k + 1; i < n; i++) {
                double l = a[i * n + k] / pivot;
                a[i * n + k] = l;
                for (int64_t c = k + 1; c < n; c++)
                    a[i * n + c] = a[i * n + c] - l * a[k * n + c];
            }
        } else if (info == 0) {
            info = k + 1;
        }
    }
    if (info != 0) return info;
    for (int64_t k = 0; k < n; k++)
        if (piv[k] != k) std::swap(b[k], b[piv[k]]);
    for (int64_t k = 0; k < n; k++)
        for (int64_t i = k + 1; i < n; i++)
            b[i] = b[i] - b[k] * a[i * n + k];
    for (int64_t k = n - 1; k >= 0; k--) {
        b[k] = b[k] / a[k * n + k];
        for (int64_t i = 0; i < k; i++)
            b[i] = b[i] - b[k] * a[i * n + k];
    }
    return 0;
}

// ---------------------------------------------------------------------------
// Generic dense integrators with caller-supplied SDEs (used by the unit-test
// goldens of test/tests.cpp; the LLG path below uses block forms).
// ---------------------------------------------------------------------------
typedef void (*sde_cb)(double *drift, double *diff, const double *x, double t, void *ctx);
typedef void (*sde_jac_cb)(double *a, double *b, double *adash, double *bdash,
                           const double *x, double ta, double tb, void *ctx);
typedef void (*fj_cb)(double *f, double *j, const double *x, void *ctx);

// integrator::heun, lib/integrators.cpp:372-405
void oracle_heun_dense(double *next, const double *x, const double *w, sde_cb sde, void *ctx,
                       int64_t n, int64_t nw, double t, double dt)
{
    std::vector<double> a(n), ta(n), b(n * nw), tb(n * nw);
    sde(a.data(), b.data(), x, t, ctx);
    for (int64_t i = 0; i < n; i++) {
        next[i] = x[i] + dt * a[i];
        for (int64_t j = 0; j < nw; j++)
            next[i] += b[j + i * nw] * w[j] * std::sqrt(dt);
    }
    sde(ta.data(), tb.data(), next, t + dt, ctx);
    for (int64_t i = 0; i < n; i++) {
        next[i] = x[i] + 0.5 * dt * (ta[i] + a[i]);
        for (int64_t j = 0; j < nw; j++)
            next[i] += 0.5 * w[j] * std::sqrt(dt) * (tb[j + i * nw] + b[j + i * nw]);
    }
}

// driver::heun, lib/integrators.cpp:429-457
void oracle_heun_driver(double *states, const double *x0, const double *wiener, sde_cb sde,
                        void *ctx, int64_t n_steps, int64_t n, int64_t nw, double dt)
{
    for (int64_t i = 0; i < n; i++) states[i] = x0[i];
    for (int64_t s = 0; s < n_steps; s++)
        oracle_heun_dense(states + (s + 1) * n, states + s * n, wiener + s * nw, sde, ctx, n,
                          nw, s * dt, dt);
}

// optimisation::newton_raphson_noinv, lib/optimisation.cpp:81-149
int oracle_newton_noinv(double *x_root, fj_cb fj, void *ctx, const double *x0, int64_t dim,
                        double eps, int64_t max_iter, int64_t *lapack_info)
{
    std::vector<double> x_tmp(dim), jac(dim * dim);
    for (int64_t i = 0; i < dim; i++) x_root[i] = x0[i];
    double tol = eps * oracle_nrm2(x_root, dim);
    double err = 2 * tol;
    int64_t iter = max_iter;
    *lapack_info = 0;
    while ((err > tol) && (iter-- > 0)) {
        for (int64_t i = 0; i < dim; i++) x_tmp[i] = x_root[i];
        fj(x_root, jac.data(), x_tmp.data(), ctx);
        for (int64_t i = 0; i < dim; i++) x_root[i] *= -1;
        *lapack_info = oracle_dgesv(dim, jac.data(), x_root);
        if (*lapack_info != 0) return ORACLE_SINGULAR;
        err = oracle_nrm2(x_root, dim);
        for (int64_t i = 0; i < dim; i++) x_root[i] += x_tmp[i];
    }
    return iter == -1 ? ORACLE_NEWTON_MAXITER : ORACLE_OK;
}

struct midpoint_ctx {
    sde_jac_cb sde; void *ctx;
    double *a, *b, *adash, *bdash;
    const double *x0, *dwm;
    double t, dt;
    int64_t n, w;
};

static void midpoint_fj(double *fout, double *jout, const double *in, void *vctx)
{
    midpoint_ctx *c = (midpoint_ctx *)vctx;
    const int64_t n = c->n, w = c->w;
    c->sde(c->a, c->b, c->adash, c->bdash, in, c->t + c->dt / 2, c->t, c->ctx);
    for (int64_t i = 0; i < n; i++) {
        fout[i] = in[i] - 0.5 * c->a[i] * c->dt - c->x0[i];
        for (int64_t j = 0; j < w; j++)
            fout[i] -= 0.5 * c->b[i * w + j] * c->dwm[j];
    }
    for (int64_t i = 0; i < n; i++)
        for (int64_t j = 0; j < n; j++) {
            jout[i * n + j] = (i == j) - 0.5 * c->adash[i * n + j];
            for (int64_t k = 0; k < w; k++)
                jout[i * n + j] -= 0.5 * c->bdash[i * w * n + k * n + j] * c->dwm[k];
        }
}

// integrator::implicit_midpoint, lib/integrators.cpp:576-651
int oracle_implicit_midpoint_dense(double *x, const double *x0, const double *dw,
                                   sde_jac_cb sde, void *ctx, int64_t n, int64_t w, double t,
                                   double dt, double eps, int64_t max_iter)
{
    std::vector<double> dwm(w), a(n), b(n * w), adash(n * n), bdash(n * w * n), guess(n);
    double k = 1000;
    double Ah = std::sqrt(2 * k * std::abs(std::log(dt)));
    for (int64_t i = 0; i < w; i++)
        dwm[i] = std::max(-Ah, std::min(Ah, dw[i])) * std::sqrt(dt);
    sde(a.data(), b.data(), adash.data(), bdash.data(), x0, t, t, ctx);
    for (int64_t i = 0; i < n; i++) {
        guess[i] = a[i] * dt;
        for (int64_t j = 0; j < w; j++) guess[i] += b[i * w + j] * dwm[j];
    }
    for (int64_t i = 0; i < n; i++) guess[i] = (guess[i] + x0[i]) / 2;
    midpoint_ctx c{sde, ctx, a.data(), b.data(), adash.data(), bdash.data(), x0, dwm.data(),
                   t, dt, n, w};
    int64_t info = 0;
    int flag = oracle_newton_noinv(x, midpoint_fj, &c, guess.data(), n, eps, max_iter, &info);
    for (int64_t i = 0; i < n; i++) x[i] = 2 * x[i] - x0[i];
    return flag + (int)info;
}

// driver::implicit_midpoint, lib/integrators.cpp:486-537
void oracle_implicit_driver(double *x, const double *x0, const double *dw, sde_jac_cb sde,
                            void *ctx, int64_t n, int64_t w, int64_t n_steps, double t0,
                            double dt, double eps, int64_t max_iter, int32_t *codes)
{
    double t = t0;
    for (int64_t i = 0; i < n; i++) x[i] = x0[i];
    for (int64_t s = 0; s < n_steps; s++) {
        t += dt;
        codes[s] = oracle_implicit_midpoint_dense(x + (s + 1) * n, x + s * n, dw + s * w, sde,
                                                  ctx, n, w, t, dt, eps, max_iter);
    }
}

// RngMtNorm (lib/rng.cpp:14-24): std::mt19937_64 + std::normal_distribution.
void oracle_mt_norm(uint64_t seed, double stddev, int64_t count, double *out)
{
    std::mt19937_64 gen(seed);
    std::normal_distribution<double> dist(0, stddev);
    for (int64_t i = 0; i < count; i++) out[i] = dist(gen);
}

// Néel-Brown two-state rates: lib/dom.cpp:33-59
void oracle_dom_transition_matrix(double *W, double k, double v, double T, double h, double ms,
                                  double alpha)
{
    double sigma = k * v / KB / T;
    double taun = v * ms * (1 + alpha * alpha) / 2.0 / GYROMAG / alpha / KB / T;
    double e1 = sigma * (1 - h) * (1 - h);
    double e2 = sigma * (1 + h) * (1 + h);
    double pref = taun * std::sqrt(M_PI) / std::pow(sigma, 1.5) / (1 - h * h);
    double r1 = 1.0 / pref * (1 - h) * std::exp(-e1);
    double r2 = 1.0 / pref * (1 + h) * std::exp(-e2);
    W[0] = -r2; W[1] = r1; W[2] = r2; W[3] = -r1;
}

// ---------------------------------------------------------------------------
// The sLLG cluster path in reduced units: lib/simulation.cpp:132-429.
// ---------------------------------------------------------------------------
typedef struct {
    int64_t n;                    // particles in the cluster
    const double *sr;             // thermal field strength per particle [n]
    const double *k_red;          // reduced anisotropy constants [n]
    const double *v_red;          // reduced volumes [n]
    const double *axes;           // anisotropy unit axes [n][3]
    const double *m0;             // initial magnetisation [n][3]
    const double *unit_dist;      // [n][n][3]
    const double *dist_mag;       // reduced distance magnitudes [n][n]
    int32_t field_shape;
    double happ, fapp;            // reduced field amplitude and frequency
    double k_av, v_av, alpha, ms; // average anisotropy, volume; damping; Ms
    double dt, end_time;          // reduced
    int32_t renorm, interactions, use_implicit;
    double eps;
    int64_t max_iter;             // Newton limit (reference: 1000, simulation.cpp:204)
    int64_t max_samples;
} oracle_reduced_t;

namespace {

struct Noise {
    // Either injected increments (RngArray, rng.cpp:67-94) or RngMtNorm.
    const double *arr = nullptr;
    int64_t len = 0, pos = 0;
    std::mt19937_64 gen;
    std::normal_distribution<double> dist{0.0, 1.0};
    bool exhausted = false;
    explicit Noise(uint64_t seed) : gen(seed) {}
    double get()
    {
        if (arr) {
            if (pos < len) return arr[pos++];
            exhausted = true;  // the reference throws std::out_of_range here
            return 0.0;
        }
        return dist(gen);
    }
};

struct Cluster {
    const oracle_reduced_t *p;
    int64_t n;
    std::vector<double> dist_cubes;  // [n][n]
    std::vector<double> hj_eff;      // [n][9] field-Jacobian block as the reference reads it
    double pref;

    explicit Cluster(const oracle_reduced_t *p_) : p(p_), n(p_->n)
    {
        // simulation.cpp:259-263
        dist_cubes.resize(n * n);
        for (int64_t i = 0; i < n * n; i++) dist_cubes[i] = std::pow(p->dist_mag[i], 3);
        pref = oracle_dipolar_prefactor(p->ms, p->k_av);
        // simulation.cpp:296-303 builds the dense 3N x 3N anisotropy
        // Jacobian; llg.cpp:378-389 hands drift_jacobian the pointer
        // hj + 3n and reads 9 consecutive doubles from it, i.e. flat
        // indices 3n .. 3n+8 of the dense row-major matrix.
        const int64_t n3 = 3 * n;
        hj_eff.assign(n * 9, 0.0);
        for (int64_t q = 0; q < n; q++)
            for (int64_t k = 0; k < 9; k++) {
                int64_t f = 3 * q + k;
                int64_t r = f / n3, c = f % n3;
                hj_eff[q * 9 + k] =
                    (r / 3 == c / 3) ? p->k_red[r / 3] * p->axes[r] * p->axes[c] : 0.0;
            }
    }

    // heff_func, simulation.cpp:271-290
    void field(double *h, const double *m, double t) const
    {
        for (int64_t i = 0; i < 3 * n; i++) h[i] = 0.0;
        for (int64_t q = 0; q < n; q++) {  // field.cpp:116-132
            double k_red = p->k_red[q];
            const double *ax = p->axes + 3 * q;
            const double *s = m + 3 * q;
            double dot = s[0] * ax[0] + s[1] * ax[1] + s[2] * ax[2];
            dot *= k_red;
            h[3 * q + 0] += dot * ax[0];
            h[3 * q + 1] += dot * ax[1];
            h[3 * q + 2] += dot * ax[2];
        }
        double happ = oracle_field_value(p->field_shape, t, p->happ, p->fapp);  // field.cpp:81-88
        for (int64_t q = 0; q < n; q++) h[q * 3 + 2] += happ;
        if (p->interactions)
            for (int64_t i = 0; i < n; i++) {
                for (int64_t j = 0; j < i; j++)
                    oracle_dipolar_p2p(h + i * 3, p->v_red[j], dist_cubes[i * n + j], m + j * 3,
                                       p->unit_dist + i * n * 3 + j * 3, pref);
                for (int64_t j = i + 1; j < n; j++)
                    oracle_dipolar_p2p(h + i * 3, p->v_red[j], dist_cubes[i * n + j], m + j * 3,
                                       p->unit_dist + i * n * 3 + j * 3, pref);
            }
    }

    // sde_no_jacs: llg.cpp:332-348 (drift [3n], block diffusion [n][9])
    void sde(double *a, double *b, double *h, const double *m, double t) const
    {
        field(h, m, t);
        for (int64_t q = 0; q < n; q++) {
            oracle_llg_drift(a + 3 * q, m + 3 * q, p->alpha, h + 3 * q);
            oracle_llg_diffusion(b + 9 * q, m + 3 * q, p->sr[q], p->alpha);
        }
    }

    // integrator::heun on the block-diagonal diffusion: integrators.cpp:372-405
    void heun(double *next, const double *x, const double *w, double t, double dt,
              std::vector<double> &ws) const
    {
        const int64_t n3 = 3 * n;
        double *a = ws.data(), *ta = a + n3, *h = ta + n3, *b = h + n3, *tb = b + 9 * n;
        sde(a, b, h, x, t);
        for (int64_t i = 0; i < n3; i++) {
            int64_t q = i / 3, r = i % 3;
            next[i] = x[i] + dt * a[i];
            for (int64_t c = 0; c < 3; c++)
                next[i] += b[9 * q + 3 * r + c] * w[3 * q + c] * std::sqrt(dt);
        }
        sde(ta, tb, h, next, t + dt);
        for (int64_t i = 0; i < n3; i++) {
            int64_t q = i / 3, r = i % 3;
            next[i] = x[i] + 0.5 * dt * (ta[i] + a[i]);
            for (int64_t c = 0; c < 3; c++)
                next[i] += 0.5 * w[3 * q + c] * std::sqrt(dt) *
                           (tb[9 * q + 3 * r + c] + b[9 * q + 3 * r + c]);
        }
    }

    // multi_stochastic_llg_jacobians_field_update, llg.cpp:453-481, block form:
    // a [3n], b [n][9], adash [n][9], bdash [n][27]
    void sde_jac(double *a, double *b, double *adash, double *bdash, double *h,
                 const double *m, double t) const
    {
        sde(a, b, h, m, t);
        for (int64_t q = 0; q < n; q++) {
            oracle_llg_drift_jacobian(adash + 9 * q, m + 3 * q, p->alpha, h + 3 * q,
                                      hj_eff.data() + 9 * q);
            oracle_llg_diffusion_jacobian(bdash + 27 * q, m + 3 * q, p->sr[q], p->alpha);
        }
    }

    // integrator::implicit_midpoint with newton_raphson_noinv on the
    // block-diagonal Jacobian (integrators.cpp:576-651, optimisation.cpp:81-149).
    // Partial pivoting of the dense LU never leaves a 3x3 diagonal block,
    // so the dense solve equals n independent 3x3 solves.
    int implicit(double *x, const double *x0, const double *dw, double t, double dt,
                 double Ah, std::vector<double> &ws) const
    {
        const int64_t n3 = 3 * n;
        std::vector<double> dwm(n3), a(n3), b(9 * n), adash(9 * n), bdash(27 * n), h(n3),
            guess(n3), xt(n3), F(n3), J(9 * n);
        (void)ws;
        for (int64_t i = 0; i < n3; i++)
            dwm[i] = std::max(-Ah, std::min(Ah, dw[i])) * std::sqrt(dt);
        sde_jac(a.data(), b.data(), adash.data(), bdash.data(), h.data(), x0, t);
        for (int64_t i = 0; i < n3; i++) {
            int64_t q = i / 3, r = i % 3;
            guess[i] = a[i] * dt;
            for (int64_t c = 0; c < 3; c++) guess[i] += b[9 * q + 3 * r + c] * dwm[3 * q + c];
        }
        for (int64_t i = 0; i < n3; i++) guess[i] = (guess[i] + x0[i]) / 2;

        // newton_raphson_noinv
        for (int64_t i = 0; i < n3; i++) x[i] = guess[i];
        double tol = p->eps * oracle_nrm2(x, n3);
        double err = 2 * tol;
        int64_t iter = p->max_iter;
        int flag = ORACLE_OK;
        while ((err > tol) && (iter-- > 0)) {
            for (int64_t i = 0; i < n3; i++) xt[i] = x[i];
            // FJ at time t + dt/2 (integrators.cpp:617-637)
            sde_jac(a.data(), b.data(), adash.data(), bdash.data(), h.data(), xt.data(),
                    t + dt / 2);
            for (int64_t i = 0; i < n3; i++) {
                int64_t q = i / 3, r = i % 3;
                F[i] = xt[i] - 0.5 * a[i] * dt - x0[i];
                for (int64_t c = 0; c < 3; c++) F[i] -= 0.5 * b[9 * q + 3 * r + c] * dwm[3 * q + c];
            }
            for (int64_t q = 0; q < n; q++)
                for (int64_t r = 0; r < 3; r++)
                    for (int64_t c = 0; c < 3; c++) {
                        double v = (r == c) - 0.5 * adash[9 * q + 3 * r + c];
                        for (int64_t k = 0; k < 3; k++)
                            v -= 0.5 * bdash[27 * q + 9 * r + 3 * k + c] * dwm[3 * q + k];
                        J[9 * q + 3 * r + c] = v;
                    }
            for (int64_t i = 0; i < n3; i++) x[i] = F[i] * -1;
            // dense dgesv == block solves; the first zero pivot (in dense
            // column order) aborts the whole solve with b unchanged.
            int64_t info = 0;
            std::vector<double> sol(x, x + n3);
            for (int64_t q = 0; q < n && info == 0; q++) {
                int64_t bi = oracle_dgesv(3, J.data() + 9 * q, sol.data() + 3 * q);
                if (bi != 0) info = 3 * q + bi;
            }
            if (info != 0) { flag = ORACLE_SINGULAR; break; }
            for (int64_t i = 0; i < n3; i++) x[i] = sol[i];
            err = oracle_nrm2(x, n3);
            for (int64_t i = 0; i < n3; i++) x[i] += xt[i];
        }
        if (flag == ORACLE_OK && iter == -1) flag = ORACLE_NEWTON_MAXITER;
        for (int64_t i = 0; i < n3; i++) x[i] = 2 * x[i] - x0[i];
        return flag;
    }
};

}  // namespace

// Reduced full_dynamics for one cluster: simulation.cpp:132-429.
// mx/my/mz: [n][max_samples]; field, time: [max_samples].  noise: injected
// increments consumed 3n per step (particle-major xyz, simulation.cpp:358-359),
// or NULL to draw from RngMtNorm(seed, 1).  Returns the status bits;
// *steps_out receives the number of integration steps taken.
int oracle_full_dynamics_reduced(const oracle_reduced_t *p, const double *noise,
                                 int64_t noise_len, uint64_t seed, double *mx, double *my,
                                 double *mz, double *field, double *time, int64_t *steps_out)
{
    const int64_t n = p->n, n3 = 3 * n;
    if (p->max_samples < 1) return -1;
    Cluster cl(p);
    Noise rng(seed);
    if (noise) { rng.arr = noise; rng.len = noise_len; }

    const int64_t N_samples = p->max_samples;
    const double sampling_time = p->end_time / (N_samples - 1);
    for (int64_t q = 0; q < n; q++) {  // simulation.cpp:206-219
        time[0] = 0;
        field[0] = oracle_field_value(p->field_shape, 0, p->happ, p->fapp);
        mx[q * N_samples] = p->m0[3 * q + 0];
        my[q * N_samples] = p->m0[3 * q + 1];
        mz[q * N_samples] = p->m0[3 * q + 2];
    }
    std::vector<double> pstate(n3), nstate(p->m0, p->m0 + n3), wiener(n3), ws(27 * n);
    const double Ah = std::sqrt(2 * 1000.0 * std::abs(std::log(p->dt)));  // integrators.cpp:599-600
    unsigned int step = 0;
    double t = 0;
    int status = ORACLE_OK;
    for (unsigned int sample = 1; sample < N_samples; sample++) {  // simulation.cpp:342-406
        while (t <= sample * sampling_time) {
            for (int64_t i = 0; i < n3; i++) pstate[i] = nstate[i];
            step++;
            t = step * p->dt;
            for (int64_t i = 0; i < n3; i++) wiener[i] = rng.get();
            if (rng.exhausted) { status |= ORACLE_NOISE_EXHAUSTED; goto done; }
            if (p->use_implicit)
                status |= cl.implicit(nstate.data(), pstate.data(), wiener.data(), t, p->dt, Ah,
                                      ws);
            else
                cl.heun(nstate.data(), pstate.data(), wiener.data(), t, p->dt, ws);
            if (p->renorm)
                for (int64_t o = 0; o < n3; o += 3) {
                    double norm = oracle_nrm2(nstate.data() + o, 3);
                    for (int c = 0; c < 3; c++) nstate[o + c] = nstate[o + c] / norm;
                }
        }
        time[sample] = sample * sampling_time;
        field[sample] = oracle_field_value(p->field_shape, sample * sampling_time, p->happ,
                                           p->fapp);
        for (int64_t q = 0; q < n; q++) {
            mx[q * N_samples + sample] = pstate[3 * q + 0];
            my[q * N_samples + sample] = pstate[3 * q + 1];
            mz[q * N_samples + sample] = pstate[3 * q + 2];
        }
    }
done:
    for (int64_t i = 0; i < n3; i++)
        if (!std::isfinite(nstate[i])) status |= ORACLE_NONFINITE;
    if (steps_out) *steps_out = step;
    return status;
}

// Physical-unit set-up: simulation.cpp:476-583.  Fills the reduced
// parameter block (arrays are written to caller storage) and the unit
// conversions.  out_scalars = {k_av, v_av, H_k, time_factor, dt_red,
// end_red, happ, fapp}.
void oracle_reduce_parameters(int64_t n, const double *radius, const double *anisotropy,
                              const double *location, double ms, double damping,
                              double temperature, double time_step, double end_time,
                              double field_amplitude, double field_frequency, double *sr,
                              double *k_red, double *v_red, double *unit_dist,
                              double *dist_mag, double *out_scalars)
{
    std::vector<double> volume(n);
    for (int64_t i = 0; i < n; i++)
        volume[i] = 4.0 / 3.0 * M_PI * radius[i] * radius[i] * radius[i];
    double v_sum = 0.0;
    for (int64_t i = 0; i < n; i++) v_sum += volume[i];
    double average_volume = v_sum / n;
    for (int64_t i = 0; i < n; i++) v_red[i] = volume[i] / average_volume;
    double k_sum = 0.0;
    for (int64_t i = 0; i < n; i++) k_sum += anisotropy[i];
    double average_anisotropy = k_sum / n;
    for (int64_t i = 0; i < n; i++) k_red[i] = anisotropy[i] / average_anisotropy;
    double anisotropy_field = 2 * average_anisotropy / MU0 / ms;
    double time_factor = GYROMAG * MU0 * anisotropy_field / (1 + damping * damping);
    for (int64_t i = 0; i < n; i++)
        sr[i] = std::sqrt(damping * KB * temperature / (average_anisotropy * volume[i]) /
                          (1 + damping * damping));
    std::vector<double> vec(n * n * 3);
    oracle_pairwise_geometry(location, n, vec.data(), dist_mag, unit_dist);
    double scale = std::pow(average_volume, 1. / 3);
    for (int64_t i = 0; i < n * n; i++) dist_mag[i] /= scale;
    out_scalars[0] = average_anisotropy;
    out_scalars[1] = average_volume;
    out_scalars[2] = anisotropy_field;
    out_scalars[3] = time_factor;
    out_scalars[4] = time_step * time_factor;
    out_scalars[5] = end_time * time_factor;
    out_scalars[6] = field_amplitude / anisotropy_field;
    out_scalars[7] = field_frequency / time_factor;
}

// Physical full_dynamics for one cluster: simulation.cpp:476-624.
// Outputs in SI (A/m, s).  noise/noise_len as in the reduced form.
int oracle_full_dynamics(int64_t n, const double *radius, const double *anisotropy,
                         const double *axes, const double *m0, const double *location,
                         double ms, double damping, double temperature, int32_t renorm,
                         int32_t interactions, int32_t use_implicit, double eps,
                         double time_step, double end_time, int64_t max_samples, int64_t seed,
                         int32_t field_shape, double field_amplitude, double field_frequency,
                         int64_t max_iter, const double *noise, int64_t noise_len, double *mx,
                         double *my, double *mz, double *field, double *time,
                         int64_t *steps_out)
{
    std::vector<double> sr(n), k_red(n), v_red(n), unit(n * n * 3), mag(n * n);
    double sc[8];
    oracle_reduce_parameters(n, radius, anisotropy, location, ms, damping, temperature,
                             time_step, end_time, field_amplitude, field_frequency, sr.data(),
                             k_red.data(), v_red.data(), unit.data(), mag.data(), sc);
    oracle_reduced_t p;
    p.n = n; p.sr = sr.data(); p.k_red = k_red.data(); p.v_red = v_red.data();
    p.axes = axes; p.m0 = m0; p.unit_dist = unit.data(); p.dist_mag = mag.data();
    p.field_shape = field_shape; p.happ = sc[6]; p.fapp = sc[7];
    p.k_av = sc[0]; p.v_av = sc[1]; p.alpha = damping; p.ms = ms;
    p.dt = sc[4]; p.end_time = sc[5];
    p.renorm = renorm; p.interactions = interactions; p.use_implicit = use_implicit;
    p.eps = eps; p.max_iter = max_iter; p.max_samples = max_samples;
    int st = oracle_full_dynamics_reduced(&p, noise, noise_len, (uint64_t)seed, mx, my, mz,
                                          field, time, steps_out);
    const double H_k = sc[2], tf = sc[3];
    for (int64_t q = 0; q < n; q++)  // simulation.cpp:610-621
        for (int64_t i = 0; i < max_samples; i++) {
            if (q == 0) { time[i] /= tf; field[i] *= H_k; }
            mx[q * max_samples + i] *= ms;
            my[q * max_samples + i] *= ms;
            mz[q * max_samples + i] *= ms;
        }
    return st;
}

// Ensemble of clusters sharing one geometry, one member per OpenMP task
// (the CPU baseline; the reference fans members out over joblib processes,
// magpy/model.py:202-207).  Outputs [E][n][S]; field/time [S] (member 0).
// noise: NULL or [E][noise_per_member].  statuses: [E].  n_threads<=0 uses
// the OpenMP default.
int oracle_ensemble(int64_t E, int64_t n, const double *radius, const double *anisotropy,
                    const double *axes, const double *m0, const double *location, double ms,
                    double damping, double temperature, int32_t renorm, int32_t interactions,
                    int32_t use_implicit, double eps, double time_step, double end_time,
                    int64_t max_samples, const int64_t *seeds, int32_t field_shape,
                    double field_amplitude, double field_frequency, int64_t max_iter,
                    const double *noise, int64_t noise_per_member, int32_t n_threads,
                    double *mx, double *my, double *mz, double *field, double *time,
                    int32_t *statuses)
{
#ifdef _OPENMP
    if (n_threads > 0) omp_set_num_threads(n_threads);
#endif
    const int64_t S = max_samples;
#pragma omp parallel
    {
        std::vector<double> f(S), tm(S);
#pragma omp for schedule(dynamic)
        for (int64_t e = 0; e < E; e++) {
            int64_t steps = 0;
            statuses[e] = oracle_full_dynamics(
                n, radius, anisotropy, axes, m0, location, ms, damping, temperature, renorm,
                interactions, use_implicit, eps, time_step, end_time, max_samples, seeds[e],
                field_shape, field_amplitude, field_frequency, max_iter,
                noise ? noise + e * noise_per_member : nullptr, noise_per_member,
                mx + e * n * S, my + e * n * S, mz + e * n * S, f.data(), tm.data(), &steps);
            if (e == 0) {
                std::memcpy(field, f.data(), S * sizeof(double));
                std::memcpy(time, tm.data(), S * sizeof(double));
            }
        }
    }
    return 0;
}

int oracle_max_threads()
{
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

}  // extern "C"
