// sllg_fp64.cu -- the FP64-faithful sLLG ensemble kernel (compiled with
// -fmad=false).
//
// One thread per particle.  A member of n <= 32 particles occupies n
// consecutive lanes of a warp (32/n members per warp) and synchronises with
// __syncwarp on its lane mask; a member of n > 32 particles is one CTA.  The
// member's state stays in registers for the whole run; particles exchange
// their moments through shared memory for the dipolar sum.  Per step the
// kernel follows lib/simulation.cpp:342-405: copy the state, advance the
// step counter, draw 3n increments, take one Heun (lib/integrators.cpp:372)
// or implicit-midpoint (lib/integrators.cpp:576) step at t = step*dt,
// optionally renormalise, and write the zero-order-hold sample.
#include <type_traits>
#include "common.cuh"
#include "llg64.cuh"
#include "plan.hpp"

namespace magpy {
namespace {

struct Particle {
    double ax[3];
    double k, sr, alpha;
    double hj[9];
};

struct Member {
    const MemberDev *d;
    const double *pt, *rt;  // pair tables of the member's cluster
    const float4 *pr;       // FP32 pair table (r0, r1, r2, P), [N][N], index j*n + q
    double *sm;             // [3n] shared moments
    float *smf;             // [3n] shared FP32 moments (FP32 dipolar sum)
    double *red;            // [p2] shared reduction buffer
    int n, q, p2;
    bool active;
    MemberSync ms;
};

// Shared-memory doubles per member: moments, reduction buffer and, with the
// FP32 dipolar sum, FP32 moments.
__host__ __device__ inline int slot_doubles(int n, int p2, bool dip32)
{
    return 3 * n + p2 + (dip32 ? (3 * n + 1) / 2 : 0);
}

// Dipolar sum in FP32 from the (r0, r1, r2, P) pair table: fused products,
// FP32 partial sums over 32 sources, added in FP64.  The mixed-precision
// implicit mode uses it inside the FP64 Newton solve.
__device__ inline void dipolar32(const Member &M, double h[3])
{
    const int n = M.n, q = M.q;
    double H0 = 0.0, H1 = 0.0, H2 = 0.0;
    for (int j0 = 0; j0 < n; j0 += 32) {
        const int j1 = min(n, j0 + 32);
        float h0 = 0.f, h1 = 0.f, h2 = 0.f;
        for (int j = j0; j < j1; j++) {
            const float4 r = __ldg(M.pr + (size_t)j * n + q);  // P = 0 on the diagonal
            const float mj0 = M.smf[3 * j], mj1 = M.smf[3 * j + 1], mj2 = M.smf[3 * j + 2];
            const float d3 = 3.f * __fmaf_rn(mj2, r.z, __fmaf_rn(mj1, r.y, __fmul_rn(mj0, r.x)));
            h0 = __fmaf_rn(r.w, __fmaf_rn(d3, r.x, -mj0), h0);
            h1 = __fmaf_rn(r.w, __fmaf_rn(d3, r.y, -mj1), h1);
            h2 = __fmaf_rn(r.w, __fmaf_rn(d3, r.z, -mj2), h2);
        }
        H0 += (double)h0;
        H1 += (double)h1;
        H2 += (double)h2;
    }
    h[0] += H0;
    h[1] += H1;
    h[2] += H2;
}

// Effective field of one particle: lib/simulation.cpp:271-290 (anisotropy,
// lib/field.cpp:116-132; Zeeman along z, :81-88; dipolar pair sum, :187-225).
template <bool DIP32>
__device__ void eff_field(const Member &M, const Particle &pa, double h[3], const double s[3],
                          double t)
{
    h[0] = 0.0; h[1] = 0.0; h[2] = 0.0;
    double dot = s[0] * pa.ax[0] + s[1] * pa.ax[1] + s[2] * pa.ax[2];
    dot *= pa.k;
    h[0] += dot * pa.ax[0];
    h[1] += dot * pa.ax[1];
    h[2] += dot * pa.ax[2];
    h[2] += f64::field_value(M.d->shape, t, M.d->happ, M.d->fapp);
    if (DIP32 && M.d->interactions && M.n > 1) {
        if (M.active)
            for (int c = 0; c < 3; c++) M.smf[3 * M.q + c] = (float)s[c];
        M.ms.sync();
        if (M.active) dipolar32(M, h);
        M.ms.sync();
    } else if (M.d->interactions && M.n > 1) {
        if (M.active) {
            M.sm[3 * M.q + 0] = s[0];
            M.sm[3 * M.q + 1] = s[1];
            M.sm[3 * M.q + 2] = s[2];
        }
        M.ms.sync();
        if (M.active) {
            const int n = M.n, q = M.q;
            for (int j = 0; j < n; j++) {
                if (j == q) continue;
                const double mj0 = M.sm[3 * j + 0], mj1 = M.sm[3 * j + 1], mj2 = M.sm[3 * j + 2];
                const double P = __ldg(M.pt + (size_t)j * n + q);
                const double r0 = __ldg(M.rt + ((size_t)0 * n + j) * n + q);
                const double r1 = __ldg(M.rt + ((size_t)1 * n + j) * n + q);
                const double r2 = __ldg(M.rt + ((size_t)2 * n + j) * n + q);
                const double d = mj0 * r0 + mj1 * r1 + mj2 * r2;
                h[0] += P * (3 * d * r0 - mj0);
                h[1] += P * (3 * d * r1 - mj1);
                h[2] += P * (3 * d * r2 - mj2);
            }
        }
        M.ms.sync();
    }
}

// Member-wide 2-norm with the shim's order: per-particle sequential sum of
// squares, then a pairwise tree over a power-of-two padded particle index.
__device__ double member_nrm2(const Member &M, const double x[3])
{
    if (M.active) {
        double s = 0.0;
        s = s + x[0] * x[0];
        s = s + x[1] * x[1];
        s = s + x[2] * x[2];
        M.red[M.q] = s;
        if (M.n + M.q < M.p2) M.red[M.n + M.q] = 0.0;
    }
    M.ms.sync();
    for (int stride = M.p2 / 2; stride >= 1; stride >>= 1) {
        if (M.q < stride) M.red[M.q] = M.red[M.q] + M.red[M.q + stride];
        M.ms.sync();
    }
    double r = sqrt(M.red[0]);
    M.ms.sync();
    return r;
}

__device__ inline bool member_any(const Member &M, bool pred)
{
    if (M.ms.cta) return __syncthreads_or(pred) != 0;
    return __any_sync(M.ms.mask, pred) != 0;
}

// integrator::heun, lib/integrators.cpp:372-405, on the particle's 3x3 block.
template <bool DIP32>
__device__ void heun_step(const Member &M, const Particle &pa, double x[3],
                          const double px[3], const double w[3], double t)
{
    const double dt = M.d->dt, sq = M.d->sqrt_dt;
    double h[3], a[3], b[9], xt[3];
    eff_field<DIP32>(M, pa, h, px, t);
    f64::drift(a, px, pa.alpha, h);
    f64::diffusion(b, px, pa.sr, pa.alpha);
    for (int r = 0; r < 3; r++) {
        xt[r] = px[r] + dt * a[r];
        for (int c = 0; c < 3; c++) xt[r] += b[3 * r + c] * w[c] * sq;
    }
    double ta[3], tb[9];
    eff_field<DIP32>(M, pa, h, xt, t + dt);
    f64::drift(ta, xt, pa.alpha, h);
    f64::diffusion(tb, xt, pa.sr, pa.alpha);
    for (int r = 0; r < 3; r++) {
        x[r] = px[r] + 0.5 * dt * (ta[r] + a[r]);
        for (int c = 0; c < 3; c++) x[r] += 0.5 * w[c] * sq * (tb[3 * r + c] + b[3 * r + c]);
    }
}

// integrator::implicit_midpoint (lib/integrators.cpp:576-651) with
// optimisation::newton_raphson_noinv (lib/optimisation.cpp:81-149).  The
// Jacobian is block-diagonal (the field Jacobian ignores the dipolar term,
// lib/simulation.cpp:292-303), so the dense dgesv is n independent 3x3
// solves; the convergence norm couples the whole member.
template <bool DIP32>
__device__ int32_t implicit_step(const Member &M, const Particle &pa, double x[3],
                                 const double px[3], const double w[3], double t)
{
    const double dt = M.d->dt, sq = M.d->sqrt_dt, Ah = M.d->Ah;
    double dwm[3];
    for (int c = 0; c < 3; c++) {
        double lo = (w[c] < Ah) ? w[c] : Ah;         // std::min(Ah, dw)
        dwm[c] = ((-Ah < lo) ? lo : -Ah) * sq;       // std::max(-Ah, .) * sqrt(dt)
    }
    double h[3], a[3], b[9];
    eff_field<DIP32>(M, pa, h, px, t);
    f64::drift(a, px, pa.alpha, h);
    f64::diffusion(b, px, pa.sr, pa.alpha);
    for (int r = 0; r < 3; r++) {
        double g = a[r] * dt;
        for (int c = 0; c < 3; c++) g += b[3 * r + c] * dwm[c];
        x[r] = (g + px[r]) / 2;
    }
    const double tol = M.d->eps * member_nrm2(M, x);
    double err = 2 * tol;
    int64_t iter = M.d->max_iter;
    int32_t flag = ST_OK;
    const double tm = t + dt / 2;
    while ((err > tol) && (iter-- > 0)) {
        double xt[3] = {x[0], x[1], x[2]};
        eff_field<DIP32>(M, pa, h, xt, tm);
        f64::drift(a, xt, pa.alpha, h);
        f64::diffusion(b, xt, pa.sr, pa.alpha);
        // The residual F is FP64 in both modes (it defines the root); the
        // quasi-Jacobian only steers the iteration, and the mixed mode forms
        // it and solves with it in FP32 (JT).
        using JT = typename std::conditional<DIP32, float, double>::type;
        JT adash[9], bdash[27], J[9];
        double F[3];
        {
            const JT xj[3] = {(JT)xt[0], (JT)xt[1], (JT)xt[2]};
            const JT hjv[3] = {(JT)h[0], (JT)h[1], (JT)h[2]};
            JT hjj[9];
            for (int k = 0; k < 9; k++) hjj[k] = (JT)pa.hj[k];
            f64::drift_jacobian<JT>(adash, xj, (JT)pa.alpha, hjv, hjj);
            f64::diffusion_jacobian<JT>(bdash, xj, (JT)pa.sr, (JT)pa.alpha);
        }
        for (int r = 0; r < 3; r++) {
            F[r] = xt[r] - 0.5 * a[r] * dt - px[r];
            for (int c = 0; c < 3; c++) F[r] -= 0.5 * b[3 * r + c] * dwm[c];
        }
        for (int r = 0; r < 3; r++)
            for (int c = 0; c < 3; c++) {
                JT v = (JT)(r == c) - (JT)0.5 * adash[3 * r + c];
                for (int k = 0; k < 3; k++) v -= (JT)0.5 * bdash[9 * r + 3 * k + c] * (JT)dwm[k];
                J[3 * r + c] = v;
            }
        double sol[3] = {F[0] * -1, F[1] * -1, F[2] * -1};
        for (int r = 0; r < 3; r++) x[r] = sol[r];
        JT solj[3] = {(JT)sol[0], (JT)sol[1], (JT)sol[2]};
        int info = M.active ? f64::solve3<JT>(J, solj) : 0;
        if (member_any(M, info != 0)) { flag = ST_SINGULAR; break; }
        for (int r = 0; r < 3; r++) x[r] = (double)solj[r];
        err = member_nrm2(M, x);
        for (int r = 0; r < 3; r++) x[r] += xt[r];
    }
    if (flag == ST_OK && iter == -1) flag = ST_NEWTON_MAXITER;
    for (int r = 0; r < 3; r++) x[r] = 2 * x[r] - px[r];
    return flag;
}

// MAXT: the largest CTA of the instantiation (256 for warp-packed members,
// 512 or 1024 for one member per CTA), so that the register budget of a
// thread never exceeds what a full CTA may use.
template <bool IMPLICIT, bool DIP32, int MAXT>
__global__ void __launch_bounds__(MAXT) sllg_fp64_kernel(DevPlan p)
{
    extern __shared__ double smem[];
    const int n = p.n;
    int p2 = 1;
    while (p2 < n) p2 <<= 1;
    const int slot_size = slot_doubles(n, p2, DIP32);

    Member M;
    int64_t e;
    if (n > 32) {
        e = blockIdx.x;
        M.q = threadIdx.x;
        M.active = M.q < n;
        M.ms.cta = true;
        M.ms.mask = 0xffffffffu;
        M.sm = smem;
    } else {
        const int mpw = (p.members_per_warp > 0 && p.members_per_warp < 32 / n) ? p.members_per_warp : 32 / n;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const int sub = lane / n;
        const int slot = warp * mpw + sub;
        e = (int64_t)blockIdx.x * ((blockDim.x >> 5) * mpw) + slot;
        if (sub >= mpw || e >= p.E) return;  // whole member leaves together
        M.q = lane % n;
        M.active = true;
        M.ms.cta = false;
        M.ms.mask = (n == 32) ? 0xffffffffu : (((1u << n) - 1u) << (sub * n));
        M.sm = smem + (size_t)slot * slot_size;
    }
    M.red = M.sm + 3 * n;
    M.smf = (float *)(M.red + p2);
    M.n = n;
    M.p2 = p2;
    const MemberDev *md = p.members + e;
    M.d = md;
    M.pt = p.pt + md->cluster_off;
    M.rt = p.rt + 3 * md->cluster_off;
    M.pr = DIP32 ? p.pr + md->cluster_off : nullptr;

    const int64_t P = p.P;
    const int64_t g = md->pbase + (M.active ? M.q : 0);
    Particle pa;
    double x[3], px[3];
    for (int c = 0; c < 3; c++) {
        pa.ax[c] = p.axes[c * P + g];
        x[c] = p.m0[c * P + g];
        px[c] = x[c];
    }
    pa.k = p.k_red[g];
    pa.sr = p.sr[g];
    pa.alpha = md->alpha;
    if (IMPLICIT)
        for (int k = 0; k < 9; k++) pa.hj[k] = p.hj[k * P + g];
    const double scale = p.out_scale[e];
    const int64_t S = p.S;
    const int64_t *sched = p.sched + md->sched_off;
    const double *noise = p.noise ? p.noise + md->noise_off : nullptr;
    const int64_t per_step = 3 * (int64_t)n;

    if (M.active && p.mx) {  // sample 0: the initial state, simulation.cpp:212-219
        p.mx[g] = x[0] * scale;
        p.my[g] = x[1] * scale;
        p.mz[g] = x[2] * scale;
    }
    int32_t status = ST_OK;
    uint64_t step = 0;
    int64_t s = 1;
    for (; s < S; s++) {
        const int64_t ks = sched[s];
        while ((int64_t)step < ks) {
            px[0] = x[0]; px[1] = x[1]; px[2] = x[2];
            step++;
            const double t = (double)step * md->dt;
            double w[3];
            if (noise) {
                if ((int64_t)step * per_step > md->noise_len) {
                    status |= ST_NOISE_EXHAUSTED;
                    step--;
                    goto finished;
                }
                const double *wp = noise + (int64_t)(step - 1) * per_step + 3 * M.q;
                w[0] = wp[0]; w[1] = wp[1]; w[2] = wp[2];
            } else {
                Normals4 r = wiener_normals(md->seed, step, (uint32_t)M.q);
                w[0] = r.a; w[1] = r.b; w[2] = r.c;
            }
            if (IMPLICIT) status |= implicit_step<DIP32>(M, pa, x, px, w, t);
            else heun_step<DIP32>(M, pa, x, px, w, t);
            if (md->renorm) {  // simulation.cpp:379-387
                double s2 = 0.0;
                s2 = s2 + x[0] * x[0];
                s2 = s2 + x[1] * x[1];
                s2 = s2 + x[2] * x[2];
                const double norm = sqrt(s2);
                for (int c = 0; c < 3; c++) x[c] = x[c] / norm;
            }
        }
        if (M.active && p.mx) {  // zero-order hold, simulation.cpp:398-405
            const int64_t o = s * P + g;
            p.mx[o] = px[0] * scale;
            p.my[o] = px[1] * scale;
            p.mz[o] = px[2] * scale;
        }
    }
finished:
    if (M.active && p.mx)  // samples a stopped member never reached
        for (; s < S; s++) {
            const int64_t o = s * P + g;
            p.mx[o] = NAN; p.my[o] = NAN; p.mz[o] = NAN;
        }
    bool bad = M.active && !(isfinite(x[0]) && isfinite(x[1]) && isfinite(x[2]));
    if (member_any(M, bad)) status |= ST_NONFINITE;
    if (M.q == 0) {
        if (p.status) p.status[e] = status;
        if (p.steps) p.steps[e] = (int64_t)step;
    }
}

}  // namespace

cudaError_t launch_fp64(const DevPlan &p, cudaStream_t stream)
{
    if (p.E == 0) return cudaSuccess;
    const int n = p.n;
    int p2 = 1;
    while (p2 < n) p2 <<= 1;
    // the mixed-precision implicit mode: FP64 Newton, FP32 dipolar sum
    const bool dip32 = p.use_implicit && p.pr != nullptr;
    const size_t slot = (size_t)slot_doubles(n, p2, dip32) * sizeof(double);
    dim3 grid, block;
    size_t shmem;
    if (n > 32) {
        block = dim3(((n + 31) / 32) * 32);
        grid = dim3((unsigned)p.E);
        shmem = slot;
    } else {
        const int mpw = (p.members_per_warp > 0 && p.members_per_warp < 32 / n) ? p.members_per_warp : 32 / n;
        const int warps = p.block_warps > 0 ? p.block_warps : 4;
        block = dim3(32 * warps);
        const int64_t per_block = (int64_t)warps * mpw;
        grid = dim3((unsigned)((p.E + per_block - 1) / per_block));
        shmem = slot * per_block;
    }
    const unsigned bt = block.x;
    if (p.use_implicit && dip32) {
        if (bt <= 256) sllg_fp64_kernel<true, true, 256><<<grid, block, shmem, stream>>>(p);
        else if (bt <= 512) sllg_fp64_kernel<true, true, 512><<<grid, block, shmem, stream>>>(p);
        else sllg_fp64_kernel<true, true, 1024><<<grid, block, shmem, stream>>>(p);
    } else if (p.use_implicit) {
        if (bt <= 256) sllg_fp64_kernel<true, false, 256><<<grid, block, shmem, stream>>>(p);
        else if (bt <= 512) sllg_fp64_kernel<true, false, 512><<<grid, block, shmem, stream>>>(p);
        else sllg_fp64_kernel<true, false, 1024><<<grid, block, shmem, stream>>>(p);
    } else {
        if (bt <= 256) sllg_fp64_kernel<false, false, 256><<<grid, block, shmem, stream>>>(p);
        else if (bt <= 512) sllg_fp64_kernel<false, false, 512><<<grid, block, shmem, stream>>>(p);
        else sllg_fp64_kernel<false, false, 1024><<<grid, block, shmem, stream>>>(p);
    }
    return cudaGetLastError();
}

// ---- component evaluation (device versions of the pinned functions) ----
namespace {
__global__ void components_kernel(int64_t n, const double *m, const double *h,
                                  const double *hj, const double *axis, const double *alpha,
                                  const double *sr, double *drift, double *diffusion,
                                  double *drift_jac, double *diff_jac, double *anis)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    double mm[3] = {m[3 * i], m[3 * i + 1], m[3 * i + 2]};
    double hh[3] = {h[3 * i], h[3 * i + 1], h[3 * i + 2]};
    if (drift) {
        double d[3];
        f64::drift(d, mm, alpha[i], hh);
        for (int c = 0; c < 3; c++) drift[3 * i + c] = d[c];
    }
    if (diffusion) {
        double b[9];
        f64::diffusion(b, mm, sr[i], alpha[i]);
        for (int c = 0; c < 9; c++) diffusion[9 * i + c] = b[c];
    }
    if (drift_jac) {
        double hjj[9], j[9];
        for (int c = 0; c < 9; c++) hjj[c] = hj[9 * i + c];
        f64::drift_jacobian(j, mm, alpha[i], hh, hjj);
        for (int c = 0; c < 9; c++) drift_jac[9 * i + c] = j[c];
    }
    if (diff_jac) {
        double j[27];
        f64::diffusion_jacobian(j, mm, sr[i], alpha[i]);
        for (int c = 0; c < 27; c++) diff_jac[27 * i + c] = j[c];
    }
    if (anis) {
        double ax[3] = {axis[3 * i], axis[3 * i + 1], axis[3 * i + 2]}, hh2[3];
        f64::uniaxial(hh2, mm, ax);
        for (int c = 0; c < 3; c++) anis[3 * i + c] = hh2[c];
    }
}
}  // namespace

cudaError_t launch_components(int64_t n, const double *m, const double *h, const double *hj,
                              const double *axis, const double *alpha, const double *sr,
                              double *drift, double *diffusion, double *drift_jac,
                              double *diff_jac, double *anis, cudaStream_t stream)
{
    if (n == 0) return cudaSuccess;
    components_kernel<<<(unsigned)((n + 127) / 128), 128, 0, stream>>>(
        n, m, h, hj, axis, alpha, sr, drift, diffusion, drift_jac, diff_jac, anis);
    return cudaGetLastError();
}

}  // namespace magpy
