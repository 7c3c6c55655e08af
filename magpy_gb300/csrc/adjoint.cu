// adjoint.cu -- pathwise adjoint of the stochastic Heun step over fixed noise.
//
// Forward map of one step (reduced units, per particle, with the increments w
// of the step fixed by the counter-based generator):
//     h(x)  = k (x.e) e + D x + happ s(t) z          (lib/simulation.cpp:271-290)
//     v     = dt h + sqrt(dt) sr w
//     F(m,v)= -(m x v) - alpha (m (m.v) - v |m|^2)    (drift and diffusion of
//             lib/llg.cpp:14-106 share this form, linear in v)
//     x~    = x + F(x, v1(x)),   x' = x + (F(x, v1(x)) + F(x~, v2(x~))) / 2
// (the Stratonovich Heun step of lib/integrators.cpp:372-405).
//
// Reverse step, for the adjoint lambda' = dJ/dx':
//     g2 = lambda'/2,  mu2 = M(x~)^T g2,  eta2 = dt mu2
//     lam~ = J_m(x~,v2)^T g2 + (A + D)^T eta2
//     g1 = lambda'/2 + lam~,  mu1 = M(x)^T g1,  eta1 = dt mu1
//     lambda = lambda' + lam~ + J_m(x,v1)^T g1 + (A + D)^T eta1
// with M(m)^T u = m x u - alpha (m (m.u) - u |m|^2),
//      J_m(m,v)^T u = u x v - alpha ((m.v) u + (m.u) v - 2 (u.v) m),
//      A = k e e^T (symmetric), D^T = V D V^-1 (V = diag of reduced volumes,
//      so the forward pair table serves the transpose too).
// Parameter sensitivities accumulated along the way:
//     Gh = sum mu.h (d/d dt), Gw = sum mu.(sr w) (d/d sqrt(dt)),
//     Ga = sum g.dF/dalpha, Ghapp = sum eta_z s, Gc = sum eta.(D x)/c.
// Checkpoints every C steps keep the float-float state; each segment is
// recomputed forward (same code, same bits) into a buffer of moments and
// then swept backward.
#include "common.cuh"
#include "plan.hpp"

namespace magpy {
namespace {

struct DDa { float hi, lo; };

__device__ inline DDa dd_add2(DDa x, float d)
{
    const float y = d + x.lo;
    const float s = x.hi + y;
    const float bb = s - x.hi;
    const float err = (x.hi - (s - bb)) + (y - bb);
    return DDa{s, err};
}

__device__ inline void Fv(float o[3], const float m[3], float alpha, const float v[3])
{
    const float c0 = m[1] * v[2] - m[2] * v[1];
    const float c1 = m[2] * v[0] - m[0] * v[2];
    const float c2 = m[0] * v[1] - m[1] * v[0];
    const float mv = m[0] * v[0] + m[1] * v[1] + m[2] * v[2];
    const float mm = m[0] * m[0] + m[1] * m[1] + m[2] * m[2];
    o[0] = fmaf(alpha, v[0] * mm - m[0] * mv, -c0);
    o[1] = fmaf(alpha, v[1] * mm - m[1] * mv, -c1);
    o[2] = fmaf(alpha, v[2] * mm - m[2] * mv, -c2);
}

// M(m)^T u
__device__ inline void MT(float o[3], const float m[3], float alpha, const float u[3])
{
    const float mu = m[0] * u[0] + m[1] * u[1] + m[2] * u[2];
    const float mm = m[0] * m[0] + m[1] * m[1] + m[2] * m[2];
    o[0] = m[1] * u[2] - m[2] * u[1] - alpha * (m[0] * mu - u[0] * mm);
    o[1] = m[2] * u[0] - m[0] * u[2] - alpha * (m[1] * mu - u[1] * mm);
    o[2] = m[0] * u[1] - m[1] * u[0] - alpha * (m[2] * mu - u[2] * mm);
}

// J_m(m, v)^T u, accumulated into o
__device__ inline void JmT_add(float o[3], const float m[3], float alpha, const float v[3],
                               const float u[3])
{
    const float mv = m[0] * v[0] + m[1] * v[1] + m[2] * v[2];
    const float mu = m[0] * u[0] + m[1] * u[1] + m[2] * u[2];
    const float uv = u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
    o[0] += u[1] * v[2] - u[2] * v[1] - alpha * (mv * u[0] + mu * v[0] - 2.f * uv * m[0]);
    o[1] += u[2] * v[0] - u[0] * v[2] - alpha * (mv * u[1] + mu * v[1] - 2.f * uv * m[1]);
    o[2] += u[0] * v[1] - u[1] * v[0] - alpha * (mv * u[2] + mu * v[2] - 2.f * uv * m[2]);
}

// u . dF/dalpha
__device__ inline float dFda(const float m[3], const float v[3], const float u[3])
{
    const float mv = m[0] * v[0] + m[1] * v[1] + m[2] * v[2];
    const float mu = m[0] * u[0] + m[1] * u[1] + m[2] * u[2];
    const float uv = u[0] * v[0] + u[1] * v[1] + u[2] * v[2];
    const float mm = m[0] * m[0] + m[1] * m[1] + m[2] * m[2];
    return -(mu * mv - uv * mm);
}

struct AdjMember {
    int n, q;
    bool active;
    MemberSync ms;
    float *sm;            // [3n] exchange buffer
    const float4 *pr;     // pair table (r0, r1, r2, P), index j*n + q
    float ax[3], k, srq, vq;
    uint64_t seed;
    int64_t e, g;         // member, global particle index
};

// sum_j P_qj (3 r_qj (r_qj . s_j) - s_j): the dipolar field of the moments s
__device__ inline void dip(const AdjMember &M, const float s[3], float out[3])
{
    out[0] = out[1] = out[2] = 0.f;
    if (M.n < 2) return;
    if (M.active) {
        M.sm[3 * M.q] = s[0];
        M.sm[3 * M.q + 1] = s[1];
        M.sm[3 * M.q + 2] = s[2];
    }
    M.ms.sync();
    if (M.active)
        for (int j = 0; j < M.n; j++) {
            const float4 r = __ldg(M.pr + (size_t)j * M.n + M.q);
            const float s0 = M.sm[3 * j], s1 = M.sm[3 * j + 1], s2 = M.sm[3 * j + 2];
            const float d3 = 3.f * (s0 * r.x + s1 * r.y + s2 * r.z);
            out[0] += r.w * (d3 * r.x - s0);
            out[1] += r.w * (d3 * r.y - s1);
            out[2] += r.w * (d3 * r.z - s2);
        }
    M.ms.sync();
}

struct AdjArgs {
    int64_t E, P, S, K;
    int n, C, interactions;
    const MemberDev *members;
    const double *m0, *axes, *k_red, *sr, *v_red;
    const float4 *pr;
    const float2 *stab;   // sin of the applied waveform at t_k and t_k + dt, per step
    float happ, dt, sq, alpha, c;
    const int64_t *sched;
    float *ck;            // [K/C + 1][6][P] checkpoints (hi xyz, lo xyz)
    float *seg;           // [C][3][P] moments of the segment being swept
    const double *out_scale; // [E] Ms
    double *mx, *my, *mz; // samples [S][P]
    const double *wz;     // [S] dJ/d(reduced m_z of any particle at sample s)
    double *grad;         // [5] Gh, Gw, Ga, Ghapp, Gc
    int32_t *status;
};

__device__ inline bool setup_member(const AdjArgs &A, AdjMember &M, float *smem)
{
    const int n = A.n;
    if (n > 32) {
        M.e = blockIdx.x;
        M.q = threadIdx.x;
        M.active = M.q < n;
        M.ms.cta = true;
        M.ms.mask = 0xffffffffu;
        M.sm = smem;
    } else {
        const int mpw = 32 / n;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, sub = lane / n;
        const int slot = warp * mpw + sub;
        M.e = (int64_t)blockIdx.x * ((blockDim.x >> 5) * mpw) + slot;
        if (sub >= mpw || M.e >= A.E) return false;
        M.q = lane % n;
        M.active = true;
        M.ms.cta = false;
        M.ms.mask = (n == 32) ? 0xffffffffu : (((1u << n) - 1u) << (sub * n));
        M.sm = smem + (size_t)slot * 3 * n;
    }
    M.n = n;
    M.pr = A.pr;
    M.g = M.e * n + (M.active ? M.q : 0);
    for (int c = 0; c < 3; c++) M.ax[c] = (float)A.axes[c * A.P + M.g];
    M.k = (float)A.k_red[M.g];
    M.srq = (float)A.sr[M.g];
    M.vq = (float)A.v_red[M.g];
    M.seed = A.members[M.e].seed;
    return true;
}

__device__ inline void field_at(const AdjArgs &A, const AdjMember &M, const float m[3], float s,
                                float h[3], float d[3])
{
    if (A.interactions) dip(M, m, d);
    else d[0] = d[1] = d[2] = 0.f;
    const float dot = (m[0] * M.ax[0] + m[1] * M.ax[1] + m[2] * M.ax[2]) * M.k;
    h[0] = dot * M.ax[0] + d[0];
    h[1] = dot * M.ax[1] + d[1];
    h[2] = dot * M.ax[2] + d[2] + A.happ * s;
}

// one forward step (step index k, 1-based) of the float-float state x
__device__ inline void fstep(const AdjArgs &A, const AdjMember &M, DDa x[3], int64_t k)
{
    const Normals4 r = wiener_normals(M.seed, (uint64_t)k, (uint32_t)M.q);
    const float w[3] = {r.a, r.b, r.c};
    const float2 s = A.stab ? __ldg(A.stab + (k - 1)) : make_float2(1.f, 1.f);
    const float m[3] = {x[0].hi, x[1].hi, x[2].hi};
    const float ssr = A.sq * M.srq;
    float h[3], d[3], v[3], f1[3], f2[3], xt[3];
    field_at(A, M, m, s.x, h, d);
    for (int c = 0; c < 3; c++) v[c] = fmaf(A.dt, h[c], ssr * w[c]);
    Fv(f1, m, A.alpha, v);
    for (int c = 0; c < 3; c++) xt[c] = m[c] + f1[c];
    field_at(A, M, xt, s.y, h, d);
    for (int c = 0; c < 3; c++) v[c] = fmaf(A.dt, h[c], ssr * w[c]);
    Fv(f2, xt, A.alpha, v);
    for (int c = 0; c < 3; c++) x[c] = dd_add2(x[c], fmaf(0.5f, f2[c], 0.5f * f1[c]));
}

__device__ inline void write_sample_a(const AdjArgs &A, const AdjMember &M, int64_t s,
                                      const DDa x[3])
{
    if (!M.active || !A.mx) return;
    const int64_t o = s * A.P + M.g;
    const double sc = A.out_scale[M.e];
    A.mx[o] = ((double)x[0].hi + (double)x[0].lo) * sc;
    A.my[o] = ((double)x[1].hi + (double)x[1].lo) * sc;
    A.mz[o] = ((double)x[2].hi + (double)x[2].lo) * sc;
}

__device__ inline void write_ck(const AdjArgs &A, const AdjMember &M, int64_t c, const DDa x[3])
{
    if (!M.active) return;
    float *o = A.ck + c * 6 * A.P + M.g;
    for (int i = 0; i < 3; i++) {
        o[i * A.P] = x[i].hi;
        o[(3 + i) * A.P] = x[i].lo;
    }
}

__global__ void adj_forward_kernel(AdjArgs A)
{
    extern __shared__ float smem_a[];
    AdjMember M;
    if (!setup_member(A, M, smem_a)) return;
    const int64_t P = A.P;
    DDa x[3];
    for (int c = 0; c < 3; c++) {
        const double v = A.m0[c * P + M.g];
        x[c].hi = (float)v;
        x[c].lo = (float)(v - (double)x[c].hi);
    }
    write_ck(A, M, 0, x);
    write_sample_a(A, M, 0, x);
    int64_t s_next = 1;
    for (int64_t step = 1; step <= A.K; step++) {
        while (s_next < A.S && A.sched[s_next] == step) write_sample_a(A, M, s_next++, x);
        fstep(A, M, x, step);
        if (step % A.C == 0) write_ck(A, M, step / A.C, x);
    }
    bool bad = M.active && !(isfinite(x[0].hi) && isfinite(x[1].hi) && isfinite(x[2].hi));
    const bool any = M.ms.cta ? (__syncthreads_or(bad) != 0) : (__any_sync(M.ms.mask, bad) != 0);
    if (M.q == 0 && A.status) A.status[M.e] = any ? ST_NONFINITE : ST_OK;
}

// reverse of step k (1-based) taken from the moments m = x_{k-1}.hi
__device__ inline void bstep(const AdjArgs &A, const AdjMember &M, const float m[3], int64_t k,
                             float lam[3], float G[5])
{
    const Normals4 r = wiener_normals(M.seed, (uint64_t)k, (uint32_t)M.q);
    const float w[3] = {r.a, r.b, r.c};
    const float2 s = A.stab ? __ldg(A.stab + (k - 1)) : make_float2(1.f, 1.f);
    const float ssr = A.sq * M.srq, dt = A.dt, al = A.alpha;
    float h1[3], d1[3], v1[3], f1[3], xt[3], h2[3], d2[3], v2[3];
    field_at(A, M, m, s.x, h1, d1);
    for (int c = 0; c < 3; c++) v1[c] = fmaf(dt, h1[c], ssr * w[c]);
    Fv(f1, m, al, v1);
    for (int c = 0; c < 3; c++) xt[c] = m[c] + f1[c];
    field_at(A, M, xt, s.y, h2, d2);
    for (int c = 0; c < 3; c++) v2[c] = fmaf(dt, h2[c], ssr * w[c]);
    const float sw[3] = {M.srq * w[0], M.srq * w[1], M.srq * w[2]};
    const float inv_c = A.c != 0.f ? 1.f / A.c : 0.f;
    const float inv_v = 1.f / M.vq;

    // stage 2
    float g2[3] = {0.5f * lam[0], 0.5f * lam[1], 0.5f * lam[2]};
    float mu2[3], lt[3] = {0.f, 0.f, 0.f}, eta2[3];
    MT(mu2, xt, al, g2);
    JmT_add(lt, xt, al, v2, g2);
    G[2] += dFda(xt, v2, g2);
    for (int c = 0; c < 3; c++) eta2[c] = dt * mu2[c];
    G[0] += mu2[0] * h2[0] + mu2[1] * h2[1] + mu2[2] * h2[2];
    G[1] += mu2[0] * sw[0] + mu2[1] * sw[1] + mu2[2] * sw[2];
    float de = M.k * (M.ax[0] * eta2[0] + M.ax[1] * eta2[1] + M.ax[2] * eta2[2]);
    for (int c = 0; c < 3; c++) lt[c] += de * M.ax[c];
    if (A.interactions) {
        const float et[3] = {eta2[0] * inv_v, eta2[1] * inv_v, eta2[2] * inv_v};
        float dd[3];
        dip(M, et, dd);
        for (int c = 0; c < 3; c++) lt[c] += M.vq * dd[c];
        G[4] += (eta2[0] * d2[0] + eta2[1] * d2[1] + eta2[2] * d2[2]) * inv_c;
    }
    G[3] += eta2[2] * s.y;

    // stage 1
    float g1[3], mu1[3], ln[3], eta1[3];
    for (int c = 0; c < 3; c++) {
        g1[c] = 0.5f * lam[c] + lt[c];
        ln[c] = lam[c] + lt[c];
    }
    MT(mu1, m, al, g1);
    JmT_add(ln, m, al, v1, g1);
    G[2] += dFda(m, v1, g1);
    for (int c = 0; c < 3; c++) eta1[c] = dt * mu1[c];
    G[0] += mu1[0] * h1[0] + mu1[1] * h1[1] + mu1[2] * h1[2];
    G[1] += mu1[0] * sw[0] + mu1[1] * sw[1] + mu1[2] * sw[2];
    de = M.k * (M.ax[0] * eta1[0] + M.ax[1] * eta1[1] + M.ax[2] * eta1[2]);
    for (int c = 0; c < 3; c++) ln[c] += de * M.ax[c];
    if (A.interactions) {
        const float et[3] = {eta1[0] * inv_v, eta1[1] * inv_v, eta1[2] * inv_v};
        float dd[3];
        dip(M, et, dd);
        for (int c = 0; c < 3; c++) ln[c] += M.vq * dd[c];
        G[4] += (eta1[0] * d1[0] + eta1[1] * d1[1] + eta1[2] * d1[2]) * inv_c;
    }
    G[3] += eta1[2] * s.x;
    for (int c = 0; c < 3; c++) lam[c] = ln[c];
}

__global__ void adj_backward_kernel(AdjArgs A)
{
    extern __shared__ float smem_a[];
    AdjMember M;
    if (!setup_member(A, M, smem_a)) return;
    const int64_t P = A.P;
    float lam[3] = {0.f, 0.f, 0.f};
    double Gt[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    int64_t s_ptr = A.S - 1;
    const int64_t nseg = (A.K + A.C - 1) / A.C;
    for (int64_t c = nseg - 1; c >= 0; c--) {
        const int64_t k0 = c * A.C, k1 = (k0 + A.C < A.K) ? k0 + A.C : A.K;
        DDa x[3];
        const float *ck = A.ck + c * 6 * P + M.g;
        for (int i = 0; i < 3; i++) x[i] = DDa{ck[i * P], ck[(3 + i) * P]};
        float *sg = A.seg + M.g;
        for (int64_t k = k0; k < k1; k++) {
            if (M.active)
                for (int i = 0; i < 3; i++) sg[((k - k0) * 3 + i) * P] = x[i].hi;
            fstep(A, M, x, k + 1);
        }
        float G[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
        for (int64_t k = k1 - 1; k >= k0; k--) {
            float m[3];
            for (int i = 0; i < 3; i++) m[i] = sg[((k - k0) * 3 + i) * P];
            bstep(A, M, m, k + 1, lam, G);
            // samples s >= 1 hold x_{sched[s]-1}: add their objective weights
            while (s_ptr >= 1 && A.sched[s_ptr] - 1 > k) s_ptr--;
            while (s_ptr >= 1 && A.sched[s_ptr] - 1 == k) lam[2] += (float)A.wz[s_ptr--];
        }
        for (int i = 0; i < 5; i++) Gt[i] += (double)G[i];
    }
    if (M.active)
        for (int i = 0; i < 5; i++) atomicAdd(&A.grad[i], Gt[i]);
}

}  // namespace

namespace adj {

struct Launch {
    dim3 grid, block;
    size_t shmem;
};

static Launch shape(int n, int64_t E)
{
    Launch L;
    if (n > 32) {
        L.block = dim3(((n + 31) / 32) * 32);
        L.grid = dim3((unsigned)E);
        L.shmem = 3 * n * sizeof(float);
    } else {
        const int mpw = 32 / n, warps = 4;
        L.block = dim3(32 * warps);
        const int64_t per_block = (int64_t)warps * mpw;
        L.grid = dim3((unsigned)((E + per_block - 1) / per_block));
        L.shmem = 3 * n * sizeof(float) * per_block;
    }
    return L;
}

}  // namespace adj

cudaError_t launch_adjoint(const AdjointArgs &a, bool backward, cudaStream_t stream)
{
    AdjArgs A;
    A.E = a.p.E; A.P = a.p.P; A.S = a.p.S; A.K = a.K;
    A.n = a.p.n; A.C = a.C; A.interactions = a.interactions;
    A.members = a.p.members; A.m0 = a.p.m0; A.axes = a.p.axes; A.k_red = a.p.k_red;
    A.sr = a.p.sr; A.v_red = a.v_red; A.pr = a.p.pr; A.stab = (const float2 *)a.stab;
    A.happ = a.happ; A.dt = a.dt; A.sq = a.sq; A.alpha = a.alpha; A.c = a.c;
    A.sched = a.p.sched; A.ck = a.ck; A.seg = a.seg; A.out_scale = a.p.out_scale;
    A.mx = a.p.mx; A.my = a.p.my; A.mz = a.p.mz; A.wz = a.wz; A.grad = a.grad;
    A.status = a.p.status;
    if (A.E == 0) return cudaSuccess;
    const adj::Launch L = adj::shape(A.n, A.E);
    if (backward) adj_backward_kernel<<<L.grid, L.block, L.shmem, stream>>>(A);
    else adj_forward_kernel<<<L.grid, L.block, L.shmem, stream>>>(A);
    return cudaGetLastError();
}

}  // namespace magpy
