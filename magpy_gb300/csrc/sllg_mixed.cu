// sllg_mixed.cu -- mixed-precision sLLG ensemble kernel (Heun).
//
// Same thread/member mapping and step/sample structure as the FP64 kernel,
// with FP32 arithmetic for the field, drift and diffusion evaluations and a
// compensated (float-float, ~48-bit significand) state: each Heun step adds
// an FP32 increment of size ~|a| dt + |B| sqrt(dt) to the two-float state
// with an error-free two-sum, so the state does not accumulate one FP32
// rounding of |m| ~ 1 per step.  The applied field is read from a per-step
// table computed in FP64 (t = step*dt reaches 1e6 in reduced units, beyond
// FP32 resolution).
#include "common.cuh"
#include "plan.hpp"
#include "llg64.cuh"

namespace magpy {
namespace {

struct DD { float hi, lo; };

__device__ inline DD dd_add(DD a, float d)
{
    float s = a.hi + d;
    float v = s - a.hi;
    float e = (a.hi - (s - v)) + (d - v);
    e += a.lo;
    float hi = s + e;
    return DD{hi, e - (hi - s)};
}

struct MemberF {
    float dt, sq, alpha, happ;
    int shape;
    const float *ftab;     // [K][2] field at t=step*dt and t+dt, or null (constant)
    const float4 *pr;      // pair table (r0, r1, r2, P), [N][N], index j*n + q
    float *sm;             // [3n] shared moments
    int n, q;
    bool active, interactions;
    MemberSync ms;
};

__device__ inline void field32(const MemberF &M, float h[3], const float s[3], const float ax[3],
                               float k, float happ)
{
    float dot = (s[0] * ax[0] + s[1] * ax[1] + s[2] * ax[2]) * k;
    h[0] = dot * ax[0];
    h[1] = dot * ax[1];
    h[2] = dot * ax[2] + happ;
    if (M.interactions && M.n > 1) {
        if (M.active) {
            M.sm[3 * M.q + 0] = s[0];
            M.sm[3 * M.q + 1] = s[1];
            M.sm[3 * M.q + 2] = s[2];
        }
        M.ms.sync();
        if (M.active) {
            const int n = M.n, q = M.q;
            float h0 = 0.f, h1 = 0.f, h2 = 0.f;
            for (int j = 0; j < n; j++) {
                const float4 r = __ldg(M.pr + (size_t)j * n + q);  // P = 0 on the diagonal
                const float mj0 = M.sm[3 * j], mj1 = M.sm[3 * j + 1], mj2 = M.sm[3 * j + 2];
                const float d3 = 3.f * (mj0 * r.x + mj1 * r.y + mj2 * r.z);
                h0 += r.w * (d3 * r.x - mj0);
                h1 += r.w * (d3 * r.y - mj1);
                h2 += r.w * (d3 * r.z - mj2);
            }
            h[0] += h0; h[1] += h1; h[2] += h2;
        }
        M.ms.sync();
    }
}

__device__ inline void drift32(float d[3], const float m[3], float a, const float h[3])
{
    // a = -m x h - alpha m x (m x h), written as in lib/llg.cpp:14-29
    d[0] = m[2] * h[1] - m[1] * h[2] + a * (h[0] * (m[1] * m[1] + m[2] * m[2]) - m[0] * (m[1] * h[1] + m[2] * h[2]));
    d[1] = m[0] * h[2] - m[2] * h[0] + a * (h[1] * (m[0] * m[0] + m[2] * m[2]) - m[1] * (m[0] * h[0] + m[2] * h[2]));
    d[2] = m[1] * h[0] - m[0] * h[1] + a * (h[2] * (m[0] * m[0] + m[1] * m[1]) - m[2] * (m[0] * h[0] + m[1] * h[1]));
}

// B(m) w for the 3x3 diffusion of lib/llg.cpp:92-106
__device__ inline void diffw32(float o[3], const float m[3], float sr, float a, const float w[3])
{
    const float b0 = a * (m[1] * m[1] + m[2] * m[2]), b1 = m[2] - a * m[0] * m[1],
                b2 = -(m[1] + a * m[0] * m[2]);
    const float b3 = -(m[2] + a * m[0] * m[1]), b4 = a * (m[0] * m[0] + m[2] * m[2]),
                b5 = m[0] - a * m[1] * m[2];
    const float b6 = m[1] - a * m[0] * m[2], b7 = -(m[0] + a * m[1] * m[2]),
                b8 = a * (m[0] * m[0] + m[1] * m[1]);
    o[0] = sr * (b0 * w[0] + b1 * w[1] + b2 * w[2]);
    o[1] = sr * (b3 * w[0] + b4 * w[1] + b5 * w[2]);
    o[2] = sr * (b6 * w[0] + b7 * w[1] + b8 * w[2]);
}

// MAXT = 0: no register cap (CTAs of up to 640 threads); 1024: members of
// more than 640 particles, one CTA of up to 1024 threads each.
template <int MAXT>
__global__ void __launch_bounds__(MAXT > 0 ? MAXT : 640)
    sllg_mixed_kernel(DevPlan p, const float *ftab_all, const float4 *pr_all)
{
    extern __shared__ float smf[];
    const int n = p.n;
    MemberF M;
    int64_t e;
    if (n > 32) {
        e = blockIdx.x;
        M.q = threadIdx.x;
        M.active = M.q < n;
        M.ms.cta = true;
        M.ms.mask = 0xffffffffu;
        M.sm = smf;
    } else {
        const int mpw = (p.members_per_warp > 0 && p.members_per_warp < 32 / n) ? p.members_per_warp : 32 / n;
        const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
        const int sub = lane / n;
        const int slot = warp * mpw + sub;
        e = (int64_t)blockIdx.x * ((blockDim.x >> 5) * mpw) + slot;
        if (sub >= mpw || e >= p.E) return;
        M.q = lane % n;
        M.active = true;
        M.ms.cta = false;
        M.ms.mask = (n == 32) ? 0xffffffffu : (((1u << n) - 1u) << (sub * n));
        M.sm = smf + (size_t)slot * 3 * n;
    }
    M.n = n;
    const MemberDev *md = p.members + e;
    M.dt = (float)md->dt;
    M.sq = (float)md->sqrt_dt;
    M.alpha = (float)md->alpha;
    M.happ = (float)md->happ;
    M.shape = md->shape;
    M.interactions = md->interactions != 0;
    M.ftab = (md->shape == FIELD_CONSTANT) ? nullptr : ftab_all;
    M.pr = pr_all + md->cluster_off;

    const int64_t P = p.P;
    const int64_t g = md->pbase + (M.active ? M.q : 0);
    float ax[3];
    DD x[3];
    float px[3];
    for (int c = 0; c < 3; c++) {
        ax[c] = (float)p.axes[c * P + g];
        const double v = p.m0[c * P + g];
        x[c].hi = (float)v;
        x[c].lo = (float)(v - (double)x[c].hi);
    }
    const float k = (float)p.k_red[g], sr = (float)p.sr[g];
    const double scale = p.out_scale[e];
    const int64_t S = p.S;
    const int64_t *sched = p.sched + md->sched_off;
    const double *noise = p.noise ? p.noise + md->noise_off : nullptr;
    const int64_t per_step = 3 * (int64_t)n;
    const float *ftab = M.ftab;

    if (M.active && p.mx) {
        p.mx[g] = ((double)x[0].hi + (double)x[0].lo) * scale;
        p.my[g] = ((double)x[1].hi + (double)x[1].lo) * scale;
        p.mz[g] = ((double)x[2].hi + (double)x[2].lo) * scale;
    }
    DD pxd[3] = {x[0], x[1], x[2]};
    int32_t status = ST_OK;
    uint64_t step = 0;
    int64_t s = 1;
    for (; s < S; s++) {
        const int64_t ks = sched[s];
        while ((int64_t)step < ks) {
            pxd[0] = x[0]; pxd[1] = x[1]; pxd[2] = x[2];
            step++;
            float w[3];
            if (noise) {
                if ((int64_t)step * per_step > md->noise_len) {
                    status |= ST_NOISE_EXHAUSTED;
                    step--;
                    goto finished;
                }
                const double *wp = noise + (int64_t)(step - 1) * per_step + 3 * M.q;
                w[0] = (float)wp[0]; w[1] = (float)wp[1]; w[2] = (float)wp[2];
            } else {
                Normals4 r = wiener_normals(md->seed, step, (uint32_t)M.q);
                w[0] = r.a; w[1] = r.b; w[2] = r.c;
            }
            float h1 = M.happ, h2 = M.happ;
            if (ftab) {
                const float2 f = __ldg(reinterpret_cast<const float2 *>(ftab) + (step - 1));
                h1 = f.x;
                h2 = f.y;
            }
            for (int c = 0; c < 3; c++) px[c] = pxd[c].hi;
            float h[3], a[3], bw[3], xt[3];
            field32(M, h, px, ax, k, h1);
            drift32(a, px, M.alpha, h);
            diffw32(bw, px, sr, M.alpha, w);
            for (int c = 0; c < 3; c++) xt[c] = px[c] + (M.dt * a[c] + M.sq * bw[c]);
            float ta[3], tbw[3];
            field32(M, h, xt, ax, k, h2);
            drift32(ta, xt, M.alpha, h);
            diffw32(tbw, xt, sr, M.alpha, w);
            for (int c = 0; c < 3; c++) {
                const float dlt = 0.5f * M.dt * (a[c] + ta[c]) + 0.5f * M.sq * (bw[c] + tbw[c]);
                x[c] = dd_add(pxd[c], dlt);
            }
            if (md->renorm) {
                const float nrm = sqrtf(x[0].hi * x[0].hi + x[1].hi * x[1].hi + x[2].hi * x[2].hi);
                const float inv = 1.0f / nrm;
                for (int c = 0; c < 3; c++) { x[c].hi *= inv; x[c].lo *= inv; }
            }
        }
        if (M.active && p.mx) {
            const int64_t o = s * P + g;
            p.mx[o] = ((double)pxd[0].hi + (double)pxd[0].lo) * scale;
            p.my[o] = ((double)pxd[1].hi + (double)pxd[1].lo) * scale;
            p.mz[o] = ((double)pxd[2].hi + (double)pxd[2].lo) * scale;
        }
    }
finished:
    if (M.active && p.mx)
        for (; s < S; s++) {
            const int64_t o = s * P + g;
            p.mx[o] = NAN; p.my[o] = NAN; p.mz[o] = NAN;
        }
    {
        bool bad = M.active && !(isfinite(x[0].hi) && isfinite(x[1].hi) && isfinite(x[2].hi));
        bool any = M.ms.cta ? (__syncthreads_or(bad) != 0) : (__any_sync(M.ms.mask, bad) != 0);
        if (any) status |= ST_NONFINITE;
    }
    if (M.q == 0) {
        if (p.status) p.status[e] = status;
        if (p.steps) p.steps[e] = (int64_t)step;
    }
}

// Clusters of more than 32 particles whose members all share one cluster
// and its parameters: MPC members per CTA, thread q integrates particle q of
// each of them, so every pair-table entry read for the dipolar sums serves
// MPC members (one member per CTA streams the whole n x n table through L1
// once per field evaluation).  Moments of the CTA's members are exchanged in
// shared memory, one buffer per Heun stage; between the stages a member
// keeps its state, its increments w and s1 = dt a + sqrt(dt) B w.
template <int MPC, int MAXT>
__global__ void __launch_bounds__(MAXT, MAXT <= 256 ? (MPC == 2 ? 3 : 2) : 1)
    sllg_mixed_multi_kernel(DevPlan p, const float *ftab_all, const float4 *pr_all)
{
    extern __shared__ float4 sm4[];  // [2][MPC][n]
    const int n = p.n, q = threadIdx.x;
    const bool active = q < n;
    const int64_t e0 = (int64_t)blockIdx.x * MPC;
    const MemberDev *md0 = p.members + e0;
    const float dt = (float)md0->dt, sq = (float)md0->sqrt_dt, alpha = (float)md0->alpha;
    const float happ = (float)md0->happ;
    const float *ftab = (md0->shape == FIELD_CONSTANT) ? nullptr : ftab_all;
    const float4 *pr = pr_all + md0->cluster_off;
    const bool inter = md0->interactions != 0 && n > 1;
    const bool renorm = md0->renorm != 0;
    const int64_t P = p.P;
    const int64_t g0 = md0->pbase + (active ? q : 0);
    const float ax[3] = {(float)p.axes[g0], (float)p.axes[P + g0], (float)p.axes[2 * P + g0]};
    const float k = (float)p.k_red[g0], sr = (float)p.sr[g0];
    const int64_t S = p.S;
    const int64_t *sched = p.sched + md0->sched_off;
    const int64_t per_step = 3 * (int64_t)n;

    bool valid[MPC];
    uint64_t seed[MPC];
    const double *noise[MPC];
    double scale[MPC];
    DD x[MPC][3], pxd[MPC][3];
#pragma unroll
    for (int m = 0; m < MPC; m++) {
        const int64_t e = e0 + m;
        valid[m] = e < p.E;
        const MemberDev *md = p.members + (valid[m] ? e : e0);
        seed[m] = md->seed;
        noise[m] = p.noise ? p.noise + md->noise_off : nullptr;
        scale[m] = p.out_scale[valid[m] ? e : e0];
        const int64_t g = md->pbase + (active ? q : 0);
        for (int c = 0; c < 3; c++) {
            const double v = p.m0[c * P + g];
            x[m][c].hi = (float)v;
            x[m][c].lo = (float)(v - (double)x[m][c].hi);
            pxd[m][c] = x[m][c];
        }
        if (active && valid[m] && p.mx) {
            p.mx[e * n + q] = ((double)x[m][0].hi + (double)x[m][0].lo) * scale[m];
            p.my[e * n + q] = ((double)x[m][1].hi + (double)x[m][1].lo) * scale[m];
            p.mz[e * n + q] = ((double)x[m][2].hi + (double)x[m][2].lo) * scale[m];
        }
    }
    float4 *buf0 = sm4, *buf1 = sm4 + MPC * n;
    int32_t status = ST_OK;
    uint64_t step = 0;
    int64_t s = 1;
    for (; s < S; s++) {
        const int64_t ks = sched[s];
        while ((int64_t)step < ks) {
            step++;
            if (p.noise && (int64_t)step * per_step > md0->noise_len) {
                status |= ST_NOISE_EXHAUSTED;
                step--;
                goto finished;
            }
            float h1 = happ, h2 = happ;
            if (ftab) {
                const float2 f = __ldg(reinterpret_cast<const float2 *>(ftab) + (step - 1));
                h1 = f.x;
                h2 = f.y;
            }
            float w[MPC][3], s1[MPC][3], hd[MPC][3];
            // stage 1: field at the current state
#pragma unroll
            for (int m = 0; m < MPC; m++) {
                for (int c = 0; c < 3; c++) pxd[m][c] = x[m][c];
                if (active)
                    buf0[m * n + q] = make_float4(x[m][0].hi, x[m][1].hi, x[m][2].hi, 0.f);
            }
            __syncthreads();
#pragma unroll
            for (int m = 0; m < MPC; m++) hd[m][0] = hd[m][1] = hd[m][2] = 0.f;
            if (inter && active)
                for (int j = 0; j < n; j++) {
                    const float4 r = __ldg(pr + (size_t)j * n + q);  // P = 0 on the diagonal
#pragma unroll
                    for (int m = 0; m < MPC; m++) {
                        const float4 mj = buf0[m * n + j];
                        const float d3 = 3.f * (mj.x * r.x + mj.y * r.y + mj.z * r.z);
                        hd[m][0] += r.w * (d3 * r.x - mj.x);
                        hd[m][1] += r.w * (d3 * r.y - mj.y);
                        hd[m][2] += r.w * (d3 * r.z - mj.z);
                    }
                }
#pragma unroll
            for (int m = 0; m < MPC; m++) {
                if (noise[m]) {
                    const double *wp = noise[m] + (int64_t)(step - 1) * per_step + 3 * q;
                    w[m][0] = (float)wp[0]; w[m][1] = (float)wp[1]; w[m][2] = (float)wp[2];
                } else {
                    const Normals4 rn = wiener_normals(seed[m], step, (uint32_t)q);
                    w[m][0] = rn.a; w[m][1] = rn.b; w[m][2] = rn.c;
                }
                const float px[3] = {pxd[m][0].hi, pxd[m][1].hi, pxd[m][2].hi};
                const float dot = (px[0] * ax[0] + px[1] * ax[1] + px[2] * ax[2]) * k;
                const float h[3] = {dot * ax[0] + hd[m][0], dot * ax[1] + hd[m][1],
                                    dot * ax[2] + h1 + hd[m][2]};
                float a[3], bw[3];
                drift32(a, px, alpha, h);
                diffw32(bw, px, sr, alpha, w[m]);
                for (int c = 0; c < 3; c++) s1[m][c] = dt * a[c] + sq * bw[c];
                if (active)
                    buf1[m * n + q] = make_float4(px[0] + s1[m][0], px[1] + s1[m][1],
                                                  px[2] + s1[m][2], 0.f);
            }
            __syncthreads();
            // stage 2: field at the predictor
#pragma unroll
            for (int m = 0; m < MPC; m++) hd[m][0] = hd[m][1] = hd[m][2] = 0.f;
            if (inter && active)
                for (int j = 0; j < n; j++) {
                    const float4 r = __ldg(pr + (size_t)j * n + q);
#pragma unroll
                    for (int m = 0; m < MPC; m++) {
                        const float4 mj = buf1[m * n + j];
                        const float d3 = 3.f * (mj.x * r.x + mj.y * r.y + mj.z * r.z);
                        hd[m][0] += r.w * (d3 * r.x - mj.x);
                        hd[m][1] += r.w * (d3 * r.y - mj.y);
                        hd[m][2] += r.w * (d3 * r.z - mj.z);
                    }
                }
#pragma unroll
            for (int m = 0; m < MPC; m++) {
                const float xt[3] = {pxd[m][0].hi + s1[m][0], pxd[m][1].hi + s1[m][1],
                                     pxd[m][2].hi + s1[m][2]};
                const float dot = (xt[0] * ax[0] + xt[1] * ax[1] + xt[2] * ax[2]) * k;
                const float h[3] = {dot * ax[0] + hd[m][0], dot * ax[1] + hd[m][1],
                                    dot * ax[2] + h2 + hd[m][2]};
                float ta[3], tbw[3];
                drift32(ta, xt, alpha, h);
                diffw32(tbw, xt, sr, alpha, w[m]);
                for (int c = 0; c < 3; c++)
                    x[m][c] = dd_add(pxd[m][c], 0.5f * (s1[m][c] + (dt * ta[c] + sq * tbw[c])));
                if (renorm) {
                    const float nrm = sqrtf(x[m][0].hi * x[m][0].hi + x[m][1].hi * x[m][1].hi +
                                            x[m][2].hi * x[m][2].hi);
                    const float inv = 1.0f / nrm;
                    for (int c = 0; c < 3; c++) { x[m][c].hi *= inv; x[m][c].lo *= inv; }
                }
            }
        }
#pragma unroll
        for (int m = 0; m < MPC; m++)
            if (active && valid[m] && p.mx) {
                const int64_t o = s * P + (e0 + m) * n + q;
                p.mx[o] = ((double)pxd[m][0].hi + (double)pxd[m][0].lo) * scale[m];
                p.my[o] = ((double)pxd[m][1].hi + (double)pxd[m][1].lo) * scale[m];
                p.mz[o] = ((double)pxd[m][2].hi + (double)pxd[m][2].lo) * scale[m];
            }
    }
finished:
#pragma unroll
    for (int m = 0; m < MPC; m++) {
        if (active && valid[m] && p.mx)
            for (int64_t t = s; t < S; t++) {
                const int64_t o = t * P + (e0 + m) * n + q;
                p.mx[o] = NAN; p.my[o] = NAN; p.mz[o] = NAN;
            }
        const bool bad = active && valid[m] &&
                         !(isfinite(x[m][0].hi) && isfinite(x[m][1].hi) && isfinite(x[m][2].hi));
        const int any = __syncthreads_or(bad);
        if (q == 0 && valid[m]) {
            if (p.status) p.status[e0 + m] = status | (any ? ST_NONFINITE : 0);
            if (p.steps) p.steps[e0 + m] = (int64_t)step;
        }
    }
}

// Applied field per step, in FP64 then rounded: entry 2(k-1) is h(k*dt),
// 2(k-1)+1 is h(k*dt + dt) (lib/integrators.cpp:386, :394 evaluate the
// stages at t and t + dt with t = step*dt, lib/simulation.cpp:355).
__global__ void field_table_kernel(float *tab, int64_t K, double dt, int shape, double happ,
                                   double fapp)
{
    int64_t k = blockIdx.x * (int64_t)blockDim.x + threadIdx.x + 1;
    if (k > K) return;
    tab[2 * (k - 1)] = f64::heun_field_f32(shape, dt, happ, fapp, k, 0);
    tab[2 * (k - 1) + 1] = f64::heun_field_f32(shape, dt, happ, fapp, k, 1);
}

__global__ void pair_table_kernel(float4 *out, const double *pt, const double *rt, int64_t n,
                                  int64_t clusters)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nn = n * n;
    if (i >= nn * clusters) return;
    const int64_t c = i / nn, r = i % nn;
    const double *P = pt + c * nn;
    const double *R = rt + 3 * c * nn;
    out[i] = make_float4((float)R[r], (float)R[nn + r], (float)R[2 * nn + r], (float)P[r]);
}

__global__ void wiener_kernel(uint64_t seed, int64_t n, int64_t K, double *out)
{
    int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n * K) return;
    const int64_t k = i / n + 1, q = i % n;
    Normals4 r = wiener_normals(seed, (uint64_t)k, (uint32_t)q);
    double *o = out + (k - 1) * 3 * n + 3 * q;
    o[0] = r.a;
    o[1] = r.b;
    o[2] = r.c;
}

}  // namespace

cudaError_t mixed_prepare(const DevPlan &p, int64_t clusters, int64_t K, double dt, int shape,
                          double happ, double fapp, float **ftab, float4 **pr,
                          cudaStream_t stream)
{
    *ftab = nullptr;
    *pr = nullptr;
    cudaError_t err;
    if (shape != FIELD_CONSTANT && K > 0) {
        err = pool_alloc((void **)ftab, 2 * K * sizeof(float));
        if (err != cudaSuccess) return err;
        field_table_kernel<<<(unsigned)((K + 255) / 256), 256, 0, stream>>>(*ftab, K, dt, shape,
                                                                            happ, fapp);
        if ((err = cudaGetLastError()) != cudaSuccess) return err;
    }
    const int64_t n = p.n;
    if (p.pt && clusters > 0) {
        const int64_t tot = clusters * n * n;
        err = pool_alloc((void **)pr, tot * sizeof(float4));
        if (err != cudaSuccess) return err;
        pair_table_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, stream>>>(*pr, p.pt, p.rt, n,
                                                                             clusters);
        if ((err = cudaGetLastError()) != cudaSuccess) return err;
    }
    return cudaSuccess;
}

cudaError_t mixed_fill_tables(const DevPlan &p, int64_t clusters, int64_t K, double dt,
                              int shape, double happ, double fapp, float *ftab, float4 *pr,
                              cudaStream_t stream)
{
    if (ftab && shape != FIELD_CONSTANT && K > 0) {
        field_table_kernel<<<(unsigned)((K + 255) / 256), 256, 0, stream>>>(ftab, K, dt, shape,
                                                                            happ, fapp);
        cudaError_t err = cudaGetLastError();
        if (err != cudaSuccess) return err;
    }
    const int64_t n = p.n;
    if (pr && p.pt && clusters > 0) {
        const int64_t tot = clusters * n * n;
        pair_table_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, stream>>>(pr, p.pt, p.rt, n,
                                                                             clusters);
        return cudaGetLastError();
    }
    return cudaSuccess;
}

cudaError_t launch_mixed(const DevPlan &p, cudaStream_t stream)
{
    if (p.E == 0) return cudaSuccess;
    if (p.use_implicit) return cudaErrorInvalidValue;
    const int n = p.n;
    dim3 grid, block;
    size_t shmem;
    if (n > 32) {
        block = dim3(((n + 31) / 32) * 32);
        grid = dim3((unsigned)p.E);
        shmem = 3 * n * sizeof(float);
    } else {
        const int mpw = (p.members_per_warp > 0 && p.members_per_warp < 32 / n) ? p.members_per_warp : 32 / n;
        const int warps = p.block_warps > 0 ? p.block_warps : 4;
        block = dim3(32 * warps);
        const int64_t per_block = (int64_t)warps * mpw;
        grid = dim3((unsigned)((p.E + per_block - 1) / per_block));
        shmem = 3 * n * sizeof(float) * per_block;
    }
    const int mpc = p.members_per_warp;
    if (n > 32 && p.shared_cluster && (mpc == 2 || mpc == 4)) {
        const unsigned blocks = (unsigned)((p.E + mpc - 1) / mpc);
        const size_t sm = (size_t)2 * mpc * n * sizeof(float4);
        if (block.x <= 256) {
            if (mpc == 2) sllg_mixed_multi_kernel<2, 256><<<blocks, block, sm, stream>>>(p, p.ftab, p.pr);
            else sllg_mixed_multi_kernel<4, 256><<<blocks, block, sm, stream>>>(p, p.ftab, p.pr);
        } else {
            if (mpc == 2) sllg_mixed_multi_kernel<2, 1024><<<blocks, block, sm, stream>>>(p, p.ftab, p.pr);
            else sllg_mixed_multi_kernel<4, 1024><<<blocks, block, sm, stream>>>(p, p.ftab, p.pr);
        }
        return cudaGetLastError();
    }
    if (block.x <= 640) sllg_mixed_kernel<0><<<grid, block, shmem, stream>>>(p, p.ftab, p.pr);
    else sllg_mixed_kernel<1024><<<grid, block, shmem, stream>>>(p, p.ftab, p.pr);
    return cudaGetLastError();
}

cudaError_t launch_wiener(uint64_t seed, int64_t n_particles, int64_t n_steps, double *out,
                          cudaStream_t stream)
{
    const int64_t tot = n_particles * n_steps;
    if (tot == 0) return cudaSuccess;
    wiener_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, stream>>>(seed, n_particles, n_steps,
                                                                   out);
    return cudaGetLastError();
}

}  // namespace magpy
