// sllg_tc.cu -- mixed-precision sLLG with the dipolar field on the tensor cores.
//
// For E members that share one cluster geometry, the dipolar field of
// lib/field.cpp:187-225 is a fixed 3N x 3N matrix D times the stacked
// moments:  h_dip[3q+c] = sum_{j,c'} D[3q+c][3j+c'] m_j[c'],  with
// D[3q+c][3j+c'] = P_qj (3 r_qj[c] r_qj[c'] - delta_cc') for j != q and 0 on
// the diagonal blocks (P_qj = mu0 Ms^2/(8 pi K) v_j / r_qj^3).
//
// One CTA integrates NM = 32 members for the whole run.  D (split into two
// FP16 matrices, D ~ D_hi + D_lo/2048) stays in shared memory; every Heun
// stage the CTA writes its members' moments as FP16 hi/lo into a shared
// tile B = [B_hi | B_lo] (3N x 64: 32 members' FP16 high parts, then their
// scaled residuals), one thread issues per k-step
//     [acc_main | acc_corr]  (+)= D_hi [B_hi | B_lo]      (N = 64)
//      acc_corr              +=  D_lo  B_hi               (N = 32)
// with tcgen05.mma (M=128, N=32, K=16, FP32 accumulators in tensor memory),
// and the epilogue forms h = acc_main + acc_corr/2048 (about 22 significant
// bits; the dropped D_lo B_lo term is 2^-22 relative).  Everything else --
// anisotropy and Zeeman terms, drift, diffusion, increments from the in-kernel
// generator, the compensated state update, samples -- runs on the CUDA cores
// in FP32 exactly as in sllg_mixed.cu.
#include <algorithm>
#include <cuda_fp16.h>
#include "common.cuh"
#include "plan.hpp"
#include "tc_ptx.cuh"

namespace magpy {

namespace {

constexpr int NM = 32;           // members per CTA = MMA N
constexpr int TC_THREADS = 512;  // 16 warps: 4 TMEM sub-partitions x 4 column quarters
constexpr int HS_STRIDE = NM + 1;
constexpr int MAX_ITEMS = 4;     // (particle, member) items per thread: n * 32 <= 2048
constexpr uint32_t WAIT_LIMIT = 1u << 24;
constexpr int32_t ST_WATCHDOG = 16;
// element distance from member row j to row j + 32 in a 64-row core-matrix grid
constexpr uint32_t LO_SHIFT = (NM / 8) * 64;

struct TcLayout {
    int n, n3, MP, KP, tiles;
    size_t d_bytes;   // one FP16 split of D
    size_t bh_bytes;  // B tile (hi + lo) aliased with the FP32 field exchange
    size_t par_off, sr_off, bar_off, total;
};

__host__ __device__ inline TcLayout tc_layout(int n)
{
    TcLayout L;
    L.n = n;
    L.n3 = 3 * n;
    L.tiles = (L.n3 + 127) / 128;
    L.MP = 128 * L.tiles;
    L.KP = ((L.n3 + 15) / 16) * 16;
    L.d_bytes = (size_t)L.MP * L.KP * 2;
    size_t b = (size_t)2 * L.KP * NM * 2, h = (size_t)L.n3 * HS_STRIDE * 4;
    L.bh_bytes = ((b > h ? b : h) + 127) & ~(size_t)127;
    L.par_off = 2 * L.d_bytes + L.bh_bytes;
    L.sr_off = L.par_off + (size_t)16 * n;
    L.bar_off = (L.sr_off + (size_t)4 * n + 15) & ~(size_t)15;
    L.total = L.bar_off + 16 + 4 * NM;  // mbarrier, TMEM slot, per-member flags
    return L;
}

// D from the pair tables of one cluster (double), split into FP16 hi/lo in
// the core-matrix layout, rows/columns beyond 3N zero.
__global__ void build_d_kernel(const double *pt, const double *rt, int n, int MP, int KP,
                               __half *dhi, __half *dlo)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= MP * KP) return;
    const int r = idx / KP, k = idx % KP;
    double v = 0.0;
    const int n3 = 3 * n;
    if (r < n3 && k < n3) {
        const int q = r / 3, c = r % 3, j = k / 3, c2 = k % 3;
        if (q != j) {
            const double P = pt[(size_t)j * n + q];
            const double rc = rt[((size_t)c * n + j) * n + q];
            const double rc2 = rt[((size_t)c2 * n + j) * n + q];
            v = P * (3.0 * rc * rc2 - (c == c2 ? 1.0 : 0.0));
        }
    }
    const __half hi = __double2half(v);
    const __half lo = __double2half((v - (double)__half2float(hi)) * (double)tc::SPLIT_SCALE);
    const uint32_t o = tc::cm_offset(r, k, MP);
    dhi[o] = hi;
    dlo[o] = lo;
}

// Per-CTA context of the tensor-core rounds.
struct TcCtx {
    TcLayout L;
    __half *sDhi, *sDlo, *sBhi, *sBlo;
    float *sH;
    uint64_t *bar;
    uint32_t tmem;
    uint32_t phase;
};

__device__ inline void tc_setup(TcCtx &C, unsigned char *sm, const __half *dhi, const __half *dlo,
                                int n)
{
    C.L = tc_layout(n);
    C.sDhi = (__half *)sm;
    C.sDlo = (__half *)(sm + C.L.d_bytes);
    C.sBhi = (__half *)(sm + 2 * C.L.d_bytes);  // [B_hi | B_lo]: rows 0..31 and 32..63
    C.sBlo = C.sBhi + LO_SHIFT;                 // row 32 of the same core-matrix grid
    C.sH = (float *)(sm + 2 * C.L.d_bytes);
    C.bar = (uint64_t *)(sm + C.L.bar_off);
    uint32_t *slot = (uint32_t *)(sm + C.L.bar_off + 8);
    C.phase = 0;
    // D: global -> shared, 16 bytes at a time
    const uint4 *src_hi = (const uint4 *)dhi, *src_lo = (const uint4 *)dlo;
    uint4 *dst_hi = (uint4 *)C.sDhi, *dst_lo = (uint4 *)C.sDlo;
    const int chunks = (int)(C.L.d_bytes / 16);
    for (int i = threadIdx.x; i < chunks; i += blockDim.x) {
        dst_hi[i] = src_hi[i];
        dst_lo[i] = src_lo[i];
    }
    // B tile zero (padding rows of K must stay zero)
    uint4 *b = (uint4 *)C.sBhi;
    const int bchunks = (int)(C.L.bh_bytes / 16);
    for (int i = threadIdx.x; i < bchunks; i += blockDim.x) b[i] = make_uint4(0, 0, 0, 0);
    if (threadIdx.x == 0) tc::mbar_init(C.bar, 1);
    if (threadIdx.x < 32) tc::tmem_alloc(slot, 64u * C.L.tiles);
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    C.tmem = *slot;
}

__device__ inline void tc_teardown(TcCtx &C)
{
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc::fence_after_sync();
        tc::tmem_dealloc(C.tmem, 64u * C.L.tiles);
    }
}

// Zero the K-padding rows of the B tile (3N <= k < KP) after the aliased
// field exchange has overwritten them.
__device__ inline void tc_zero_pad(TcCtx &C)
{
    const int pad = C.L.KP - C.L.n3;
    for (int i = threadIdx.x; i < pad * NM; i += blockDim.x) {
        const int k = C.L.n3 + i / NM, j = i % NM;
        const uint32_t o = tc::cm_offset(j, k, 2 * NM);
        C.sBhi[o] = __float2half(0.f);
        C.sBlo[o] = __float2half(0.f);
    }
}

__device__ inline void tc_put(TcCtx &C, int j, int q, const float m[3])
{
    for (int c = 0; c < 3; c++) {
        __half hi, lo;
        tc::split_f16(m[c], hi, lo);
        const uint32_t o = tc::cm_offset(j, 3 * q + c, 2 * NM);
        C.sBhi[o] = hi;
        C.sBlo[o] = lo;
    }
}

// One field round: B (already written and proxy-fenced by every thread)
// -> MMAs -> accumulators -> shared FP32 field sH[row][member].  Returns false
// (uniformly) if the tensor-core completion did not arrive in time.
__device__ inline bool tc_round(TcCtx &C)
{
    const TcLayout &L = C.L;
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x == 0) {
        tc::fence_after_sync();
        const uint32_t idesc = tc::idesc_f16_f32(128, NM);
        // descriptors of (tile 0, k-step 0); later ones advance the 14-bit
        // start-address field (byte offset / 16), which stays below 2^14
        // inside the 227 KB shared window
        const uint32_t idesc64 = tc::idesc_f16_f32(128, 2 * NM);
        const uint32_t a_lbo = (L.MP / 8) * 128, b_lbo = (2 * NM / 8) * 128;
        const uint64_t ah0 = tc::smem_desc(tc::smem_addr(C.sDhi), a_lbo, 128);
        const uint64_t al0 = tc::smem_desc(tc::smem_addr(C.sDlo), a_lbo, 128);
        const uint64_t b0 = tc::smem_desc(tc::smem_addr(C.sBhi), b_lbo, 128);
        const uint32_t a_kstep = (uint32_t)(2 * (L.MP / 8) * 128) >> 4;  // two k core matrices
        const uint32_t b_kstep = (uint32_t)(2 * (2 * NM / 8) * 128) >> 4;
        const uint32_t a_tile = (uint32_t)(16 * 128) >> 4;               // 16 row groups
        const int ksteps = L.KP / 16;
        for (int t = 0; t < L.tiles; t++) {
            const uint32_t acc = C.tmem + 64 * t;
            for (int s = 0; s < ksteps; s++) {
                const uint64_t da = (uint64_t)(a_tile * t + a_kstep * s);
                const uint64_t db = (uint64_t)(b_kstep * s);
                // [main | corr] (+)= D_hi [B_hi | B_lo]; corr += D_lo B_hi (rows 0..31 of B)
                tc::mma_f16(acc, ah0 + da, b0 + db, idesc64, s > 0);
                tc::mma_f16(acc + 32, al0 + da, b0 + db, idesc, 1);
            }
        }
        tc::mma_commit(C.bar);
    }
    const bool ok = tc::mbar_wait_bounded(C.bar, C.phase, WAIT_LIMIT);
    C.phase ^= 1u;
    if (__syncthreads_or(!ok)) return false;
    tc::fence_after_sync();
    // accumulators -> sH (aliases B, whose reads by the MMAs have completed)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = warp & 3, quarter = warp >> 2;
    const uint32_t lanes = (uint32_t)(32 * sub) << 16;
    for (int t = 0; t < L.tiles; t++) {
        float vm[8], vc[8];
        tc::tmem_ld8(C.tmem + lanes + 64 * t + 8 * quarter, vm);
        tc::tmem_ld8(C.tmem + lanes + 64 * t + 32 + 8 * quarter, vc);
        tc::tmem_ld_wait();
        const int row = 128 * t + 32 * sub + lane;
        if (row < L.n3)
            for (int c = 0; c < 8; c++)
                C.sH[row * HS_STRIDE + 8 * quarter + c] = vm[c] + vc[c] * (1.0f / tc::SPLIT_SCALE);
    }
    tc::fence_before_sync();
    __syncthreads();
    return true;
}

// ---- batched dipolar field through the tensor cores (component entry) ----
// m: [E][n][3] (double), h: [E][n][3] (double), one CTA per 32 members.
__global__ void __launch_bounds__(TC_THREADS, 1)
    tc_dipolar_kernel(const __half *dhi, const __half *dlo, int n, int64_t E, const double *m,
                      double *h, int *flag)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    TcCtx C;
    tc_setup(C, sm, dhi, dlo, n);
    const int64_t base = (int64_t)blockIdx.x * NM;
    for (int i = threadIdx.x; i < n * NM; i += blockDim.x) {
        const int q = i % n, j = i / n;
        float v[3] = {0.f, 0.f, 0.f};
        if (base + j < E)
            for (int c = 0; c < 3; c++) v[c] = (float)m[((base + j) * n + q) * 3 + c];
        tc_put(C, j, q, v);
    }
    tc::fence_proxy_async();
    const bool ok = tc_round(C);
    if (!ok) {
        if (threadIdx.x == 0) atomicOr(flag, 1);
    } else {
        for (int i = threadIdx.x; i < n * NM; i += blockDim.x) {
            const int q = i % n, j = i / n;
            if (base + j < E)
                for (int c = 0; c < 3; c++)
                    h[((base + j) * n + q) * 3 + c] = (double)C.sH[(3 * q + c) * HS_STRIDE + j];
        }
    }
    if (!ok) tc::mbar_wait_bounded(C.bar, C.phase ^ 1u, WAIT_LIMIT);
    tc_teardown(C);
}

struct DDf { float hi, lo; };

__device__ inline DDf dd_add(DDf a, float d)
{
    float s = a.hi + d;
    float v = s - a.hi;
    float e = (a.hi - (s - v)) + (d - v);
    e += a.lo;
    float hi = s + e;
    return DDf{hi, e - (hi - s)};
}

__device__ inline void drift32(float d[3], const float m[3], float a, const float h[3])
{
    d[0] = m[2] * h[1] - m[1] * h[2] + a * (h[0] * (m[1] * m[1] + m[2] * m[2]) - m[0] * (m[1] * h[1] + m[2] * h[2]));
    d[1] = m[0] * h[2] - m[2] * h[0] + a * (h[1] * (m[0] * m[0] + m[2] * m[2]) - m[1] * (m[0] * h[0] + m[2] * h[2]));
    d[2] = m[1] * h[0] - m[0] * h[1] + a * (h[2] * (m[0] * m[0] + m[1] * m[1]) - m[2] * (m[0] * h[0] + m[1] * h[1]));
}

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

// ---- the integrator ----
// Items are (particle q, member j) pairs.  Warp w serves the 8 members
// j = 8 (w % 4) + (lane % 8) and the 16 particles 16 (w / 4) + 4 k + lane / 8
// (k = 0..3), so a thread owns four particles of one member.  Per item the
// state is a float-float triple x; between the two Heun stages it keeps
// A = F(m, v1) / 2 and the increments w.
//
// Stage increment: the reference's drift a = -m x h - alpha m x (m x h)
// (lib/llg.cpp:14-29) and diffusion B(m) w = sr (-m x w - alpha m x (m x w))
// (lib/llg.cpp:92-106, the same form with w in place of h), so
//     dt a + sqrt(dt) B w = F(m, dt h + sqrt(dt) sr w),
//     F(m, v) = -(m x v) - alpha (m (m.v) - v |m|^2),
// one evaluation of a map that is linear in v.

__device__ inline void llg_F(float o[3], const float m[3], float alpha, const float v[3])
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

// x + d for a float-float x (error-free two-sum of hi and d + lo).
__device__ inline DDf dd_add_ts(DDf x, float d)
{
    const float y = d + x.lo;
    const float s = x.hi + y;
    const float bb = s - x.hi;
    const float err = (x.hi - (s - bb)) + (y - bb);
    return DDf{s, err};
}

// B-tile offsets of the three components of (q, j): o0 | o1 << 16 and o2.
__device__ inline void item_offsets(int j, int q, uint32_t &o01, uint32_t &o2)
{
    o01 = tc::cm_offset(j, 3 * q, 2 * NM) | (tc::cm_offset(j, 3 * q + 1, 2 * NM) << 16);
    o2 = tc::cm_offset(j, 3 * q + 2, 2 * NM);
}

__device__ inline void put3(TcCtx &C, uint32_t o01, uint32_t o2, float m0, float m1, float m2)
{
    const __half2 h01 = __float22half2_rn(make_float2(m0, m1));
    const __half2 h2x = __float22half2_rn(make_float2(m2, 0.f));
    const float2 f01 = __half22float2(h01);
    const float f2 = __low2float(h2x);
    const __half2 l01 = __float22half2_rn(make_float2((m0 - f01.x) * tc::SPLIT_SCALE,
                                                      (m1 - f01.y) * tc::SPLIT_SCALE));
    const __half2 l2x = __float22half2_rn(make_float2((m2 - f2) * tc::SPLIT_SCALE, 0.f));
    const uint32_t o0 = o01 & 0xffffu, o1 = o01 >> 16;
    C.sBhi[o0] = __low2half(h01);
    C.sBhi[o1] = __high2half(h01);
    C.sBhi[o2] = __low2half(h2x);
    C.sBlo[o0] = __low2half(l01);
    C.sBlo[o1] = __high2half(l01);
    C.sBlo[o2] = __low2half(l2x);
}

__device__ inline void write_sample(const DevPlan &p, int64_t s, int64_t e, int n, int q,
                                    const DDf xk[3])
{
    const int64_t o = s * p.P + e * n + q;
    const double sc = p.out_scale[e];
    p.mx[o] = ((double)xk[0].hi + (double)xk[0].lo) * sc;
    p.my[o] = ((double)xk[1].hi + (double)xk[1].lo) * sc;
    p.mz[o] = ((double)xk[2].hi + (double)xk[2].lo) * sc;
}

__global__ void __launch_bounds__(TC_THREADS, 1)
    sllg_tc_kernel(DevPlan p, const __half *dhi, const __half *dlo)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    TcCtx C;
    const int n = p.n;
    tc_setup(C, sm, dhi, dlo, n);
    const TcLayout &L = C.L;
    float4 *sPar = (float4 *)(sm + L.par_off);
    float *sSr = (float *)(sm + L.sr_off);
    int *sFlag = (int *)(sm + L.bar_off + 16);  // [NM] per-member status bits

    const int64_t base = (int64_t)blockIdx.x * NM;
    const MemberDev *m0d = p.members + base;  // members of a launch share their parameters
    const int64_t P = p.P;
    for (int q = threadIdx.x; q < n; q += blockDim.x) {
        const int64_t g = m0d->pbase + q;
        sPar[q] = make_float4((float)p.axes[g], (float)p.axes[P + g], (float)p.axes[2 * P + g],
                              (float)p.k_red[g]);
        sSr[q] = (float)p.sr[g];
    }
    if (threadIdx.x < NM) sFlag[threadIdx.x] = 0;

    const float dt = (float)m0d->dt, sq = (float)m0d->sqrt_dt, alpha = (float)m0d->alpha;
    const float happ = (float)m0d->happ;
    const bool renorm = m0d->renorm != 0;
    const int64_t S = p.S;
    const int64_t *sched = p.sched + m0d->sched_off;
    const int64_t K = S > 1 ? sched[S - 1] : 0;
    const int64_t per_step = 3 * (int64_t)n;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int j = 8 * (warp & 3) + (lane & 7);
    const int q0 = 16 * (warp >> 2) + (lane >> 3);  // particles q0 + 4k
    const int64_t e = base + j;
    const bool valid = e < p.E;
    const uint64_t seed = valid ? p.members[e].seed : 0;
    const double *noise = (p.noise && valid) ? p.noise + p.members[e].noise_off : nullptr;
    int nit = 0;
    uint32_t o01[MAX_ITEMS], o2[MAX_ITEMS];
    DDf x[MAX_ITEMS][3];
#pragma unroll
    for (int k = 0; k < MAX_ITEMS; k++) {
        const int q = q0 + 4 * k;
        o01[k] = 0; o2[k] = 0;
        if (q < n) {
            nit = k + 1;
            item_offsets(j, q, o01[k], o2[k]);
        }
        for (int c = 0; c < 3; c++) {
            float hi = 0.f, lo = 0.f;
            if (q < n && valid) {
                const double v = p.m0[c * P + e * n + q];
                hi = (float)v;
                lo = (float)(v - (double)hi);
            }
            x[k][c] = DDf{hi, lo};
        }
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < MAX_ITEMS; k++)
        if (q0 + 4 * k < n) put3(C, o01[k], o2[k], x[k][0].hi, x[k][1].hi, x[k][2].hi);
    tc::fence_proxy_async();
    if (p.mx && valid)  // sample 0: the initial state (lib/simulation.cpp:212-219)
        for (int k = 0; k < MAX_ITEMS; k++)
            if (q0 + 4 * k < n) write_sample(p, 0, e, n, q0 + 4 * k, x[k]);
    (void)nit;

    int32_t status = ST_OK;
    int64_t s_next = 1;
    int64_t step = 0;
    bool alive = true;
    for (step = 1; step <= K; step++) {
        // samples recorded before step `step` hold the state after step-1 steps
        while (s_next < S && sched[s_next] == step) {
            if (p.mx && valid)
                for (int k = 0; k < MAX_ITEMS; k++)
                    if (q0 + 4 * k < n) write_sample(p, s_next, e, n, q0 + 4 * k, x[k]);
            s_next++;
        }
        if (p.noise && step * per_step > m0d->noise_len) {
            status |= ST_NOISE_EXHAUSTED;
            break;
        }
        float h1 = happ, h2 = happ;
        if (p.ftab) {
            const float2 f = __ldg(reinterpret_cast<const float2 *>(p.ftab) + (step - 1));
            h1 = f.x;
            h2 = f.y;
        }
        // stage 1: field at the current state
        if (!tc_round(C)) { status |= ST_WATCHDOG; alive = false; break; }
        float hd[MAX_ITEMS][3];
#pragma unroll
        for (int k = 0; k < MAX_ITEMS; k++)
            if (q0 + 4 * k < n)
                for (int c = 0; c < 3; c++)
                    hd[k][c] = C.sH[(3 * (q0 + 4 * k) + c) * HS_STRIDE + j];
        __syncthreads();
        float A[MAX_ITEMS][3], w[MAX_ITEMS][3];
#pragma unroll
        for (int k = 0; k < MAX_ITEMS; k++) {
            const int q = q0 + 4 * k;
            if (q >= n) continue;
            const float4 pa = sPar[q];
            const float ssr = sq * sSr[q];
            if (noise) {
                const double *wp = noise + (step - 1) * per_step + 3 * q;
                w[k][0] = (float)wp[0]; w[k][1] = (float)wp[1]; w[k][2] = (float)wp[2];
            } else {
                const Normals4 r = wiener_normals(seed, (uint64_t)step, (uint32_t)q);
                w[k][0] = r.a; w[k][1] = r.b; w[k][2] = r.c;
            }
            const float m[3] = {x[k][0].hi, x[k][1].hi, x[k][2].hi};
            const float dot = (m[0] * pa.x + m[1] * pa.y + m[2] * pa.z) * pa.w;
            const float v[3] = {fmaf(dt, dot * pa.x + hd[k][0], ssr * w[k][0]),
                                fmaf(dt, dot * pa.y + hd[k][1], ssr * w[k][1]),
                                fmaf(dt, dot * pa.z + h1 + hd[k][2], ssr * w[k][2])};
            float inc[3];
            llg_F(inc, m, alpha, v);
            for (int c = 0; c < 3; c++) A[k][c] = 0.5f * inc[c];
            // predictor x~ = x + dt a + sqrt(dt) B w
            const float xt0 = valid ? m[0] + inc[0] : 0.f;
            const float xt1 = valid ? m[1] + inc[1] : 0.f;
            const float xt2 = valid ? m[2] + inc[2] : 0.f;
            put3(C, o01[k], o2[k], xt0, xt1, xt2);
        }
        tc_zero_pad(C);
        tc::fence_proxy_async();
        // stage 2: field at the predictor
        if (!tc_round(C)) { status |= ST_WATCHDOG; alive = false; break; }
#pragma unroll
        for (int k = 0; k < MAX_ITEMS; k++)
            if (q0 + 4 * k < n)
                for (int c = 0; c < 3; c++)
                    hd[k][c] = C.sH[(3 * (q0 + 4 * k) + c) * HS_STRIDE + j];
        __syncthreads();
#pragma unroll
        for (int k = 0; k < MAX_ITEMS; k++) {
            const int q = q0 + 4 * k;
            if (q >= n) continue;
            const float4 pa = sPar[q];
            const float ssr = sq * sSr[q];
            const float m[3] = {x[k][0].hi + 2.f * A[k][0], x[k][1].hi + 2.f * A[k][1],
                                x[k][2].hi + 2.f * A[k][2]};
            const float dot = (m[0] * pa.x + m[1] * pa.y + m[2] * pa.z) * pa.w;
            const float v[3] = {fmaf(dt, dot * pa.x + hd[k][0], ssr * w[k][0]),
                                fmaf(dt, dot * pa.y + hd[k][1], ssr * w[k][1]),
                                fmaf(dt, dot * pa.z + h2 + hd[k][2], ssr * w[k][2])};
            float inc[3];
            llg_F(inc, m, alpha, v);
            for (int c = 0; c < 3; c++) x[k][c] = dd_add_ts(x[k][c], fmaf(0.5f, inc[c], A[k][c]));
            if (renorm) {
                const float nrm = sqrtf(x[k][0].hi * x[k][0].hi + x[k][1].hi * x[k][1].hi +
                                        x[k][2].hi * x[k][2].hi);
                const float inv = 1.0f / nrm;
                for (int c = 0; c < 3; c++) { x[k][c].hi *= inv; x[k][c].lo *= inv; }
            }
            if (!valid) for (int c = 0; c < 3; c++) x[k][c] = DDf{0.f, 0.f};
            put3(C, o01[k], o2[k], x[k][0].hi, x[k][1].hi, x[k][2].hi);
        }
        tc_zero_pad(C);
        tc::fence_proxy_async();
    }
    // the loop leaves `step` one past the last completed step
    step -= 1;
    if (!alive) tc::mbar_wait_bounded(C.bar, C.phase ^ 1u, WAIT_LIMIT);  // in-flight MMAs
    if (p.mx && valid)  // samples a stopped member never reached
        for (; s_next < S; s_next++)
            for (int k = 0; k < MAX_ITEMS; k++)
                if (q0 + 4 * k < n) {
                    const int64_t o = s_next * P + e * n + q0 + 4 * k;
                    p.mx[o] = NAN; p.my[o] = NAN; p.mz[o] = NAN;
                }
    bool bad = false;
    for (int k = 0; k < MAX_ITEMS; k++)
        if (q0 + 4 * k < n)
            bad |= !(isfinite(x[k][0].hi) && isfinite(x[k][1].hi) && isfinite(x[k][2].hi));
    if (valid && bad) atomicOr(&sFlag[j], ST_NONFINITE);
    __syncthreads();
    if (threadIdx.x < NM && base + threadIdx.x < p.E) {
        const int64_t em = base + threadIdx.x;
        if (p.status) p.status[em] = status | sFlag[threadIdx.x];
        if (p.steps) p.steps[em] = step;
    }
    tc_teardown(C);
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
TcDims tc_dims(int n)
{
    const TcLayout L = tc_layout(n);
    return TcDims{L.MP, L.KP, (size_t)L.MP * L.KP};
}

bool tc_supported(int n) { return n >= 2 && n <= 64 && tc_layout(n).total <= 232448; }

size_t tc_smem_bytes(int n) { return tc_layout(n).total; }

cudaError_t tc_build_d(const double *pt, const double *rt, int n, __half **dhi, __half **dlo,
                       cudaStream_t stream)
{
    const TcLayout L = tc_layout(n);
    cudaError_t err = cudaMalloc((void **)dhi, 2 * L.d_bytes);
    if (err != cudaSuccess) return err;
    *dlo = *dhi + (size_t)L.MP * L.KP;
    const int tot = L.MP * L.KP;
    build_d_kernel<<<(tot + 255) / 256, 256, 0, stream>>>(pt, rt, n, L.MP, L.KP, *dhi, *dlo);
    return cudaGetLastError();
}

// Raises the kernel's dynamic shared-memory limit, once per device, to the
// largest layout, so that launches made while a stream is being captured
// need no set-up call (plans call this when they are created).
cudaError_t tc_init_attributes()
{
    static bool done[64] = {};
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
    err = cudaFuncSetAttribute(sllg_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)tc_smem_bytes(64));
    if (err == cudaSuccess && dev >= 0 && dev < 64) done[dev] = true;
    return err;
}

cudaError_t launch_tc(const DevPlan &p, const __half *dhi, const __half *dlo, cudaStream_t stream)
{
    if (p.E == 0) return cudaSuccess;
    if (!tc_supported(p.n)) return cudaErrorNotSupported;
    const size_t smem = tc_smem_bytes(p.n);
    cudaError_t err = tc_init_attributes();
    if (err != cudaSuccess) return err;
    const unsigned grid = (unsigned)((p.E + NM - 1) / NM);
    sllg_tc_kernel<<<grid, TC_THREADS, smem, stream>>>(p, dhi, dlo);
    return cudaGetLastError();
}

cudaError_t launch_tc_dipolar(const __half *dhi, const __half *dlo, int n, int64_t E,
                              const double *m, double *h, int *flag, size_t slack,
                              cudaStream_t stream)
{
    const size_t smem = tc_smem_bytes(n) + slack;
    cudaError_t err = cudaFuncSetAttribute(tc_dipolar_kernel,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (err != cudaSuccess) return err;
    const unsigned grid = (unsigned)((E + NM - 1) / NM);
    tc_dipolar_kernel<<<grid, TC_THREADS, smem, stream>>>(dhi, dlo, n, E, m, h, flag);
    return cudaGetLastError();
}

}  // namespace magpy
