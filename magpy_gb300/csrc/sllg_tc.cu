// sllg_tc.cu -- mixed-precision sLLG with the dipolar field on the tensor cores.
//
// For E members that share one cluster geometry, the dipolar field of
// lib/field.cpp:187-225 is a fixed 3N x 3N matrix D times the stacked
// moments:  h_dip[3q+c] = sum_{j,c'} D[3q+c][3j+c'] m_j[c'],  with
// D[3q+c][3j+c'] = P_qj (3 r_qj[c] r_qj[c'] - delta_cc') for j != q and 0 on
// the diagonal blocks (P_qj = mu0 Ms^2/(8 pi K) v_j / r_qj^3).
//
// One CTA integrates NM = 32 members for the whole run, as two groups of 16
// that take turns on the tensor cores: while the MMAs of one group run, the
// CUDA cores integrate the other group.  D, split into two FP16 matrices
// (D ~ D_hi + D_lo/2048), stays in tensor memory as the MMAs' A operand.
// Every Heun stage of a group the threads write its members' moments as FP16
// hi/lo into the group's shared tile B = [B_hi | B_lo] (3N x 32), and per
// 128-row tile of D one thread of a dedicated issuing warp issues per k-step
//     [acc_main | acc_corr]  (+)= D_hi [B_hi | B_lo]      (N = 32)
//      acc_corr              +=  D_lo  B_hi               (N = 16)
// with tcgen05.mma (M = 128, K = 16, FP32 accumulators in tensor memory) and
// commits to the group's mbarrier; the epilogue forms
// h = acc_main + acc_corr/2048 (about 22 significant bits; the dropped
// D_lo B_lo term is 2^-22 relative).  A step is four phases -- (group 0,
// stage 1), (1, 1), (0, 2), (1, 2) -- and each phase reads its group's
// accumulators while no MMA is in flight, then issues the other group's
// MMAs and integrates its own group while they run.  Everything else --
// anisotropy and Zeeman terms, drift, diffusion, increments from the
// in-kernel generator, the compensated state update, samples -- runs on the
// CUDA cores in FP32.
#include <algorithm>
#include <cuda_fp16.h>
#include "common.cuh"
#include "plan.hpp"
#include "tc_ptx.cuh"
#include "llg32.cuh"
#include "llg64.cuh"

namespace magpy {

namespace {

constexpr int NM = 32;           // members per CTA
constexpr int GM = 16;           // members per group (two groups per CTA)
constexpr int ITEM_THREADS = 512; // 16 item warps: 4 TMEM sub-partitions x 4 column quarters
constexpr int TC_THREADS = ITEM_THREADS + 64;  // + one warp per 128-row tile that only
                                               // issues that tile's MMAs
// Field tile row stride (floats): 20 makes the epilogue's 128-bit stores (32
// consecutive rows, four columns) and the integrator's reads (8 member
// columns of 4 particle pairs) free of bank conflicts.
constexpr int GH_STRIDE = 20;
constexpr int HS_STRIDE = NM + 1;  // field exchange of the single-round dipolar entry
constexpr int ITEMS = 2;         // (particle, member) items per thread and group
constexpr uint32_t WAIT_LIMIT = 1u << 24;
constexpr int FIELD_BLOCK = 32;  // steps of applied field computed at a time (one per lane)
constexpr int32_t ST_WATCHDOG = 16;

// Layouts.  In global memory (and in the dipolar entry's shared memory) D is
// stored row-group outermost ([row/8][k/8] core matrices), so its rows past
// 3N never need storage: the MMAs of the last 128-row tile read whatever
// follows (their accumulator rows are never used), and the shared allocation
// is sized so that those reads stay inside it.  The integrator keeps D in
// tensor memory instead (tmem_d_col), and its shared memory holds only the B
// tiles, field tiles, increments and parameters.
struct TcLayout {
    int n, n3, tiles, KP, rg;
    size_t a_sbo;     // bytes between row groups of D
    size_t d_bytes;   // one FP16 split of D (rg row groups)
    size_t a_span;    // bytes the MMAs of one split read (tiles x 16 row groups)
    size_t buf_off;   // first byte after D_hi, D_lo
    // integrator: per group a B tile and a field tile; the increments and
    // the half stage-1 update, kept from stage 1 for stage 2; the low words of
    // the float-float state; per particle pair the parameters
    size_t gb_bytes, gh_bytes, w_off, a_off, par_off, sr_off, bar_off, total;
    // single-round dipolar entry (32 members): B tile aliased with the field exchange
    size_t bh_bytes, bar_off_dip, total_dip;
};

__host__ __device__ inline size_t up(size_t x, size_t a) { return (x + a - 1) / a * a; }

__host__ __device__ inline TcLayout tc_layout(int n)
{
    TcLayout L;
    L.n = n;
    L.n3 = 3 * n;
    L.tiles = (L.n3 + 127) / 128;
    L.KP = ((L.n3 + 15) / 16) * 16;
    L.rg = (L.n3 + 7) / 8;
    L.a_sbo = (size_t)(L.KP / 8) * 128;
    L.d_bytes = (size_t)L.rg * L.a_sbo;
    L.a_span = (size_t)16 * L.tiles * L.a_sbo;
    L.buf_off = 2 * L.d_bytes;
    const size_t reach = L.d_bytes + L.a_span;  // end of D_lo's MMA reads
    L.gb_bytes = up((size_t)2 * GM * L.KP * 2, 128);
    L.gh_bytes = up((size_t)L.n3 * GH_STRIDE * 4, 128);
    L.w_off = 2 * L.gb_bytes + 2 * L.gh_bytes;  // integrator buffers start at 0
    L.a_off = L.w_off + (size_t)2 * 3 * ITEM_THREADS * 16;  // [g][3] float4 per thread
    L.par_off = L.a_off + (size_t)2 * 3 * ITEM_THREADS * 8;  // [g][3] float2 per thread
    const size_t pairs = (size_t)(n + 1) / 2;
    L.sr_off = L.par_off + 32 * pairs;                       // [pair][2] float4
    L.bar_off = up(L.sr_off + 8 * pairs, 16);                // [pair] float2
    // two mbarriers, TMEM slot, member flags, member seeds and noise offsets,
    // applied-field ring (two blocks of FIELD_BLOCK steps, float2 per step)
    L.total = up(L.bar_off + 32 + 4 * NM + 16 * NM + 2 * FIELD_BLOCK * 8, 128);
    const size_t b = (size_t)2 * L.KP * NM * 2, h = (size_t)L.n3 * HS_STRIDE * 4;
    L.bh_bytes = up(b > h ? b : h, 128);
    L.bar_off_dip = up(L.buf_off + L.bh_bytes, 16);
    L.total_dip = L.bar_off_dip + 16;
    if (L.total_dip < reach) L.total_dip = reach;
    L.total_dip = up(L.total_dip, 128);
    return L;
}

// TMEM columns of the dipolar entry: per tile [main 32 | corr 32].
__host__ __device__ inline uint32_t tmem_cols(const TcLayout &L)
{
    return L.tiles == 1 ? 64u : 128u;
}

// Integrator tensor memory: accumulators in columns [0, 64 tiles) (per tile
// two groups x [main 16 | corr 16]), then D: for tile t and split s (0 hi,
// 1 lo) KP/2 columns at d_col(t, s), row r of the tile in lane r, two
// consecutive K elements per column.  Allocation rounded to a power of two.
__host__ __device__ inline uint32_t tmem_d_col(const TcLayout &L, int t, int sp)
{
    return (uint32_t)(64 * L.tiles + (2 * t + sp) * (L.KP / 2));
}
__host__ __device__ inline uint32_t tmem_cols_int(const TcLayout &L)
{
    const uint32_t need = (uint32_t)(64 * L.tiles + L.tiles * L.KP);
    uint32_t c = 32;
    while (c < need) c <<= 1;
    return c;
}

// D from the pair tables of one cluster (double), split into FP16 hi/lo in
// the row-group-outermost core-matrix layout; rows and columns beyond 3N zero.
__global__ void build_d_kernel(const double *pt, const double *rt, int n, int rows, int KP,
                               __half *dhi, __half *dlo)
{
    const int idx = blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= rows * KP) return;
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
    const uint32_t o = tc::cm_offset_rows(r, k, KP);
    dhi[o] = hi;
    dlo[o] = lo;
}

// D: global -> shared (both splits, contiguous), 16 bytes at a time.
__device__ inline void load_d(unsigned char *sm, const __half *dhi, const TcLayout &L)
{
    const uint4 *src = (const uint4 *)dhi;
    uint4 *dst = (uint4 *)sm;
    const int chunks = (int)(2 * L.d_bytes / 16);
    for (int i = threadIdx.x; i < chunks; i += blockDim.x) dst[i] = src[i];
}

// Descriptors of D_hi / D_lo at (tile 0, k-step 0).  Later ones advance the
// 14-bit start-address field (byte offset / 16), which stays below 2^14 inside
// the 227 KB shared window.
struct ADesc {
    uint64_t hi, lo;
    uint32_t kstep, tile;
};

__device__ inline ADesc a_desc(const unsigned char *sm, const TcLayout &L)
{
    ADesc a;
    const uint32_t s0 = tc::smem_addr(sm);
    a.hi = tc::smem_desc(s0, 128, (uint32_t)L.a_sbo);
    a.lo = tc::smem_desc(s0 + (uint32_t)L.d_bytes, 128, (uint32_t)L.a_sbo);
    a.kstep = (2 * 128) >> 4;                       // two core matrices along K
    a.tile = (uint32_t)((16 * L.a_sbo) >> 4);      // 16 row groups
    return a;
}

// ---- batched dipolar field through the tensor cores (component entry) ----
// m: [E][n][3] (double), h: [E][n][3] (double), one CTA per 32 members, one
// round: B = [B_hi | B_lo] (64 rows), field exchange aliased with B.
__global__ void __launch_bounds__(ITEM_THREADS, 1)
    tc_dipolar_kernel(const __half *dhi, int n, int64_t E, const double *m, double *h, int *flag)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    const TcLayout L = tc_layout(n);
    __half *sB = (__half *)(sm + L.buf_off);
    float *sH = (float *)(sm + L.buf_off);
    uint64_t *bar = (uint64_t *)(sm + L.bar_off_dip);
    uint32_t *slot = (uint32_t *)(sm + L.bar_off_dip + 8);
    load_d(sm, dhi, L);
    uint4 *b = (uint4 *)sB;
    for (int i = threadIdx.x; i < (int)(L.bh_bytes / 16); i += blockDim.x)
        b[i] = make_uint4(0, 0, 0, 0);
    __syncthreads();
    const int64_t base = (int64_t)blockIdx.x * NM;
    const uint32_t lo_shift = (NM / 8) * 64;  // row 32 of the 64-row grid
    for (int i = threadIdx.x; i < n * NM; i += blockDim.x) {
        const int q = i % n, j = i / n;
        for (int c = 0; c < 3; c++) {
            const float v = base + j < E ? (float)m[((base + j) * n + q) * 3 + c] : 0.f;
            __half hi, lo;
            tc::split_f16(v, hi, lo);
            const uint32_t o = tc::cm_offset(j, 3 * q + c, 2 * NM);
            sB[o] = hi;
            sB[o + lo_shift] = lo;
        }
    }
    if (threadIdx.x == 0) tc::mbar_init(bar, 1);
    if (threadIdx.x < 32) tc::tmem_alloc(slot, tmem_cols(L));
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tmem = *slot;
    if (threadIdx.x == 0) {
        const ADesc A = a_desc(sm, L);
        const uint32_t idesc64 = tc::idesc_f16_f32(128, 2 * NM), idesc32 = tc::idesc_f16_f32(128, NM);
        const uint32_t b_lbo = (2 * NM / 8) * 128;
        const uint64_t b0 = tc::smem_desc(tc::smem_addr(sB), b_lbo, 128);
        const uint32_t b_kstep = (2 * b_lbo) >> 4;
        for (int t = 0; t < L.tiles; t++)
            for (int s = 0; s < L.KP / 16; s++) {
                const uint64_t da = (uint64_t)(A.tile * t + A.kstep * s);
                const uint64_t db = (uint64_t)(b_kstep * s);
                tc::mma_f16(tmem + 64 * t, A.hi + da, b0 + db, idesc64, s > 0);
                tc::mma_f16(tmem + 64 * t + 32, A.lo + da, b0 + db, idesc32, 1);
            }
        tc::mma_commit(bar);
    }
    const bool ok = __all_sync(0xffffffffu, tc::mbar_wait_bounded(bar, 0, WAIT_LIMIT));
    tc::fence_after_sync();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = warp & 3, quarter = warp >> 2;
    if (ok) {
        const uint32_t lanes = (uint32_t)(32 * sub) << 16;
        // the B tile is no longer read: the field exchange reuses it
        for (int t = 0; t < L.tiles; t++) {
            float vm[8], vc[8];
            tc::tmem_ld8(tmem + lanes + 64 * t + 8 * quarter, vm);
            tc::tmem_ld8(tmem + lanes + 64 * t + 32 + 8 * quarter, vc);
            tc::tmem_ld_wait();
            const int row = 128 * t + 32 * sub + lane;
            if (row < L.n3)
                for (int c = 0; c < 8; c++)
                    sH[row * HS_STRIDE + 8 * quarter + c] = vm[c] + vc[c] * (1.0f / tc::SPLIT_SCALE);
        }
    }
    tc::fence_before_sync();
    const bool any_bad = __syncthreads_or(!ok);
    if (any_bad) {
        if (threadIdx.x == 0) atomicOr(flag, 1);
        // the MMAs may still be in flight: wait for them (bounded) before the
        // tensor memory is released
        tc::mbar_wait_bounded(bar, 0, WAIT_LIMIT);
    } else {
        for (int i = threadIdx.x; i < n * NM; i += blockDim.x) {
            const int q = i % n, j = i / n;
            if (base + j < E)
                for (int c = 0; c < 3; c++)
                    h[((base + j) * n + q) * 3 + c] = (double)sH[(3 * q + c) * HS_STRIDE + j];
        }
    }
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc::fence_after_sync();
        tc::tmem_dealloc(tmem, tmem_cols(L));
    }
}

// ---- the integrator ----
// Items are (particle q, member j) pairs.  In each group warp w serves the
// 8 members j = 8 (w % 2) + (lane % 8) and the particle pairs
// pp = 4 (w / 2) + lane / 8, so a thread owns particles 2 pp and 2 pp + 1 of
// one member per group (one generator call gives the pair's six normals, and
// the pair's six components are three aligned words of a B-tile row), and
// the same particles of the same member slot in both groups.
// Per item the state is a float-float triple x; between the two Heun stages
// it keeps A = F(m, v1) / 2 and the increments w; the stage map F and the
// state update are those of llg32.cuh.

// Offsets in a group's B tile (32 rows: B_hi rows 0..15, B_lo rows 16..31)
// of the pair's three words, K = 6 pp + 2 s (s = 0, 1, 2): even K, so each
// word holds two consecutive K elements of one core-matrix row.  Packed as
// o01 = o0 | o1 << 16 and o2 (element offsets).
constexpr uint32_t G_LO_SHIFT = (GM / 8) * 64;  // element distance from row j to row j + 16
__device__ inline void pair_offsets(int j, int pp, uint32_t &o01, uint32_t &o2)
{
    o01 = tc::cm_offset(j, 6 * pp, 2 * GM) | (tc::cm_offset(j, 6 * pp + 2, 2 * GM) << 16);
    o2 = tc::cm_offset(j, 6 * pp + 4, 2 * GM);
}

// One word of B_hi and of B_lo: x ~ hi + lo / 2048 for two K elements.
__device__ inline void put_word(__half *bt, uint32_t o, float a, float b)
{
    const __half2 h = __floats2half2_rn(a, b);
    const float2 f = __half22float2(h);
    const __half2 l = __floats2half2_rn((a - f.x) * tc::SPLIT_SCALE, (b - f.y) * tc::SPLIT_SCALE);
    *reinterpret_cast<__half2 *>(bt + o) = h;
    *reinterpret_cast<__half2 *>(bt + o + G_LO_SHIFT) = l;
}

// The six components (particle 2 pp: m[0..2], 2 pp + 1: m[3..5]) of a
// member slot.  A particle past the cluster (2 pp + 1 = n for odd n) writes
// zeros where its word shares a row with the last particle, and its last
// word (which may lie past the tile's K) not at all.
__device__ inline void put_pair(__half *bt, uint32_t o01, uint32_t o2, bool live0, bool live1,
                                const float m[6])
{
    if (!live0) return;
    put_word(bt, o01 & 0xffffu, m[0], m[1]);
    put_word(bt, o01 >> 16, m[2], live1 ? m[3] : 0.f);
    if (live1) put_word(bt, o2, m[4], m[5]);
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

// Item k (0 or 1) of a thread's packed state as a float-float triple; the
// low words of component c at xl[c ITEM_THREADS].
__device__ inline void item_state(DDf out[3], const float2 xh[3], const float2 *xl, int k)
{
#pragma unroll
    for (int c = 0; c < 3; c++) {
        const float2 lo = xl[c * ITEM_THREADS];
        out[c] = k == 0 ? DDf{xh[c].x, lo.x} : DDf{xh[c].y, lo.y};
    }
}

// Per-CTA state of the two groups' tensor-core rounds.
struct Rounds {
    TcLayout L;
    __half *sB[2];
    float *sH[2];
    uint64_t *bar;
    uint32_t tmem;
    uint32_t phase[2];
    uint32_t limit;  // polls of a phase wait before the watchdog gives up
    bool inflight[2];
};

// D (global, row-group-outermost FP16 splits) -> tensor memory.  Warp w of
// the item warps stores, for its sub-partition's 32 lanes, the (tile, split)
// pairs u = w / 4, w / 4 + 4, ..., eight columns at a time (KP / 2 is a
// multiple of 8); rows past the stored ones are zero.
__device__ inline void load_d_tmem(const Rounds &R, const __half *dhi)
{
    const TcLayout &L = R.L;
    if (threadIdx.x >= ITEM_THREADS) return;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = warp & 3, quarter = warp >> 2;
    const size_t split = (size_t)8 * L.rg * L.KP;  // elements of one split
    const int ncol = L.KP / 2;
    for (int u = quarter; u < 2 * L.tiles; u += 4) {
        const int t = u >> 1, sp = u & 1;
        const int r = 128 * t + 32 * sub + lane;
        const __half *src = dhi + sp * split;
        for (int c0 = 0; c0 < ncol; c0 += 8) {
            uint32_t v[8];
#pragma unroll
            for (int i = 0; i < 8; i++)
                v[i] = r < 8 * L.rg
                           ? *reinterpret_cast<const uint32_t *>(
                                 src + tc::cm_offset_rows((uint32_t)r, (uint32_t)(2 * (c0 + i)),
                                                          (uint32_t)L.KP))
                           : 0u;
            const uint32_t col = tmem_d_col(L, t, sp) + (uint32_t)c0;
            tc::tmem_st8(R.tmem + ((uint32_t)(32 * sub) << 16) + col, v);
        }
    }
    tc::tmem_st_wait();
}

// Issue group g's MMAs (issuing warps only).  Called right after a CTA
// barrier that follows all writes of the group's B tile (each writer fenced
// them to the async proxy before the barrier).  Issuing warp t issues the
// chain of tile t -- the whole warp runs the chain and one elected lane
// issues each MMA, so the operands stay warp-uniform -- and commits it to
// the group's mbarrier (which expects one arrival per tile); the tiles'
// chains go out in parallel.
__device__ inline void issue(Rounds &R, int g)
{
    const int it = ((int)threadIdx.x - ITEM_THREADS) >> 5;
    if (it < R.L.tiles) {  // warp-uniform
        tc::fence_after_sync();
        constexpr uint32_t idesc32 = tc::idesc_f16_f32(128, 2 * GM);
        constexpr uint32_t idesc16 = tc::idesc_f16_f32(128, GM);
        constexpr uint32_t b_lbo = (2 * GM / 8) * 128;
        constexpr uint32_t b_kstep = (2 * b_lbo) >> 4;
        const uint64_t b0 = tc::smem_desc(tc::smem_addr(R.sB[g]), b_lbo, 128);
        const int ksteps = R.L.KP / 16;
        const uint32_t acc = R.tmem + 64 * it + 32 * g;
        const uint32_t a_hi = R.tmem + tmem_d_col(R.L, it, 0);
        const uint32_t a_lo = R.tmem + tmem_d_col(R.L, it, 1);
        for (int s = 0; s < ksteps; s++) {
            const uint64_t b = b0 + (uint64_t)(b_kstep * s);
            // [main | corr] (+)= D_hi [B_hi | B_lo]; corr += D_lo B_hi  (K = 16)
            tc::mma_f16_ta_warp(acc, a_hi + 8 * s, b, idesc32, s > 0);
            tc::mma_f16_ta_warp(acc + GM, a_lo + 8 * s, b, idesc16, 1);
        }
        tc::mma_commit_warp(&R.bar[g]);
    }
    R.inflight[g] = true;
}

// Wait for group g's MMAs (bounded), move the accumulators to the group's
// field tile and make it visible to the CTA.  Returns false (uniformly) if
// the completion did not arrive in time.  No MMA is in flight while the
// accumulators are read: the other group's MMAs are issued after this
// function's barrier.  RT_LIMIT: the bound is the plan's run-time setting
// (a separate instantiation: a run-time bound in this wait measured 2.8 %
// slower on the headline workload than the compile-time WAIT_LIMIT).
template <bool RT_LIMIT>
__device__ inline bool finish(Rounds &R, int g)
{
    const bool ok = __all_sync(
        0xffffffffu, tc::mbar_wait_bounded(&R.bar[g], R.phase[g], RT_LIMIT ? R.limit : WAIT_LIMIT));
    tc::fence_after_sync();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int sub = warp & 3, quarter = warp >> 2;
    if (ok && threadIdx.x < ITEM_THREADS) {
        const uint32_t lanes = (uint32_t)(32 * sub) << 16;
        for (int t = 0; t < R.L.tiles; t++) {
            float vm[4], vc[4];
            const uint32_t col = R.tmem + lanes + 64 * t + 32 * g + 4 * quarter;
            tc::tmem_ld4(col, vm);
            tc::tmem_ld4(col + GM, vc);
            tc::tmem_ld_wait();
            const int row = 128 * t + 32 * sub + lane;
            if (row < R.L.n3)
                *reinterpret_cast<float4 *>(R.sH[g] + row * GH_STRIDE + 4 * quarter) =
                    make_float4(fmaf(vc[0], 1.0f / tc::SPLIT_SCALE, vm[0]),
                                fmaf(vc[1], 1.0f / tc::SPLIT_SCALE, vm[1]),
                                fmaf(vc[2], 1.0f / tc::SPLIT_SCALE, vm[2]),
                                fmaf(vc[3], 1.0f / tc::SPLIT_SCALE, vm[3]));
        }
    }
    tc::fence_before_sync();
    if (__syncthreads_or(!ok)) return false;
    R.phase[g] ^= 1u;
    R.inflight[g] = false;
    return true;
}

// The issuing warps' loop: the same sequence of phase waits and CTA
// barriers (finish) as the integrator's step loop below, with the other
// group's MMAs issued after each.  A separate loop, so that none of the
// integrator's state is live where the MMAs are issued.
//
// The issuing warps also compute the applied field ahead, FIELD_BLOCK steps
// at a time (lane l: step 32 b + 1 + l of block b; warp 0 at t, warp 1 at
// t + dt -- an FP64 sine takes ~1.6 k cycles on this part's FP64 pipe, so it
// is paid once per block, not per step).  Block b sits in ring slot b % 2 as
// float2 per step; block b + 1 is written after the first phase barrier of
// block b's first step, and the integrator first reads it more than 30
// steps later; the slot it overwrites (block b - 1) was last read before
// that barrier.
__device__ inline void field_block(float2 *sF2, const MemberDev *md, int64_t b, int64_t K)
{
    const int it = ((int)threadIdx.x - ITEM_THREADS) >> 5, lane = threadIdx.x & 31;
    const int64_t k = FIELD_BLOCK * b + 1 + lane;
    if (k <= K) {
        float *dst = reinterpret_cast<float *>(sF2 + FIELD_BLOCK * (b & 1) + lane);
        dst[it] = f64::heun_field_f32(md->shape, md->dt, md->happ, md->fapp, k, it);
    }
}

template <bool RT_LIMIT>
__device__ inline void issuer_loop(Rounds &R, int64_t K, int64_t noise_steps,
                                   const MemberDev *md, float2 *sF2)
{
    bool alive = true;
    for (int64_t step = 1; step <= K && alive; step++) {
        if (step > noise_steps) break;
#pragma unroll
        for (int g = 0; g < 2; g++) {
            if (!finish<RT_LIMIT>(R, g)) { alive = false; break; }
            issue(R, 1 - g);
            if (g == 0 && ((step - 1) % FIELD_BLOCK) == 0)
                field_block(sF2, md, (step - 1) / FIELD_BLOCK + 1, K);
        }
        if (!alive) break;
#pragma unroll
        for (int g = 0; g < 2; g++) {
            if (!finish<RT_LIMIT>(R, g)) { alive = false; break; }
            if (g == 0 || step < K) issue(R, 1 - g);
        }
    }
}

template <bool RT_LIMIT>
__global__ void __launch_bounds__(TC_THREADS, 1)
    sllg_tc_kernel(DevPlan p, const __half *dhi)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    const int n = p.n;
    Rounds R;
    R.L = tc_layout(n);
    const TcLayout &L = R.L;
    R.sB[0] = (__half *)sm;
    R.sB[1] = (__half *)(sm + L.gb_bytes);
    R.sH[0] = (float *)(sm + 2 * L.gb_bytes);
    R.sH[1] = (float *)(sm + 2 * L.gb_bytes + L.gh_bytes);
    R.bar = (uint64_t *)(sm + L.bar_off);
    uint32_t *slot = (uint32_t *)(sm + L.bar_off + 16);
    int *sFlag = (int *)(sm + L.bar_off + 32);  // [NM] per-member status bits
    // [NM] per-member generator seeds and injected-noise offsets (kept here,
    // not in registers: the integrator's allocation is at its limit)
    uint64_t *sSeed = (uint64_t *)(sm + L.bar_off + 32 + 4 * NM);
    int64_t *sNoff = (int64_t *)(sm + L.bar_off + 32 + 4 * NM + 8 * NM);
    // applied field of step k: h(k dt), h(k dt + dt) in slot ((k - 1) / 32) % 2
    float2 *sF2 = (float2 *)(sm + L.bar_off + 32 + 4 * NM + 16 * NM);
    // per particle pair (2 pp, 2 pp + 1), both particles side by side:
    // (ax, ax', ay, ay'), (az, az', K, K') and sqrt(dt) x noise scale
    float4 *sPar = (float4 *)(sm + L.par_off);
    float2 *sSr = (float2 *)(sm + L.sr_off);
    // kept from stage 1 for stage 2, per (group, item, thread): (A, w0) and (w1, w2)
    // per (group, thread), both items side by side: (A0, A1), (A2, w0),
    // (w1, w2) kept from stage 1 for stage 2, and the state's low words
    float4 *sAW = (float4 *)(sm + L.w_off);
    float2 *sXL = (float2 *)(sm + L.a_off);
    R.phase[0] = R.phase[1] = 0;
    R.limit = p.wait_limit;
    R.inflight[0] = R.inflight[1] = false;

    // both B tiles zero (the K-padding rows 3N..KP stay zero for the run)
    uint4 *bz = (uint4 *)sm;
    for (int i = threadIdx.x; i < (int)(2 * L.gb_bytes / 16); i += blockDim.x)
        bz[i] = make_uint4(0, 0, 0, 0);
    const int64_t base = (int64_t)blockIdx.x * NM;
    const MemberDev *m0d = p.members + base;  // members of a launch share their parameters
    const int64_t P = p.P;
    for (int i = threadIdx.x; i < (n + 1) / 2; i += blockDim.x) {
        float a[2][4], r[2];
        for (int k = 0; k < 2; k++) {
            const int q = 2 * i + k;
            a[k][0] = a[k][1] = a[k][2] = a[k][3] = r[k] = 0.f;
            if (q < n) {
                const int64_t gq = m0d->pbase + q;
                a[k][0] = (float)p.axes[gq];
                a[k][1] = (float)p.axes[P + gq];
                a[k][2] = (float)p.axes[2 * P + gq];
                a[k][3] = (float)p.k_red[gq];
                r[k] = (float)m0d->sqrt_dt * (float)p.sr[gq];
            }
        }
        sPar[2 * i] = make_float4(a[0][0], a[1][0], a[0][1], a[1][1]);
        sPar[2 * i + 1] = make_float4(a[0][2], a[1][2], a[0][3], a[1][3]);
        sSr[i] = make_float2(r[0], r[1]);
    }
    if (threadIdx.x < NM) {
        const int64_t em = base + threadIdx.x;
        const bool ok = em < p.E;
        sFlag[threadIdx.x] = 0;
        sSeed[threadIdx.x] = ok ? p.members[em].seed : 0;
        sNoff[threadIdx.x] = ok ? p.members[em].noise_off : 0;
    }
    if (threadIdx.x == 0) {
        tc::mbar_init(&R.bar[0], (uint32_t)L.tiles);
        tc::mbar_init(&R.bar[1], (uint32_t)L.tiles);
    }
    if (threadIdx.x < 32) tc::tmem_alloc(slot, tmem_cols_int(L));
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    R.tmem = *slot;
    load_d_tmem(R, dhi);  // ordered before the first MMA by the barrier below

    const float dt = (float)m0d->dt, alpha = (float)m0d->alpha;
    const bool renorm = m0d->renorm != 0;
    const int64_t S = p.S;
    const int64_t *sched = p.sched + m0d->sched_off;
    const int64_t K = S > 1 ? sched[S - 1] : 0;
    const int64_t per_step = 3 * (int64_t)n;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int jl = 8 * (warp & 1) + (lane & 7);      // member slot within a group
    // particles 2 pp + k; the issuing warps get pp >= 32: no items
    const int pp = 4 * (warp >> 1) + (lane >> 3);
    const int q0 = 2 * pp;
    const bool live[ITEMS] = {q0 < n, q0 + 1 < n};
    const int64_t e0 = base + jl;  // member of group g: e0 + GM g
    bool valid[2];
    const bool inj = p.noise != nullptr;  // injected increments instead of the generator
    uint32_t o01 = 0, o2 = 0;
    if (q0 < n) pair_offsets(jl, pp, o01, o2);
    // State: component c of both items (particles q0, q0 + 1) as the .x and
    // .y halves of float2 values, float-float: the high words xh in
    // registers, the low words (read and written once per step) in shared
    // memory, sXL[(3 g + c) ITEM_THREADS + thread].  The stage arithmetic runs
    // two items per packed instruction.  A particle past the cluster starts
    // (and stays) at zero.
    float2 xh[2][3];
    float2 *const xlt = sXL + threadIdx.x;
#pragma unroll
    for (int g = 0; g < 2; g++) valid[g] = e0 + GM * g < p.E;
#pragma unroll
    for (int g = 0; g < 2; g++)
        for (int c = 0; c < 3; c++) {
            float hv[ITEMS], lv[ITEMS];
            for (int k = 0; k < ITEMS; k++) {
                const int q = q0 + k;
                hv[k] = lv[k] = 0.f;
                if (q < n && valid[g]) {
                    const double v = p.m0[c * P + (e0 + GM * g) * n + q];
                    hv[k] = (float)v;
                    lv[k] = (float)(v - (double)hv[k]);
                }
            }
            xh[g][c] = make_float2(hv[0], hv[1]);
            if (threadIdx.x < ITEM_THREADS)
                xlt[(3 * g + c) * ITEM_THREADS] = make_float2(lv[0], lv[1]);
        }
#pragma unroll
    for (int g = 0; g < 2; g++) {
        const float m6[6] = {xh[g][0].x, xh[g][1].x, xh[g][2].x,
                             xh[g][0].y, xh[g][1].y, xh[g][2].y};
        put_pair(R.sB[g], o01, o2, live[0], live[1], m6);
        if (p.mx && valid[g])  // sample 0: the initial state (lib/simulation.cpp:212-219)
            for (int k = 0; k < ITEMS; k++)
                if (q0 + k < n) {
                    DDf t[3];
                    item_state(t, xh[g], xlt + 3 * g * ITEM_THREADS, k);
                    write_sample(p, 0, e0 + GM * g, n, q0 + k, t);
                }
    }
    if (threadIdx.x >= ITEM_THREADS) field_block(sF2, m0d, 0, K);  // steps 1..32
    tc::fence_proxy_async();
    tc::fence_before_sync();
    __syncthreads();
    int32_t status = ST_OK;
    int64_t s_next = 1;
    int64_t step = 0;
    bool alive = true;
    // No global load sits at the head of a step: the step of the next sample
    // is kept in a register and the applied field is fetched a step ahead.
    int64_t next_sample = S > 1 ? sched[1] : -1;
    const int64_t noise_steps = p.noise ? m0d->noise_len / per_step : K;
    if (threadIdx.x >= ITEM_THREADS) {  // issuing warps
        if (K > 0) issue(R, 0);
        issuer_loop<RT_LIMIT>(R, K, noise_steps, m0d, sF2);
    } else {
    if (K > 0) R.inflight[0] = true;
    for (step = 1; step <= K && alive; step++) {
        // samples recorded before step `step` hold the state after step-1 steps
        while (next_sample == step) {
            if (p.mx)
                for (int g = 0; g < 2; g++)
                    if (valid[g])
                        for (int k = 0; k < ITEMS; k++)
                            if (q0 + k < n) {
                                DDf t[3];
                                item_state(t, xh[g], xlt + 3 * g * ITEM_THREADS, k);
                                write_sample(p, s_next, e0 + GM * g, n, q0 + k, t);
                            }
            s_next++;
            next_sample = s_next < S ? sched[s_next] : -1;
        }
        if (step > noise_steps) {  // step * 3N > noise_len
            status |= ST_NOISE_EXHAUSTED;
            break;
        }
        const float2 hf = sF2[FIELD_BLOCK * (((step - 1) / FIELD_BLOCK) & 1) + ((step - 1) % FIELD_BLOCK)];
        const float h1 = hf.x, h2 = hf.y;
        // Schedule of a step: (group 0, stage 1), (1, 1), (0, 2), (1, 2).  Each
        // phase reads its group's accumulators, issues the other group's next
        // MMAs, then integrates its group while those run.
        // stage 1 of each group: field at the current state -> predictor
#pragma unroll
        for (int g = 0; g < 2; g++) {
            if (!finish<RT_LIMIT>(R, g)) { status |= ST_WATCHDOG; alive = false; break; }
            R.inflight[1 - g] = true;  // (1, 1) on the state, or (0, 2) on the predictor
            PairNormals wn;
            if (!inj && live[0])
                wn = wiener_pair(sSeed[GM * g + jl], (uint64_t)step, (uint32_t)pp);
            if (live[0]) {
                // both items; a particle past the cluster (odd n) reads the
                // first one's tables, and its results are dropped
                const int qa = q0, qb = live[1] ? q0 + 1 : q0;
                const float *ha = R.sH[g] + 3 * qa * GH_STRIDE + jl;
                const float *hb = R.sH[g] + 3 * qb * GH_STRIDE + jl;
                const float2 hd[3] = {make_float2(ha[0], hb[0]),
                                      make_float2(ha[GH_STRIDE], hb[GH_STRIDE]),
                                      make_float2(ha[2 * GH_STRIDE], hb[2 * GH_STRIDE])};
                const float4 pxy = sPar[2 * pp], pzk = sPar[2 * pp + 1];  // easy axes, K
                const float2 ax = make_float2(pxy.x, pxy.y), ay = make_float2(pxy.z, pxy.w);
                const float2 az = make_float2(pzk.x, pzk.y), ak = make_float2(pzk.z, pzk.w);
                const float2 ssr = sSr[pp];
                float2 w[3];
                if (inj) {
                    float wv[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
                    if (valid[g])
                        for (int k = 0; k < ITEMS; k++)
                            if (k == 0 || live[1]) {
                                const double *wp = p.noise + sNoff[GM * g + jl] +
                                                   (step - 1) * per_step + 3 * (q0 + k);
                                for (int c = 0; c < 3; c++) wv[3 * k + c] = (float)wp[c];
                            }
                    for (int c = 0; c < 3; c++) w[c] = make_float2(wv[c], wv[3 + c]);
                } else {
                    for (int c = 0; c < 3; c++) w[c] = make_float2(wn.n[c], wn.n[3 + c]);
                }
                const float2 *m = xh[g];
                const float2 dot = mul2(fma2(m[2], az, fma2(m[1], ay, mul2(m[0], ax))), ak);
                const float2 v[3] = {
                    fma2(f2(dt), fma2(dot, ax, hd[0]), mul2(ssr, w[0])),
                    fma2(f2(dt), fma2(dot, ay, hd[1]), mul2(ssr, w[1])),
                    fma2(f2(dt), fma2(dot, az, add2(hd[2], f2(h1))), mul2(ssr, w[2]))};
                float2 inc[3];
                llg_F2(inc, m, f2(alpha), v);
                float2 A[3], pr[3];
                for (int c = 0; c < 3; c++) {
                    A[c] = mul2(f2(0.5f), inc[c]);
                    // predictor x~ = x + dt a + sqrt(dt) B w
                    pr[c] = valid[g] ? add2(m[c], inc[c]) : f2(0.f);
                }
                float4 *aw = sAW + 3 * g * ITEM_THREADS + threadIdx.x;
                aw[0] = make_float4(A[0].x, A[0].y, A[1].x, A[1].y);
                aw[ITEM_THREADS] = make_float4(A[2].x, A[2].y, w[0].x, w[0].y);
                aw[2 * ITEM_THREADS] = make_float4(w[1].x, w[1].y, w[2].x, w[2].y);
                const float xt[6] = {pr[0].x, pr[1].x, pr[2].x, pr[0].y, pr[1].y, pr[2].y};
                put_pair(R.sB[g], o01, o2, live[0], live[1], xt);
            }
            tc::fence_proxy_async();
        }
        if (!alive) break;
        // stage 2 of each group: field at the predictor -> corrector
#pragma unroll
        for (int g = 0; g < 2; g++) {
            if (!finish<RT_LIMIT>(R, g)) { status |= ST_WATCHDOG; alive = false; break; }
            // (1, 2) on the predictor, or (0, 1) of the next step on the new state
            if (g == 0 || step < K) R.inflight[1 - g] = true;
            if (live[0]) {
                const int qa = q0, qb = live[1] ? q0 + 1 : q0;
                const float *ha = R.sH[g] + 3 * qa * GH_STRIDE + jl;
                const float *hb = R.sH[g] + 3 * qb * GH_STRIDE + jl;
                const float2 hd[3] = {make_float2(ha[0], hb[0]),
                                      make_float2(ha[GH_STRIDE], hb[GH_STRIDE]),
                                      make_float2(ha[2 * GH_STRIDE], hb[2 * GH_STRIDE])};
                const float4 pxy = sPar[2 * pp], pzk = sPar[2 * pp + 1];
                const float2 ax = make_float2(pxy.x, pxy.y), ay = make_float2(pxy.z, pxy.w);
                const float2 az = make_float2(pzk.x, pzk.y), ak = make_float2(pzk.z, pzk.w);
                const float2 ssr = sSr[pp];
                const float4 *aw = sAW + 3 * g * ITEM_THREADS + threadIdx.x;
                const float4 a01 = aw[0], a2w0 = aw[ITEM_THREADS], w12 = aw[2 * ITEM_THREADS];
                const float2 A[3] = {make_float2(a01.x, a01.y), make_float2(a01.z, a01.w),
                                     make_float2(a2w0.x, a2w0.y)};
                const float2 w[3] = {make_float2(a2w0.z, a2w0.w), make_float2(w12.x, w12.y),
                                     make_float2(w12.z, w12.w)};
                const float2 m[3] = {fma2(f2(2.f), A[0], xh[g][0]), fma2(f2(2.f), A[1], xh[g][1]),
                                     fma2(f2(2.f), A[2], xh[g][2])};
                const float2 dot = mul2(fma2(m[2], az, fma2(m[1], ay, mul2(m[0], ax))), ak);
                const float2 v[3] = {
                    fma2(f2(dt), fma2(dot, ax, hd[0]), mul2(ssr, w[0])),
                    fma2(f2(dt), fma2(dot, ay, hd[1]), mul2(ssr, w[1])),
                    fma2(f2(dt), fma2(dot, az, add2(hd[2], f2(h2))), mul2(ssr, w[2]))};
                float2 inc[3];
                llg_F2(inc, m, f2(alpha), v);
                float2 *xl = xlt + 3 * g * ITEM_THREADS;
                float2 lo[3];
                for (int c = 0; c < 3; c++) {
                    lo[c] = xl[c * ITEM_THREADS];
                    dd_add_ts2(xh[g][c], lo[c], fma2(f2(0.5f), inc[c], A[c]));
                }
                if (renorm) {
                    const float2 n2 = fma2(xh[g][2], xh[g][2],
                                           fma2(xh[g][1], xh[g][1], mul2(xh[g][0], xh[g][0])));
                    const float2 inv = make_float2(1.0f / sqrtf(n2.x), 1.0f / sqrtf(n2.y));
                    for (int c = 0; c < 3; c++) {
                        xh[g][c] = mul2(xh[g][c], inv);
                        lo[c] = mul2(lo[c], inv);
                    }
                }
                for (int c = 0; c < 3; c++) {
                    if (!valid[g]) xh[g][c] = lo[c] = f2(0.f);
                    else if (!live[1]) xh[g][c].y = lo[c].y = 0.f;
                    xl[c * ITEM_THREADS] = lo[c];
                }
                const float m6[6] = {xh[g][0].x, xh[g][1].x, xh[g][2].x,
                                     xh[g][0].y, xh[g][1].y, xh[g][2].y};
                put_pair(R.sB[g], o01, o2, live[0], live[1], m6);
            }
            tc::fence_proxy_async();
        }
        if (!alive) break;
    }
    }
    // the loop leaves `step` one past the last completed step
    step -= 1;
    // MMAs still in flight (a stop before the end): wait for them with the
    // long bound (whatever the phase-wait limit), before the tensor memory is
    // released
    for (int g = 0; g < 2; g++)
        if (R.inflight[g]) tc::mbar_wait_bounded(&R.bar[g], R.phase[g], WAIT_LIMIT);
    if (p.mx)  // samples a stopped member never reached
        for (int g = 0; g < 2; g++)
            if (valid[g])
                for (int64_t s = s_next; s < S; s++)
                    for (int k = 0; k < ITEMS; k++)
                        if (q0 + k < n) {
                            const int64_t o = s * P + (e0 + GM * g) * n + q0 + k;
                            p.mx[o] = NAN; p.my[o] = NAN; p.mz[o] = NAN;
                        }
    for (int g = 0; g < 2; g++) {
        bool bad = false;
        for (int k = 0; k < ITEMS; k++)
            if (q0 + k < n) {
                DDf t[3];
                item_state(t, xh[g], xlt + 3 * g * ITEM_THREADS, k);
                bad |= !(isfinite(t[0].hi) && isfinite(t[1].hi) && isfinite(t[2].hi));
            }
        if (valid[g] && bad) atomicOr(&sFlag[GM * g + jl], ST_NONFINITE);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < NM && base + threadIdx.x < p.E) {
        const int64_t em = base + threadIdx.x;
        if (p.status) p.status[em] = status | sFlag[threadIdx.x];
        if (p.steps) p.steps[em] = step;
    }
    if (threadIdx.x < 32) {
        tc::fence_after_sync();
        tc::tmem_dealloc(R.tmem, tmem_cols_int(L));
    }
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
TcDims tc_dims(int n)
{
    const TcLayout L = tc_layout(n);
    return TcDims{8 * L.rg, L.KP, (size_t)8 * L.rg * L.KP};
}

bool tc_supported(int n)
{
    if (n < 2 || n > 64) return false;
    const TcLayout L = tc_layout(n);
    return L.total <= 232448 && L.total_dip <= 232448;
}

size_t tc_smem_bytes(int n)
{
    const TcLayout L = tc_layout(n);
    return L.total > L.total_dip ? L.total : L.total_dip;
}

cudaError_t tc_build_d(const double *pt, const double *rt, int n, __half **dhi, __half **dlo,
                       cudaStream_t stream)
{
    const TcLayout L = tc_layout(n);
    cudaError_t err = pool_alloc((void **)dhi, 2 * L.d_bytes);
    if (err != cudaSuccess) return err;
    const int rows = 8 * L.rg;
    *dlo = *dhi + (size_t)rows * L.KP;
    const int tot = rows * L.KP;
    build_d_kernel<<<(tot + 255) / 256, 256, 0, stream>>>(pt, rt, n, rows, L.KP, *dhi, *dlo);
    return cudaGetLastError();
}

// Raises the kernels' dynamic shared-memory limit, once per device, to the
// largest layout, so that launches made while a stream is being captured
// need no set-up call (plans call this when they are created).
cudaError_t tc_init_attributes()
{
    static bool done[64] = {};
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
    err = cudaFuncSetAttribute(sllg_tc_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)tc_smem_bytes(64));
    if (err == cudaSuccess)
        err = cudaFuncSetAttribute(sllg_tc_kernel<true>,
                                   cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)tc_smem_bytes(64));
    if (err == cudaSuccess)
        err = cudaFuncSetAttribute(tc_dipolar_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)tc_smem_bytes(64));
    if (err == cudaSuccess && dev >= 0 && dev < 64) done[dev] = true;
    return err;
}

cudaError_t launch_tc(const DevPlan &p, const __half *dhi, const __half *dlo, cudaStream_t stream)
{
    (void)dlo;  // D_lo follows D_hi in the same allocation
    if (p.E == 0) return cudaSuccess;
    if (!tc_supported(p.n)) return cudaErrorNotSupported;
    cudaError_t err = tc_init_attributes();
    if (err != cudaSuccess) return err;
    const unsigned grid = (unsigned)((p.E + NM - 1) / NM);
    // the plan's default phase-wait bound is the compile-time one
    if (p.wait_limit == WAIT_LIMIT)
        sllg_tc_kernel<false><<<grid, TC_THREADS, tc_layout(p.n).total, stream>>>(p, dhi);
    else
        sllg_tc_kernel<true><<<grid, TC_THREADS, tc_layout(p.n).total, stream>>>(p, dhi);
    return cudaGetLastError();
}

cudaError_t launch_tc_dipolar(const __half *dhi, const __half *dlo, int n, int64_t E,
                              const double *m, double *h, int *flag, size_t slack,
                              cudaStream_t stream)
{
    (void)dlo;
    (void)slack;  // the layout already keeps every operand read inside the allocation
    if (!tc_supported(n)) return cudaErrorNotSupported;
    cudaError_t err = tc_init_attributes();
    if (err != cudaSuccess) return err;
    const unsigned grid = (unsigned)((E + NM - 1) / NM);
    tc_dipolar_kernel<<<grid, ITEM_THREADS, tc_layout(n).total_dip, stream>>>(dhi, n, E, m, h,
                                                                            flag);
    return cudaGetLastError();
}

}  // namespace magpy
