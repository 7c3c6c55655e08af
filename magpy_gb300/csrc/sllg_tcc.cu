// sllg_tcc.cu -- mixed-precision sLLG with the dipolar field on the tensor
// cores for clusters of more than 64 particles: one thread-block cluster per
// group of NB members that share one cluster geometry.
//
// The dipolar field of lib/field.cpp:187-225 for members sharing a geometry
// is H = D M, D a fixed 3N x 3N matrix and M the 3N x NB stacked moments.
// D no longer fits one SM's tensor or shared memory, so its rows are split
// over the T = ceil(N / 42) CTAs of a cluster: CTA r owns particles
// [42 r, 42 r + 42) and the 128-row tile r of D, whose rows 3 l + c (l < 42)
// are component c of its particle l (rows 126 and 127 are zero, so no
// particle straddles two tiles).  The K index of D and of M is permuted the
// same way, K = 128 T in all.
//
// Per field evaluation ("stage") of the members of a cluster:
//   1. every CTA has written the FP16 hi/lo split of its particles' moments
//      (its 128-row K slab of B = [B_hi | B_lo], NB members) into a global
//      B buffer, and the cluster barrier orders those writes before step 2;
//   2. one thread streams D tile r and the whole B tile chunk by chunk
//      (cp.async.bulk, K = 64 per chunk, a ring of three stages in shared
//      memory completed on transaction-count mbarriers) and another issues
//      per 16-deep k-step
//          [acc_main | acc_corr]  (+)= D_hi [B_hi | B_lo]   (N = 2 NB)
//           acc_corr              +=  D_lo  B_hi            (N = NB)
//      (tcgen05.mma kind::f16, M = 128, FP32 accumulators in tensor memory);
//   3. the accumulators, h = acc_main + acc_corr / 2048, go through a shared
//      field tile to the threads that integrate the CTA's own particles,
//      which write the next stage's B slab (step 1).
// Everything else -- anisotropy and Zeeman terms, the LLG map, increments
// from the in-kernel generator, the compensated state, samples -- is the
// tensor-core kernel's (sllg_tc.cu) per-particle arithmetic, on the same
// increments (generator counter: the particle pair's global index).
//
// All mbarrier waits are bounded; a wait that runs out marks the CTA, the
// cluster stops together at its next check (every 64 steps, and once after
// the last step, so that a late one is reported too), and every
// CTA drains its own copies and MMAs in flight (long bound) before it frees
// its tensor memory.  Cluster barriers are executed by every thread of every
// CTA the same number of times, whatever happens.
#include <algorithm>
#include <cuda_fp16.h>
#include "common.cuh"
#include "llg32.cuh"
#include "llg64.cuh"
#include "plan.hpp"
#include "tc_cluster.cuh"
#include "tc_ptx.cuh"

namespace magpy {

namespace {

constexpr int PPC = 42;           // particles per CTA
constexpr int RT = 128;           // rows of D per CTA (one MMA tile)
constexpr int KC = 64;            // K elements per streamed chunk
constexpr int NS = 3;             // ring stages
constexpr int PAIRS = PPC / 2;    // particle pairs per CTA
constexpr int ITEMS = 3;          // pair items per integrating thread
constexpr int TCC_MAX_T = 16;     // CTAs per cluster (non-portable above 8)
constexpr int FIELD_BLOCK = 32;   // steps of applied field computed at a time (one per lane)
constexpr uint32_t DRAIN_LIMIT = 1u << 24;
constexpr int32_t ST_WATCHDOG = 16;

// NB members per cluster: 32, 40, 48 or 64 (Heun), 32, 40 or 64 (implicit);
// a multiple of 8, so that the main MMA's N = 2 NB is a multiple of 16.
// Accumulator columns the MMAs write: [main NB | corr NB] from the main MMA,
// and the correction MMA's N = NB rounded up to a multiple of 16 from column
// NB (for NB = 40, eight columns past 2 NB).
__host__ __device__ constexpr int tcc_acc_cols(int nb) { return nb + (nb + 15) / 16 * 16; }
template <int NB> struct Cfg {
    static constexpr int IT = PAIRS * NB / ITEMS;             // integrating threads (7 NB)
    static constexpr int IW = (IT + 31) / 32;                 // integrating warps
    static constexpr int EPI = 8;                             // epilogue warps (0..7)
    static constexpr int PROD = IW > EPI ? IW : EPI;          // producer warp
    static constexpr int MMA = PROD + 1;                      // MMA-issuing warp
    static constexpr int THREADS = 32 * (MMA + 1);
    static constexpr int FS = NB + 4;                         // field-tile row stride (floats)
    // accumulators [main NB | corr NB]; allocations are powers of two >= 32
    static constexpr uint32_t TMEM_COLS =
        tcc_acc_cols(NB) <= 32 ? 32
        : (tcc_acc_cols(NB) <= 64 ? 64 : (tcc_acc_cols(NB) <= 128 ? 128 : 256));
};

struct TccLayout {
    int n, T, K, nK, nb;
    size_t a_chunk, b_chunk, stage;  // bytes: D chunk (hi + lo), B chunk, one ring stage
    size_t f_off, par_off, sr_off, flag_off, bar_off, fld_off, total;
};

__host__ __device__ inline size_t tcc_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

__host__ __device__ inline TccLayout tcc_layout(int n, int nb)
{
    TccLayout L;
    L.n = n;
    L.nb = nb;
    L.T = (n + PPC - 1) / PPC;
    L.K = RT * L.T;
    L.nK = L.K / KC;
    L.a_chunk = (size_t)2 * RT * KC * 2;
    L.b_chunk = (size_t)2 * nb * KC * 2;
    L.stage = L.a_chunk + L.b_chunk;
    L.f_off = NS * L.stage;
    L.par_off = tcc_up(L.f_off + (size_t)RT * (nb + 4) * 4, 16);
    L.sr_off = L.par_off + (size_t)16 * PPC;
    L.flag_off = tcc_up(L.sr_off + (size_t)4 * PPC, 16);
    L.bar_off = tcc_up(L.flag_off + (size_t)4 * (nb + 4), 16);
    // applied-field ring of the Heun kernel: two blocks of FIELD_BLOCK steps,
    // float2 per step
    L.fld_off = tcc_up(L.bar_off + (size_t)8 * (2 * NS + 1) + 16, 16);
    L.total = tcc_up(L.fld_off + (size_t)2 * FIELD_BLOCK * 8, 128);
    return L;
}

// D from the pair tables of one cluster (double), split into FP16 hi/lo and
// stored tile-major: [tile r][chunk kc][split][RT x KC, row groups outermost].
__global__ void tcc_build_d_kernel(const double *pt, const double *rt, int n, int T, int K,
                                   __half *d)
{
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)RT * T * K) return;
    const int row = (int)(idx / K), k = (int)(idx % K);
    const int r = row / RT, lr = row % RT, kc = k / KC, kk = k % KC;
    const int lq = lr / 3, c = lr % 3, q = PPC * r + lq;
    const int j = PPC * (k / RT) + (k % RT) / 3, c2 = (k % RT) % 3;
    double v = 0.0;
    if (lr < 3 * PPC && (k % RT) < 3 * PPC && q < n && j < n && q != j) {
        const double P = pt[(size_t)j * n + q];
        const double rc = rt[((size_t)c * n + j) * n + q];
        const double rc2 = rt[((size_t)c2 * n + j) * n + q];
        v = P * (3.0 * rc * rc2 - (c == c2 ? 1.0 : 0.0));
    }
    const __half hi = __double2half(v);
    const __half lo = __double2half((v - (double)__half2float(hi)) * (double)tc::SPLIT_SCALE);
    const size_t chunk = ((size_t)r * (K / KC) + kc) * (size_t)(2 * RT * KC);
    const uint32_t o = tc::cm_offset_rows((uint32_t)lr, (uint32_t)kk, KC);
    d[chunk + o] = hi;
    d[chunk + RT * KC + o] = lo;
}

// Element offset, inside a B chunk, of (member j, split s, K element kk).
template <int NB>
__device__ inline uint32_t b_off(int j, int s, int kk)
{
    return tc::cm_offset((uint32_t)(j + NB * s), (uint32_t)kk, 2 * NB);
}

// Shared state of the streaming / MMA pipeline of one CTA.
struct Pipe {
    unsigned char *ring;
    uint64_t *full, *empty, *accf;
    uint32_t tmem;
    uint32_t g;       // chunks streamed so far (the same count in every thread)
    uint32_t gemms;   // GEMMs completed (accf phase)
    uint32_t issued;  // producer thread: chunk index past the last copy it issued
    uint32_t commits; // MMA thread: completion commits made on accf
    uint32_t limit;
    uint32_t ncols;   // tensor-memory columns allocated
    uint32_t dcol;    // D resident in tensor memory from this column (0: D streamed)
    uint32_t sbytes;  // bytes per ring stage: D and B chunks, or B alone when D is resident
    uint32_t boff;    // offset of the B chunk in a stage
};

// D B for this CTA's 128 rows and the NB members of the cluster: the
// producer thread streams the chunks of B tile `btile` and, unless D is
// resident in tensor memory (P.dcol != 0), of D tile `dtile`; the MMA thread
// consumes them.  Returns false in the thread whose wait ran out.  Every
// thread advances the chunk count.
template <int NB>
__device__ inline bool tcc_gemm(Pipe &P, const TccLayout &L, const unsigned char *dtile,
                                const unsigned char *btile, int warp, int lane)
{
    bool ok = true;
    if (warp == Cfg<NB>::PROD && lane == 0) {
        tc::fence_proxy_async_global();  // B slabs written by generic stores (peers: barrier)
        for (int i = 0; i < L.nK; i++) {
            const uint32_t gi = P.g + (uint32_t)i, slot = gi % NS, use = gi / NS;
            if (use > 0 && !tc::mbar_wait_bounded(&P.empty[slot], (use - 1) & 1u, P.limit)) {
                ok = false;
                break;
            }
            unsigned char *st = P.ring + slot * P.sbytes;
            P.issued = gi + 1;
            tc::mbar_arrive_expect_tx(&P.full[slot],
                                      (uint32_t)((P.dcol ? 0 : L.a_chunk) + L.b_chunk));
            if (!P.dcol)
                tc::bulk_g2s(st, dtile + (size_t)i * L.a_chunk, (uint32_t)L.a_chunk,
                             &P.full[slot]);
            tc::bulk_g2s(st + P.boff, btile + (size_t)i * L.b_chunk, (uint32_t)L.b_chunk,
                         &P.full[slot]);
        }
    }
    // The whole MMA warp runs the chain (warp-uniform operands) and one
    // elected lane issues each MMA and commit.
    if (warp == Cfg<NB>::MMA) {
        const uint32_t idesc_main = tc::idesc_f16_f32(RT, 2 * NB);
        // D_lo B_hi into [NB, NB + NC): N a multiple of 16 (for NB = 40 the
        // last 8 columns multiply the first B_lo rows into accumulator
        // columns that nothing reads)
        constexpr uint32_t NC = tcc_acc_cols(NB) - NB;
        const uint32_t idesc_corr = tc::idesc_f16_f32(RT, NC);
        const uint32_t a_sbo = (KC / 8) * 128;        // between 8-row groups of D
        const uint32_t b_lbo = (2 * NB / 8) * 128;    // between K-adjacent core matrices of B
        for (int i = 0; i < L.nK; i++) {
            const uint32_t gi = P.g + (uint32_t)i, slot = gi % NS, use = gi / NS;
            if (!__all_sync(0xffffffffu,
                            tc::mbar_wait_bounded(&P.full[slot], use & 1u, P.limit))) {
                ok = false;
                break;
            }
            tc::fence_after_sync();
            const uint32_t a0 = tc::smem_addr(P.ring + slot * P.sbytes);
            const uint32_t b0 = a0 + P.boff;
            if (P.dcol) {
                // A from tensor memory: K element k of split sp in column
                // dcol + sp K/2 + k/2
                const uint32_t ahi = P.tmem + P.dcol + (uint32_t)(KC / 2 * i);
                const uint32_t alo = ahi + (uint32_t)(L.K / 2);
#pragma unroll
                for (int s = 0; s < KC / 16; s++) {
                    const uint64_t bd = tc::smem_desc(b0 + 2u * b_lbo * s, b_lbo, 128);
                    tc::mma_f16_ta_warp(P.tmem, ahi + 8u * s, bd, idesc_main,
                                        (i > 0 || s > 0) ? 1u : 0u);
                    tc::mma_f16_ta_warp(P.tmem + NB, alo + 8u * s, bd, idesc_corr, 1u);
                }
            } else {
#pragma unroll
                for (int s = 0; s < KC / 16; s++) {
                    const uint64_t ahi = tc::smem_desc(a0 + 256u * s, 128, a_sbo);
                    const uint64_t alo = tc::smem_desc(a0 + RT * KC * 2 + 256u * s, 128, a_sbo);
                    const uint64_t bd = tc::smem_desc(b0 + 2u * b_lbo * s, b_lbo, 128);
                    tc::mma_f16_warp(P.tmem, ahi, bd, idesc_main, (i > 0 || s > 0) ? 1u : 0u);
                    tc::mma_f16_warp(P.tmem + NB, alo, bd, idesc_corr, 1u);
                }
            }
            tc::mma_commit_warp(&P.empty[slot]);
        }
        tc::mma_commit_warp(P.accf);  // once every MMA issued above has completed
        P.commits++;
    }
    P.g += (uint32_t)L.nK;
    return ok;
}

// Accumulators -> field tile F[row][member] (epilogue warps 0..7: lane quarter
// warp % 4, member half warp / 4).  Returns false if the completion did not
// arrive in time.
template <int NB>
__device__ inline bool tcc_epilogue(Pipe &P, float *F, int warp, int lane)
{
    bool ok = true;
    if (warp < Cfg<NB>::EPI) {
        ok = __all_sync(0xffffffffu, tc::mbar_wait_bounded(P.accf, P.gemms & 1u, P.limit));
        tc::fence_after_sync();
        if (ok) {
            const int quarter = warp & 3, half = warp >> 2;
            const uint32_t lanes = (uint32_t)(32 * quarter) << 16;
            const int row = 32 * quarter + lane;
            constexpr int HALF = NB / 2;  // member columns per warp (a multiple of 4)
#pragma unroll
            for (int cb = 0; cb < HALF / 8; cb++) {
                const int col = half * HALF + 8 * cb;
                float vm[8], vc[8];
                tc::tmem_ld8(P.tmem + lanes + (uint32_t)col, vm);
                tc::tmem_ld8(P.tmem + lanes + (uint32_t)(NB + col), vc);
                tc::tmem_ld_wait();
                float4 *dst = reinterpret_cast<float4 *>(F + row * Cfg<NB>::FS + col);
                dst[0] = make_float4(fmaf(vc[0], 1.0f / tc::SPLIT_SCALE, vm[0]),
                                     fmaf(vc[1], 1.0f / tc::SPLIT_SCALE, vm[1]),
                                     fmaf(vc[2], 1.0f / tc::SPLIT_SCALE, vm[2]),
                                     fmaf(vc[3], 1.0f / tc::SPLIT_SCALE, vm[3]));
                dst[1] = make_float4(fmaf(vc[4], 1.0f / tc::SPLIT_SCALE, vm[4]),
                                     fmaf(vc[5], 1.0f / tc::SPLIT_SCALE, vm[5]),
                                     fmaf(vc[6], 1.0f / tc::SPLIT_SCALE, vm[6]),
                                     fmaf(vc[7], 1.0f / tc::SPLIT_SCALE, vm[7]));
            }
            if constexpr (HALF % 8 == 4) {  // the last four columns (NB = 40)
                const int col = half * HALF + HALF - 4;
                float vm[4], vc[4];
                tc::tmem_ld4(P.tmem + lanes + (uint32_t)col, vm);
                tc::tmem_ld4(P.tmem + lanes + (uint32_t)(NB + col), vc);
                tc::tmem_ld_wait();
                *reinterpret_cast<float4 *>(F + row * Cfg<NB>::FS + col) =
                    make_float4(fmaf(vc[0], 1.0f / tc::SPLIT_SCALE, vm[0]),
                                fmaf(vc[1], 1.0f / tc::SPLIT_SCALE, vm[1]),
                                fmaf(vc[2], 1.0f / tc::SPLIT_SCALE, vm[2]),
                                fmaf(vc[3], 1.0f / tc::SPLIT_SCALE, vm[3]));
            }
        }
    }
    P.gemms++;
    tc::fence_before_sync();
    return ok;
}

// One word of B_hi and of B_lo (two consecutive K elements) for member j:
// x ~ hi + lo / 2048.
template <int NB>
__device__ inline void put_word_g(__half *chunk, int j, int kk, float a, float b)
{
    const __half2 h = __floats2half2_rn(a, b);
    const float2 f = __half22float2(h);
    const __half2 l = __floats2half2_rn((a - f.x) * tc::SPLIT_SCALE, (b - f.y) * tc::SPLIT_SCALE);
    *reinterpret_cast<__half2 *>(chunk + b_off<NB>(j, 0, kk)) = h;
    *reinterpret_cast<__half2 *>(chunk + b_off<NB>(j, 1, kk)) = l;
}

// The six components of particles 2 p, 2 p + 1 (CTA-local pair p) of member
// j into the CTA's slab of the B tile at `btile` (CTA rank r).  A particle
// past the cluster leaves its words zero (the buffer starts zeroed).
template <int NB>
__device__ inline void put_pair_g(__half *btile, int r, int p, int j, bool live0, bool live1,
                                  const float m[6])
{
    if (!live0) return;
    const int k0 = RT * r + 6 * p;
    const size_t chunk_elems = (size_t)2 * NB * KC;
#pragma unroll
    for (int w = 0; w < 3; w++) {
        if (w == 2 && !live1) break;
        const int k = k0 + 2 * w;
        __half *ch = btile + (size_t)(k / KC) * chunk_elems;
        const float a = m[2 * w], b = (w == 1 && !live1) ? 0.f : m[2 * w + 1];
        put_word_g<NB>(ch, j, k % KC, a, b);
    }
}

__device__ inline void tcc_write_sample(const DevPlan &p, int64_t s, int64_t e, int n, int q,
                                        const DDf xk[3])
{
    const int64_t o = s * p.P + e * n + q;
    const double sc = p.out_scale[e];
    p.mx[o] = ((double)xk[0].hi + (double)xk[0].lo) * sc;
    p.my[o] = ((double)xk[1].hi + (double)xk[1].lo) * sc;
    p.mz[o] = ((double)xk[2].hi + (double)xk[2].lo) * sc;
}

// Common set-up of a CTA: shared-memory carve-up, mbarriers, tensor memory
// (the accumulators, and D when `dres`: then 512 columns).
template <int NB>
__device__ inline void tcc_setup(Pipe &P, unsigned char *sm, const TccLayout &L, uint32_t limit,
                                 bool dres = false)
{
    P.ring = sm;
    P.full = (uint64_t *)(sm + L.bar_off);
    P.empty = P.full + NS;
    P.accf = P.empty + NS;
    uint32_t *slot = (uint32_t *)(P.accf + 1);
    P.g = 0;
    P.gemms = 0;
    P.issued = 0;
    P.commits = 0;
    P.limit = limit;
    P.ncols = dres ? 512u : Cfg<NB>::TMEM_COLS;
    P.dcol = dres ? (uint32_t)tcc_acc_cols(NB) : 0u;  // past every accumulator column
    // with D resident the ring holds B chunks only, packed at its start
    P.sbytes = (uint32_t)(dres ? L.b_chunk : L.stage);
    P.boff = dres ? 0u : (uint32_t)L.a_chunk;
    if (threadIdx.x == 0) {
        for (int i = 0; i < NS; i++) {
            tc::mbar_init(&P.full[i], 1);
            tc::mbar_init(&P.empty[i], 1);
        }
        tc::mbar_init(P.accf, 1);
    }
    if (threadIdx.x < 32) tc::tmem_alloc(slot, P.ncols);
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    P.tmem = *slot;
}

// D tile (global, [chunk][split][128 x KC, row groups outermost]) into tensor
// memory for the MMAs' A operand: row r in lane r, split sp's K element k in
// column dcol + sp K/2 + k/2 (two 16-bit elements per column, the even K in
// the low half).  Warps 0..7: lane quarter warp % 4, split warp / 4.  Ends
// with the stores complete; a CTA barrier must follow before the first MMA.
template <int NB>
__device__ inline void tcc_load_d_tmem(const Pipe &P, const TccLayout &L, const __half *dtile,
                                       int warp, int lane)
{
    if (warp >= 8) return;
    const int quarter = warp & 3, sp = warp >> 2;
    const uint32_t row = (uint32_t)(32 * quarter + lane);
    const uint32_t lanes = (uint32_t)(32 * quarter) << 16;
    for (int c0 = 0; c0 < L.K / 2; c0 += 8) {
        uint32_t v[8];
#pragma unroll
        for (int c = 0; c < 8; c++) {
            const int k = 2 * (c0 + c), kc = k / KC, kk = k % KC;
            const __half *src = dtile + (size_t)(2 * kc + sp) * RT * KC +
                                tc::cm_offset_rows(row, (uint32_t)kk, KC);
            v[c] = *reinterpret_cast<const uint32_t *>(src);
        }
        tc::tmem_st8(P.tmem + lanes + P.dcol + (uint32_t)(sp * (L.K / 2) + c0), v);
    }
    tc::tmem_st_wait();
    tc::fence_before_sync();
}

// Before the tensor memory is released: the producer waits (long bound) for
// the copies it issued, the MMA thread for its MMAs (the last commit).
template <int NB>
__device__ inline void tcc_drain(Pipe &P, int warp, int lane)
{
    if (warp == Cfg<NB>::PROD && lane == 0)
        for (uint32_t k = 0; k < (uint32_t)NS && k < P.issued; k++) {
            const uint32_t gi = P.issued - 1 - k;  // the last copy into each slot
            tc::mbar_wait_bounded(&P.full[gi % NS], (gi / NS) & 1u, DRAIN_LIMIT);
        }
    if (warp == Cfg<NB>::MMA && lane == 0 && P.commits > 0)
        tc::mbar_wait_bounded(P.accf, (P.commits - 1) & 1u, DRAIN_LIMIT);
    tc::fence_before_sync();
    __syncthreads();
    if (threadIdx.x < 32) {
        tc::fence_after_sync();
        tc::tmem_dealloc(P.tmem, P.ncols);
    }
}

// The OR over the cluster of each CTA's error word (every thread gets it).
__device__ inline int cluster_any_error(int *sErr, int T)
{
    __shared__ int any;
    if (threadIdx.x == 0) {
        int a = 0;
        const uint32_t base = tc::smem_addr(sErr);
        for (int r = 0; r < T; r++) a |= tc::ld_cluster_s32(tc::mapa(base, (uint32_t)r));
        any = a;
    }
    __syncthreads();
    return any;
}

// ---- the integrator ----
// Thread t < IT integrates, for member j = t % NB of the cluster's tile, the
// CTA-local particle pairs p = t / NB + 7 i (i < 3), so consecutive threads
// read consecutive members of a field-tile row.
template <int NB, bool DRES>
__global__ void __launch_bounds__(Cfg<NB>::THREADS, 1)
    sllg_tcc_kernel(DevPlan p, const __half *dglob, __half *bglob, int64_t tiles)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    using C = Cfg<NB>;
    const int n = p.n;
    const TccLayout L = tcc_layout(n, NB);
    const int r = (int)tc::cluster_ctarank();
    const int64_t tile = (int64_t)blockIdx.x / L.T;
    Pipe P;
    // DRES (up to three CTAs per cluster, n <= 126): the D tile fits in
    // tensor memory beside the accumulators, is loaded once and only B is
    // streamed; the ring's D slots are then free and hold the stage hand-off
    // instead of registers
    const bool dres = DRES;
    tcc_setup<NB>(P, sm, L, p.wait_limit, dres);
    float *F = (float *)(sm + L.f_off);
    float4 *sPar = (float4 *)(sm + L.par_off);
    float *sSr = (float *)(sm + L.sr_off);
    int *sFlag = (int *)(sm + L.flag_off);  // [NB] member status bits
    int *sErr = sFlag + NB;                 // this CTA's watchdog word
    // applied field of step k, (h(k dt), h(k dt + dt)), in ring slot
    // ((k - 1) / FIELD_BLOCK) % 2
    float2 *sF2 = (float2 *)(sm + L.fld_off);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const MemberDev *m0d = p.members;  // members of a launch share their parameters
    const int64_t P_ = p.P;
    for (int lq = threadIdx.x; lq < PPC; lq += blockDim.x) {
        const int q = PPC * r + lq;
        const int64_t gq = m0d->pbase + (q < n ? q : 0);
        sPar[lq] = make_float4((float)p.axes[gq], (float)p.axes[P_ + gq],
                               (float)p.axes[2 * P_ + gq], (float)p.k_red[gq]);
        sSr[lq] = (float)p.sr[gq];
    }
    if (threadIdx.x < NB) sFlag[threadIdx.x] = 0;
    if (threadIdx.x == 0) *sErr = 0;

    const size_t tile_elems = (size_t)L.K * 2 * NB;  // one B tile (both splits)
    __half *B0 = bglob + (size_t)tile * tile_elems;               // states
    __half *B1 = bglob + (size_t)(tiles + tile) * tile_elems;     // predictors
    const unsigned char *dtile = (const unsigned char *)dglob + (size_t)r * L.nK * L.a_chunk;
    // (ordered before the first MMA by the CTA and cluster barriers below)
    if (dres) tcc_load_d_tmem<NB>(P, L, (const __half *)dtile, warp, lane);
    const float dt = (float)m0d->dt, sq = (float)m0d->sqrt_dt, alpha = (float)m0d->alpha;
    const bool renorm = m0d->renorm != 0;
    const int64_t S = p.S;
    const int64_t *sched = p.sched + m0d->sched_off;
    const int64_t K = S > 1 ? sched[S - 1] : 0;
    const int64_t per_step = 3 * (int64_t)n;

    const bool integ = (int)threadIdx.x < C::IT;
    const int j = (int)threadIdx.x % NB;
    const int p0 = (int)threadIdx.x / NB;
    const int64_t e = tile * NB + j;
    const bool valid = integ && e < p.E;
    const uint64_t seed = valid ? p.members[e].seed : 0;
    const double *noise = (p.noise && valid) ? p.noise + p.members[e].noise_off : nullptr;
    bool live[ITEMS][2];
    // state: float-float per component, the high words in registers; the
    // low words (read and written once per step) in the D ring's freed
    // space when D is resident and there is room (up to 48 members), else
    // in registers
    constexpr bool LO_SMEM = DRES && NB <= 48;
    float xh[ITEMS][2][3], xlr[LO_SMEM ? 1 : ITEMS][2][3];
    // stage hand-off per pair item: A = F(m, v1)/2 and the increments W
    float Areg[ITEMS][6], Wreg[ITEMS][6];
    float *hand = (float *)(sm + NS * L.b_chunk);  // DRES: [24 ITEMS][THREADS]
    auto HA = [&](int i, int c) -> float & {
        if constexpr (DRES) return hand[(i * 6 + c) * C::THREADS + threadIdx.x];
        else return Areg[i][c];
    };
    auto HW = [&](int i, int c) -> float & {
        if constexpr (DRES) return hand[((ITEMS + i) * 6 + c) * C::THREADS + threadIdx.x];
        else return Wreg[i][c];
    };
    float *xlo = hand + 2 * ITEMS * 6 * C::THREADS;  // LO_SMEM: [ITEMS 2 3][THREADS]
    auto XL = [&](int i, int k, int c) -> float & {
        if constexpr (LO_SMEM) return xlo[((i * 2 + k) * 3 + c) * C::THREADS + threadIdx.x];
        else return xlr[LO_SMEM ? 0 : i][k][c];
    };
    auto item = [&](DDf out[3], int i, int k) {
        for (int c = 0; c < 3; c++) out[c] = DDf{xh[i][k][c], XL(i, k, c)};
    };
#pragma unroll
    for (int i = 0; i < ITEMS; i++) {
        const int q0 = PPC * r + 2 * (p0 + 7 * i);
        live[i][0] = valid && q0 < n;
        live[i][1] = valid && q0 + 1 < n;
#pragma unroll
        for (int k = 0; k < 2; k++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                float hi = 0.f, lo = 0.f;
                if (live[i][k]) {
                    const double v = p.m0[c * P_ + e * n + q0 + k];
                    hi = (float)v;
                    lo = (float)(v - (double)hi);
                }
                xh[i][k][c] = hi;
                XL(i, k, c) = lo;
            }
    }
    // initial state -> B0, sample 0 (lib/simulation.cpp:212-219)
#pragma unroll
    for (int i = 0; i < ITEMS; i++) {
        const int pl = p0 + 7 * i;
        const float m6[6] = {xh[i][0][0], xh[i][0][1], xh[i][0][2],
                             xh[i][1][0], xh[i][1][1], xh[i][1][2]};
        put_pair_g<NB>(B0, r, pl, j, live[i][0], live[i][1], m6);
        if (p.mx)
            for (int k = 0; k < 2; k++)
                if (live[i][k]) {
                    DDf t[3];
                    item(t, i, k);
                    tcc_write_sample(p, 0, e, n, PPC * r + 2 * pl + k, t);
                }
    }
    // The producer and MMA warps compute the applied field, FIELD_BLOCK steps
    // at a time (lane l: step 32 b + 1 + l of block b; the producer warp at t,
    // the MMA warp at t + dt; an FP64 sine takes ~1.6 k cycles on this part's
    // FP64 pipe, paid once per block).  Block b + 1 is written at the head of
    // block b's first step; every thread reads it more than 30 steps (and
    // many barriers) later, and the slot it overwrites (block b - 1) was last
    // read a step (and several barriers) earlier.
    auto field_block = [&](int64_t b) {
        if (warp == C::PROD || warp == C::MMA) {
            const int second = warp == C::MMA;
            const int64_t k = FIELD_BLOCK * b + 1 + lane;
            if (k <= K)
                reinterpret_cast<float *>(sF2 + FIELD_BLOCK * (b & 1) + lane)[second] =
                    f64::heun_field_f32(m0d->shape, m0d->dt, m0d->happ, m0d->fapp, k, second);
        }
    };
    field_block(0);
    __syncthreads();

    int32_t status = ST_OK;
    int64_t s_next = 1;
    int64_t step;
    bool stop = false;
    int64_t next_sample = S > 1 ? sched[1] : -1;
    const int64_t noise_steps = p.noise ? m0d->noise_len / per_step : K;
    for (step = 1; step <= K; step++) {
        // the cluster decides together whether to go on: a watchdog in any
        // CTA (checked every 64 steps, and once after the loop), or injected
        // noise running out
        // (the same for every member of the launch)
        if ((step & 63) == 1) {
            tc::cluster_sync();
            if (cluster_any_error(sErr, L.T)) { status |= ST_WATCHDOG; stop = true; }
        }
        if (!stop && step > noise_steps) { status |= ST_NOISE_EXHAUSTED; stop = true; }
        if (stop) break;
        while (next_sample == step) {
            if (p.mx)
#pragma unroll
                for (int i = 0; i < ITEMS; i++)
                    for (int k = 0; k < 2; k++)
                        if (live[i][k]) {
                            DDf t[3];
                            item(t, i, k);
                            tcc_write_sample(p, s_next, e, n, PPC * r + 2 * (p0 + 7 * i) + k, t);
                        }
            s_next++;
            next_sample = s_next < S ? sched[s_next] : -1;
        }
        if ((step - 1) % FIELD_BLOCK == 0) field_block((step - 1) / FIELD_BLOCK + 1);
        const float2 hf =
            sF2[FIELD_BLOCK * (((step - 1) / FIELD_BLOCK) & 1) + (step - 1) % FIELD_BLOCK];
        const float h1 = hf.x, h2 = hf.y;
#pragma unroll 1
        for (int stage = 0; stage < 2; stage++) {
            // every CTA's slab of this stage's B tile is written
            tc::fence_proxy_async_global();
            tc::cluster_sync();
            const __half *Bin = stage == 0 ? B0 : B1;
            bool ok = true;
            // a CTA whose pipeline broke skips its waits (read once per warp:
            // the MMA warp's collectives need the whole warp)
            if (__shfl_sync(0xffffffffu, *sErr, 0) == 0)
                ok = tcc_gemm<NB>(P, L, dtile, (const unsigned char *)(Bin + 0), warp, lane);
            else
                P.g += (uint32_t)L.nK;
            ok = (*sErr == 0 ? tcc_epilogue<NB>(P, F, warp, lane) : (P.gemms++, true)) && ok;
            if (!ok) atomicOr(sErr, 1);
            __syncthreads();
            __half *Bout = stage == 0 ? B1 : B0;
            const float hz = stage == 0 ? h1 : h2;
            if (integ) {
#pragma unroll
                for (int i = 0; i < ITEMS; i++) {
                    const int pl = p0 + 7 * i;
                    PairNormals wn;
                    if (stage == 0 && !noise && live[i][0])
                        wn = wiener_pair(seed, (uint64_t)step, (uint32_t)(PAIRS * r + pl));
                    float m6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
#pragma unroll
                    for (int k = 0; k < 2; k++) {
                        if (!live[i][k]) continue;
                        const int lr = 6 * pl + 3 * k;
                        const float hd0 = F[lr * C::FS + j], hd1 = F[(lr + 1) * C::FS + j],
                                    hd2 = F[(lr + 2) * C::FS + j];
                        // particle constants from shared memory (registers are
                        // kept for the state and the stage hand-off)
                        const float4 pa = sPar[2 * pl + k];
                        const float ssr = sq * sSr[2 * pl + k];
                        if (stage == 0) {
                            if (noise) {
                                const double *wp = noise + (step - 1) * per_step +
                                                   3 * (PPC * r + 2 * pl + k);
                                HW(i, 3 * k) = (float)wp[0];
                                HW(i, 3 * k + 1) = (float)wp[1];
                                HW(i, 3 * k + 2) = (float)wp[2];
                            } else {
                                HW(i, 3 * k) = wn.n[3 * k];
                                HW(i, 3 * k + 1) = wn.n[3 * k + 1];
                                HW(i, 3 * k + 2) = wn.n[3 * k + 2];
                            }
                        }
                        const float w[3] = {HW(i, 3 * k), HW(i, 3 * k + 1), HW(i, 3 * k + 2)};
                        float m[3];
                        if (stage == 0) {
                            m[0] = xh[i][k][0]; m[1] = xh[i][k][1]; m[2] = xh[i][k][2];
                        } else {
                            m[0] = xh[i][k][0] + 2.f * HA(i, 3 * k);
                            m[1] = xh[i][k][1] + 2.f * HA(i, 3 * k + 1);
                            m[2] = xh[i][k][2] + 2.f * HA(i, 3 * k + 2);
                        }
                        const float dot = (m[0] * pa.x + m[1] * pa.y + m[2] * pa.z) * pa.w;
                        const float v[3] = {fmaf(dt, dot * pa.x + hd0, ssr * w[0]),
                                            fmaf(dt, dot * pa.y + hd1, ssr * w[1]),
                                            fmaf(dt, dot * pa.z + hz + hd2, ssr * w[2])};
                        float inc[3];
                        llg_F(inc, m, alpha, v);
                        if (stage == 0) {
                            // predictor x~ = x + dt a + sqrt(dt) B w
#pragma unroll
                            for (int c = 0; c < 3; c++) {
                                HA(i, 3 * k + c) = 0.5f * inc[c];
                                m6[3 * k + c] = m[c] + inc[c];
                            }
                        } else {
#pragma unroll
                            for (int c = 0; c < 3; c++)
                            {
                                const DDf t = dd_add_ts(DDf{xh[i][k][c], XL(i, k, c)},
                                                        fmaf(0.5f, inc[c], HA(i, 3 * k + c)));
                                xh[i][k][c] = t.hi;
                                XL(i, k, c) = t.lo;
                            }
                            if (renorm) {
                                const float nrm = sqrtf(xh[i][k][0] * xh[i][k][0] +
                                                        xh[i][k][1] * xh[i][k][1] +
                                                        xh[i][k][2] * xh[i][k][2]);
                                const float inv = 1.0f / nrm;
                                for (int c = 0; c < 3; c++) {
                                    xh[i][k][c] *= inv;
                                    XL(i, k, c) *= inv;
                                }
                            }
                            m6[3 * k] = xh[i][k][0];
                            m6[3 * k + 1] = xh[i][k][1];
                            m6[3 * k + 2] = xh[i][k][2];
                        }
                    }
                    put_pair_g<NB>(Bout, r, pl, j, live[i][0], live[i][1], m6);
                }
            }
        }
    }
    // the loop leaves `step` one past the last completed step
    step -= 1;
    // a wait that ran out after the last check is reported too
    tc::cluster_sync();
    if (cluster_any_error(sErr, L.T)) status |= ST_WATCHDOG;
    if (p.mx)  // samples a stopped member never reached
        for (int64_t s = s_next; s < S; s++)
#pragma unroll
            for (int i = 0; i < ITEMS; i++)
                for (int k = 0; k < 2; k++)
                    if (live[i][k]) {
                        const int64_t o = s * P_ + e * n + PPC * r + 2 * (p0 + 7 * i) + k;
                        p.mx[o] = NAN; p.my[o] = NAN; p.mz[o] = NAN;
                    }
    bool bad = false;
#pragma unroll
    for (int i = 0; i < ITEMS; i++)
        for (int k = 0; k < 2; k++)
            if (live[i][k])
                bad |= !(isfinite(xh[i][k][0]) && isfinite(xh[i][k][1]) &&
                         isfinite(xh[i][k][2]));
    if (bad) atomicOr(&sFlag[j], ST_NONFINITE);
    tcc_drain<NB>(P, warp, lane);
    // member status: the OR over the cluster's CTAs, written by CTA 0
    tc::cluster_sync();
    if (r == 0 && threadIdx.x < NB && tile * NB + threadIdx.x < p.E) {
        const int64_t em = tile * NB + threadIdx.x;
        int32_t st = status;
        const uint32_t base = tc::smem_addr(&sFlag[threadIdx.x]);
        for (int rr = 0; rr < L.T; rr++) st |= tc::ld_cluster_s32(tc::mapa(base, (uint32_t)rr));
        if (p.status) p.status[em] = st;
        if (p.steps) p.steps[em] = step;
    }
    tc::cluster_sync();  // no CTA leaves while another may read its shared memory
}

// Dipolar field alone: h = D m for E members of one cluster (m, h: [E][n][3]
// double), through the same tiles and pipeline; one stage.
template <int NB>
__global__ void __launch_bounds__(Cfg<NB>::THREADS, 1)
    tcc_dipolar_kernel(int n, int64_t E, const __half *dglob, __half *bglob, const double *m,
                       double *h, int *flag)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    using C = Cfg<NB>;
    const TccLayout L = tcc_layout(n, NB);
    const int r = (int)tc::cluster_ctarank();
    const int64_t tile = (int64_t)blockIdx.x / L.T;
    Pipe P;
    tcc_setup<NB>(P, sm, L, DRAIN_LIMIT);
    float *F = (float *)(sm + L.f_off);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __half *Bt = bglob + (size_t)tile * L.K * 2 * NB;
    const unsigned char *dtile = (const unsigned char *)dglob + (size_t)r * L.nK * L.a_chunk;
    for (int u = threadIdx.x; u < PAIRS * NB; u += blockDim.x) {
        const int j = u % NB, pl = u / NB;
        const int64_t e = tile * NB + j;
        const int q0 = PPC * r + 2 * pl;
        float m6[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const bool l0 = e < E && q0 < n, l1 = e < E && q0 + 1 < n;
        for (int k = 0; k < 2; k++)
            if (k == 0 ? l0 : l1)
                for (int c = 0; c < 3; c++) m6[3 * k + c] = (float)m[(e * n + q0 + k) * 3 + c];
        put_pair_g<NB>(Bt, r, pl, j, l0, l1, m6);
    }
    tc::fence_proxy_async_global();
    tc::cluster_sync();
    bool ok = tcc_gemm<NB>(P, L, dtile, (const unsigned char *)Bt, warp, lane);
    ok = tcc_epilogue<NB>(P, F, warp, lane) && ok;
    if (__syncthreads_or(!ok)) {
        if (threadIdx.x == 0) atomicOr(flag, 1);
    } else {
        for (int u = threadIdx.x; u < PPC * NB; u += blockDim.x) {
            const int j = u % NB, lq = u / NB;
            const int64_t e = tile * NB + j;
            const int q = PPC * r + lq;
            if (e < E && q < n)
                for (int c = 0; c < 3; c++)
                    h[(e * n + q) * 3 + c] = (double)F[(3 * lq + c) * C::FS + j];
        }
    }
    tcc_drain<NB>(P, warp, lane);
    tc::cluster_sync();
}

// ---- implicit midpoint (lib/integrators.cpp:576-651) with the Newton
// iteration of lib/optimisation.cpp:81-149, mixed precision ----
// The members of a thread-block cluster iterate in lockstep: one cluster GEMM
// per iteration gives the dipolar field at every member's current iterate; a
// member whose iteration has stopped keeps its state (its columns of the
// product are computed and not used), so each member takes the iterations
// the per-member loop would.  State, increments, residual and the
// convergence norms are FP64; the dipolar field comes from the tensor cores
// (~22 significant bits) and the quasi-Jacobian and its 3x3 solves are FP32,
// as in the mixed implicit mode of the CUDA-core kernel.  The Newton
// equation, its FP64 residual and the stopping test (|dx| <= eps |guess|,
// member-wide, at most max_iter iterations) are the reference's; the
// Jacobian that steers it is J = I - dt a'/2 - sum_k b'_k dwm_k / 2 with each
// particle's own anisotropy field Jacobian k e e^T and without the dipolar
// coupling (block-diagonal).  The reference writes the drift term without dt
// (integrators.cpp:633) and hands llg::drift_jacobian another particle's
// block of the field Jacobian (llg.cpp:386); its iteration then contracts by
// ~1/2 per step and needs ~40 iterations per step at dt = 2e-13 s, this one
// by ~dt |D| and a few.  Both converge to the same root within the same
// tolerance (the FP64-faithful kernel keeps the reference's iteration).  The member-wide norms are summed
// over the CTA's particles in a fixed order, then over the cluster's CTAs in
// rank order through distributed shared memory: every CTA takes the same
// decisions from the same numbers.
//
// Stage increments use dt a + B dwm = F(m, dt h + sr dwm), the LLG map of
// llg32.cuh in FP64 (drift and diffusion share the form).
__device__ inline void llg_F64(double o[3], const double m[3], double alpha, const double v[3])
{
    const double c0 = m[1] * v[2] - m[2] * v[1];
    const double c1 = m[2] * v[0] - m[0] * v[2];
    const double c2 = m[0] * v[1] - m[1] * v[0];
    const double mv = m[0] * v[0] + m[1] * v[1] + m[2] * v[2];
    const double mm = m[0] * m[0] + m[1] * m[1] + m[2] * m[2];
    o[0] = fma(alpha, v[0] * mm - m[0] * mv, -c0);
    o[1] = fma(alpha, v[1] * mm - m[1] * mv, -c1);
    o[2] = fma(alpha, v[2] * mm - m[2] * mv, -c2);
}

// Per-particle constants of a CTA's 42 particles: FP64 for the residual,
// FP32 copies for the Jacobian.
struct ImpPar {
    double ax[PPC][3], k[PPC], sr[PPC];
    float axf[PPC][3], kf[PPC], srf[PPC], hjf[PPC][9];
};

__host__ __device__ inline size_t tcc_imp_smem(const TccLayout &L)
{
    // after the Heun layout: particle constants, per-(p0, member) partial
    // sums, and the cluster-exchanged partials / flags (double-buffered)
    // ... and, in the 32- and 40-member forms, each particle's step increments kept
    // for the Newton iterations: sr dwm (FP64) and dwm (FP32), 3 each
    const size_t kept =
        L.nb <= 40 ? (size_t)(8 + 4) * 3 * 2 * ITEMS * (PAIRS * (size_t)L.nb / ITEMS) : 0;
    return tcc_up(L.total, 16) + sizeof(ImpPar) + (size_t)8 * 7 * L.nb + (size_t)8 * 2 * L.nb +
           (size_t)4 * 2 * L.nb + (size_t)8 * L.nb + (size_t)4 * L.nb + 64 + kept;
}

template <int NB>
__global__ void __launch_bounds__(Cfg<NB>::THREADS, 1)
    sllg_tcc_implicit_kernel(DevPlan p, const __half *dglob, __half *bglob, int64_t tiles)
{
    extern __shared__ __align__(1024) unsigned char sm[];
    using C = Cfg<NB>;
    const int n = p.n;
    const TccLayout L = tcc_layout(n, NB);
    const int r = (int)tc::cluster_ctarank();
    const int64_t tile = (int64_t)blockIdx.x / L.T;
    Pipe P;
    tcc_setup<NB>(P, sm, L, p.wait_limit);
    float *F = (float *)(sm + L.f_off);
    int *sFlag = (int *)(sm + L.flag_off);  // [NB] member status bits (this CTA)
    int *sErr = sFlag + NB;
    unsigned char *xs = sm + tcc_up(L.total, 16);
    ImpPar *par = (ImpPar *)xs;
    double *red = (double *)(xs + sizeof(ImpPar));          // [7][NB]
    double *part = red + 7 * NB;                              // [2][NB] exchanged
    int *pflag = (int *)(part + 2 * NB);                      // [2][NB] exchanged
    double *sNorm = (double *)(pflag + 2 * NB);               // [NB] combined norm
    int *sSing = (int *)(sNorm + NB);                         // [NB] combined singular flag
    double *sField = (double *)(sSing + NB);                  // applied field at t, t + dt/2
    // 32-member form: the step's sr dwm (FP64) and dwm (FP32) per particle,
    // [(i*2 + k)*3 + c][IT], written at the initial guess, read by the
    // Newton iterations (the larger forms recompute them)
    constexpr bool KEEP_DW = NB <= 40;
    double *sSdw = sField + 8;
    float *sDwf = (float *)(sSdw + (KEEP_DW ? 6 * ITEMS * C::IT : 0));

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const MemberDev *m0d = p.members;
    const int64_t P_ = p.P;
    for (int lq = threadIdx.x; lq < PPC; lq += blockDim.x) {
        const int q = PPC * r + lq;
        const int64_t gq = m0d->pbase + (q < n ? q : 0);
        for (int c = 0; c < 3; c++) par->ax[lq][c] = p.axes[c * P_ + gq];
        par->k[lq] = p.k_red[gq];
        par->sr[lq] = p.sr[gq];
        for (int c = 0; c < 3; c++) par->axf[lq][c] = (float)par->ax[lq][c];
        par->kf[lq] = (float)par->k[lq];
        par->srf[lq] = (float)par->sr[lq];
        // the particle's own anisotropy field Jacobian k e e^T
        for (int a = 0; a < 3; a++)
            for (int b = 0; b < 3; b++)
                par->hjf[lq][3 * a + b] = (float)(par->k[lq] * par->ax[lq][a] * par->ax[lq][b]);
    }
    if (threadIdx.x < NB) sFlag[threadIdx.x] = 0;
    if (threadIdx.x == 0) *sErr = 0;

    const size_t tile_elems = (size_t)L.K * 2 * NB;
    __half *Bbuf[2] = {bglob + (size_t)tile * tile_elems, bglob + (size_t)(tiles + tile) * tile_elems};
    const unsigned char *dtile = (const unsigned char *)dglob + (size_t)r * L.nK * L.a_chunk;

    const double dt = m0d->dt, sq = m0d->sqrt_dt, alpha = m0d->alpha, Ah = m0d->Ah;
    const double eps = m0d->eps;
    const int64_t max_iter = m0d->max_iter;
    const float alpha_f = (float)alpha, dt_f = (float)dt, sq_f = (float)sq;
    const bool renorm = m0d->renorm != 0;
    const int64_t S = p.S;
    const int64_t *sched = p.sched + m0d->sched_off;
    const int64_t K = S > 1 ? sched[S - 1] : 0;
    const int64_t per_step = 3 * (int64_t)n;

    const bool integ = (int)threadIdx.x < C::IT;
    const int j = (int)threadIdx.x % NB;
    const int p0 = (int)threadIdx.x / NB;
    const int64_t e = tile * NB + j;
    const bool valid = integ && e < p.E;
    const uint64_t seed = valid ? p.members[e].seed : 0;
    const double *noise = (p.noise && valid) ? p.noise + p.members[e].noise_off : nullptr;
    bool live[ITEMS][2];
    double x[ITEMS][2][3], px[ITEMS][2][3];
#pragma unroll
    for (int i = 0; i < ITEMS; i++) {
        const int q0 = PPC * r + 2 * (p0 + 7 * i);
        live[i][0] = valid && q0 < n;
        live[i][1] = valid && q0 + 1 < n;
#pragma unroll
        for (int k = 0; k < 2; k++)
#pragma unroll
            for (int c = 0; c < 3; c++) {
                x[i][k][c] = live[i][k] ? p.m0[c * P_ + e * n + q0 + k] : 0.0;
                px[i][k][c] = x[i][k][c];
            }
    }
    int wb = 0;  // B buffer the next GEMM reads
    int pc = 0;  // partials buffer of the next exchange
    auto write_B = [&](int buf) {
#pragma unroll
        for (int i = 0; i < ITEMS; i++) {
            const float m6[6] = {(float)x[i][0][0], (float)x[i][0][1], (float)x[i][0][2],
                                 (float)x[i][1][0], (float)x[i][1][1], (float)x[i][1][2]};
            put_pair_g<NB>(Bbuf[buf], r, p0 + 7 * i, j, live[i][0], live[i][1], m6);
        }
    };
    // Member-wide sum of `v` over the cluster (fixed order); returns it in the
    // threads of member j, and ORs `flag` likewise.  Ends with a CTA barrier.
    auto cluster_sum = [&](double v, int flag, double &sum, int &any) {
        if (integ) red[p0 * NB + j] = v;
        if (integ && flag) atomicOr(&pflag[pc * NB + j], 1);
        __syncthreads();
        if (threadIdx.x < NB) {
            double s_ = 0.0;
            for (int q = 0; q < 7; q++) s_ += red[q * NB + threadIdx.x];
            part[pc * NB + threadIdx.x] = s_;
        }
        tc::fence_proxy_async_global();  // this stage's B slab (generic stores) -> bulk reads
        tc::cluster_sync();
        if (threadIdx.x < NB) {
            double s_ = 0.0;
            int f_ = 0;
            const uint32_t pa = tc::smem_addr(&part[pc * NB + threadIdx.x]);
            const uint32_t fa = tc::smem_addr(&pflag[pc * NB + threadIdx.x]);
            for (int rr = 0; rr < L.T; rr++) {
                s_ += tc::ld_cluster_f64(tc::mapa(pa, (uint32_t)rr));
                f_ |= tc::ld_cluster_s32(tc::mapa(fa, (uint32_t)rr));
            }
            sNorm[threadIdx.x] = s_;
            sSing[threadIdx.x] = f_;
        }
        __syncthreads();
        // the other buffer is next: clear its flags (no CTA writes it before
        // the next cluster barrier, which every CTA reaches after reading this one)
        if (threadIdx.x < NB) pflag[(pc ^ 1) * NB + threadIdx.x] = 0;
        pc ^= 1;
        sum = sNorm[j];
        any = sSing[j];
    };
    if (threadIdx.x < 2 * NB) pflag[threadIdx.x] = 0;
    write_B(0);
    if (p.mx)  // sample 0: the initial state (lib/simulation.cpp:212-219)
#pragma unroll
        for (int i = 0; i < ITEMS; i++)
            for (int k = 0; k < 2; k++)
                if (live[i][k]) {
                    const int64_t o = e * n + PPC * r + 2 * (p0 + 7 * i) + k;
                    const double sc = p.out_scale[e];
                    p.mx[o] = x[i][k][0] * sc; p.my[o] = x[i][k][1] * sc; p.mz[o] = x[i][k][2] * sc;
                }
    __syncthreads();

    // the GEMM on B[wb] and its field tile; false if a wait ran out
    auto field = [&]() {
        bool ok = true;
        if (__shfl_sync(0xffffffffu, *sErr, 0) == 0)
            ok = tcc_gemm<NB>(P, L, dtile, (const unsigned char *)Bbuf[wb], warp, lane);
        else P.g += (uint32_t)L.nK;
        ok = (*sErr == 0 ? tcc_epilogue<NB>(P, F, warp, lane) : (P.gemms++, true)) && ok;
        if (!ok) atomicOr(sErr, 1);
        __syncthreads();
    };

    int32_t status = ST_OK;
    int64_t s_next = 1;
    int64_t step;
    bool stop = false;
    int64_t next_sample = S > 1 ? sched[1] : -1;
    const int64_t noise_steps = p.noise ? m0d->noise_len / per_step : K;
    for (step = 1; step <= K; step++) {
        if ((step & 63) == 1) {
            tc::cluster_sync();
            if (cluster_any_error(sErr, L.T)) { status |= ST_WATCHDOG; stop = true; }
        }
        if (!stop && step > noise_steps) { status |= ST_NOISE_EXHAUSTED; stop = true; }
        if (stop) break;
        while (next_sample == step) {  // zero-order hold: the state after step - 1 steps
            if (p.mx)
#pragma unroll
                for (int i = 0; i < ITEMS; i++)
                    for (int k = 0; k < 2; k++)
                        if (live[i][k]) {
                            const int64_t o = s_next * P_ + e * n + PPC * r + 2 * (p0 + 7 * i) + k;
                            const double sc = p.out_scale[e];
                            p.mx[o] = x[i][k][0] * sc;
                            p.my[o] = x[i][k][1] * sc;
                            p.mz[o] = x[i][k][2] * sc;
                        }
            s_next++;
            next_sample = s_next < S ? sched[s_next] : -1;
        }
        const double t = (double)step * dt;  // lib/simulation.cpp:350-355
        if (threadIdx.x == 0) {
            sField[0] = f64::field_value(m0d->shape, t, m0d->happ, m0d->fapp);
            sField[1] = f64::field_value(m0d->shape, t + dt / 2, m0d->happ, m0d->fapp);
        }
        // increments of this step, clamped and scaled (integrators.cpp:599-602),
        // are recomputed where needed rather than kept: FP64 for the residual,
        // FP32 for the Jacobian.  The generator's normals never reach the
        // clamp (|w| <= 5.65 < Ah), so only injected increments are clamped.
        auto dwm_of = [&](int i, int k, double out[3], float outf[3]) {
            const int q = PPC * r + 2 * (p0 + 7 * i) + k;
            if (noise) {
                const double *wp = noise + (step - 1) * per_step + 3 * q;
                for (int c = 0; c < 3; c++) {
                    const double lo = (wp[c] < Ah) ? wp[c] : Ah;
                    out[c] = ((-Ah < lo) ? lo : -Ah) * sq;
                    outf[c] = (float)out[c];
                }
            } else {
                const Normals4 nr = wiener_normals(seed, (uint64_t)step, (uint32_t)q);
                const float w[3] = {nr.a, nr.b, nr.c};
                for (int c = 0; c < 3; c++) {
                    out[c] = (double)w[c] * sq;
                    outf[c] = w[c] * sq_f;
                }
            }
        };
        // field at the current state -> the initial guess (g + x0) / 2
        field();
        const double h_t = sField[0], h_m = sField[1];
        double part_v = 0.0;
        if (integ) {
#pragma unroll
            for (int i = 0; i < ITEMS; i++)
#pragma unroll
                for (int k = 0; k < 2; k++) {
                    px[i][k][0] = x[i][k][0]; px[i][k][1] = x[i][k][1]; px[i][k][2] = x[i][k][2];
                    if (!live[i][k]) continue;
                    const int lq = 2 * (p0 + 7 * i) + k;
                    const double *ax = par->ax[lq];
                    const double *m = px[i][k];
                    const double dot = (m[0] * ax[0] + m[1] * ax[1] + m[2] * ax[2]) * par->k[lq];
                    double dwm[3];
                    float dwf[3];
                    dwm_of(i, k, dwm, dwf);
                    const double sr = par->sr[lq];
                    if constexpr (KEEP_DW)
                        for (int c = 0; c < 3; c++) {
                            sSdw[((i * 2 + k) * 3 + c) * C::IT + threadIdx.x] = sr * dwm[c];
                            sDwf[((i * 2 + k) * 3 + c) * C::IT + threadIdx.x] = dwf[c];
                        }
                    const double v[3] = {
                        dt * (dot * ax[0] + (double)F[(3 * lq) * C::FS + j]) + sr * dwm[0],
                        dt * (dot * ax[1] + (double)F[(3 * lq + 1) * C::FS + j]) + sr * dwm[1],
                        dt * (dot * ax[2] + h_t + (double)F[(3 * lq + 2) * C::FS + j]) + sr * dwm[2]};
                    double g[3];
                    llg_F64(g, m, alpha, v);
                    for (int c = 0; c < 3; c++) {
                        x[i][k][c] = (g[c] + m[c]) / 2;
                        part_v += x[i][k][c] * x[i][k][c];
                    }
                }
        }
        write_B(wb ^ 1);
        wb ^= 1;
        double nrm2;
        int sing_any;
        cluster_sum(part_v, 0, nrm2, sing_any);
        const double tol = eps * sqrt(nrm2);
        double err = 2 * tol;
        int64_t iter = max_iter;
        bool active = valid;
        int32_t mflag = ST_OK;
        for (;;) {
            // while ((err > tol) && (iter-- > 0)), per member
            bool go = false;
            if (active) {
                if (err > tol) {
                    go = iter > 0;
                    iter--;
                }
                if (!go) active = false;
            }
            if (!__syncthreads_or(go)) break;
            field();  // dipolar field at every member's current iterate
            double dsum = 0.0;
            int sing = 0;
            if (go) {
#pragma unroll
                for (int i = 0; i < ITEMS; i++)
#pragma unroll
                    for (int k = 0; k < 2; k++) {
                        if (!live[i][k]) continue;
                        const int lq = 2 * (p0 + 7 * i) + k;
                        const double *ax = par->ax[lq];
                        const double xt[3] = {x[i][k][0], x[i][k][1], x[i][k][2]};
                        const double dot =
                            (xt[0] * ax[0] + xt[1] * ax[1] + xt[2] * ax[2]) * par->k[lq];
                        const double h[3] = {dot * ax[0] + (double)F[(3 * lq) * C::FS + j],
                                             dot * ax[1] + (double)F[(3 * lq + 1) * C::FS + j],
                                             dot * ax[2] + h_m +
                                                 (double)F[(3 * lq + 2) * C::FS + j]};
                        double sdw[3];  // sr dwm
                        float dwf[3];
                        if constexpr (KEEP_DW) {
                            for (int c = 0; c < 3; c++) {
                                sdw[c] = sSdw[((i * 2 + k) * 3 + c) * C::IT + threadIdx.x];
                                dwf[c] = sDwf[((i * 2 + k) * 3 + c) * C::IT + threadIdx.x];
                            }
                        } else {
                            double dwm[3];
                            dwm_of(i, k, dwm, dwf);
                            for (int c = 0; c < 3; c++) sdw[c] = par->sr[lq] * dwm[c];
                        }
                        const double v[3] = {fma(dt, h[0], sdw[0]), fma(dt, h[1], sdw[1]),
                                             fma(dt, h[2], sdw[2])};
                        double g[3];
                        llg_F64(g, xt, alpha, v);
                        // F(y) = y - a dt / 2 - x0 - B dwm / 2 (integrators.cpp:621-627)
                        float sol[3];
                        for (int c = 0; c < 3; c++)
                            sol[c] = (float)(fma(0.5, g[c], px[i][k][c]) - xt[c]);
                        // Jacobian in FP32 from FP32 copies of the state and field
                        const float xf[3] = {(float)xt[0], (float)xt[1], (float)xt[2]};
                        const float *axf = par->axf[lq];
                        const float dotf = (xf[0] * axf[0] + xf[1] * axf[1] + xf[2] * axf[2]) *
                                           par->kf[lq];
                        const float hf[3] = {fmaf(dotf, axf[0], F[(3 * lq) * C::FS + j]),
                                             fmaf(dotf, axf[1], F[(3 * lq + 1) * C::FS + j]),
                                             fmaf(dotf, axf[2], F[(3 * lq + 2) * C::FS + j]) +
                                                 (float)h_m};
                        float adash[9], bdash[27], J[9];
                        f64::drift_jacobian<float>(adash, xf, alpha_f, hf, par->hjf[lq]);
                        f64::diffusion_jacobian<float>(bdash, xf, par->srf[lq], alpha_f);
                        for (int rr = 0; rr < 3; rr++)
                            for (int c = 0; c < 3; c++) {
                                float jv = (float)(rr == c) - 0.5f * dt_f * adash[3 * rr + c];
                                for (int kk = 0; kk < 3; kk++)
                                    jv -= 0.5f * bdash[9 * rr + 3 * kk + c] * dwf[kk];
                                J[3 * rr + c] = jv;
                            }
                        if (f64::solve3<float>(J, sol) != 0) {
                            sing = 1;
                            continue;  // the member stops with its current iterate
                        }
                        for (int c = 0; c < 3; c++) {
                            const double d = (double)sol[c];
                            dsum += d * d;
                            x[i][k][c] = xt[c] + d;
                        }
                    }
            }
            write_B(wb ^ 1);
            wb ^= 1;
            double d2;
            cluster_sum(dsum, sing, d2, sing_any);
            err = sqrt(d2);
            if (go && sing_any) { mflag |= ST_SINGULAR; active = false; }
        }
        if (valid && mflag == ST_OK && iter == -1) mflag |= ST_NEWTON_MAXITER;
        status |= mflag;
        // x = 2 y - x0 (integrators.cpp:647), optional renormalisation
        // (lib/simulation.cpp:379-387)
#pragma unroll
        for (int i = 0; i < ITEMS; i++)
#pragma unroll
            for (int k = 0; k < 2; k++) {
                if (!live[i][k]) continue;
                for (int c = 0; c < 3; c++) x[i][k][c] = 2 * x[i][k][c] - px[i][k][c];
                if (renorm) {
                    const double nrm = sqrt(x[i][k][0] * x[i][k][0] + x[i][k][1] * x[i][k][1] +
                                            x[i][k][2] * x[i][k][2]);
                    for (int c = 0; c < 3; c++) x[i][k][c] = x[i][k][c] / nrm;
                }
            }
        write_B(wb ^ 1);
        wb ^= 1;
    }
    step -= 1;
    // a wait that ran out after the last check is reported too
    tc::cluster_sync();
    if (cluster_any_error(sErr, L.T)) status |= ST_WATCHDOG;
    if (p.mx)
        for (int64_t s2 = s_next; s2 < S; s2++)
#pragma unroll
            for (int i = 0; i < ITEMS; i++)
                for (int k = 0; k < 2; k++)
                    if (live[i][k]) {
                        const int64_t o = s2 * P_ + e * n + PPC * r + 2 * (p0 + 7 * i) + k;
                        p.mx[o] = NAN; p.my[o] = NAN; p.mz[o] = NAN;
                    }
    bool bad = false;
#pragma unroll
    for (int i = 0; i < ITEMS; i++)
        for (int k = 0; k < 2; k++)
            if (live[i][k])
                bad |= !(isfinite(x[i][k][0]) && isfinite(x[i][k][1]) && isfinite(x[i][k][2]));
    if (bad) atomicOr(&sFlag[j], ST_NONFINITE);
    if (integ && valid && status) atomicOr(&sFlag[j], status);
    tcc_drain<NB>(P, warp, lane);
    tc::cluster_sync();
    if (r == 0 && threadIdx.x < NB && tile * NB + threadIdx.x < p.E) {
        const int64_t em = tile * NB + threadIdx.x;
        int32_t st = status & (ST_WATCHDOG | ST_NOISE_EXHAUSTED);
        const uint32_t base = tc::smem_addr(&sFlag[threadIdx.x]);
        for (int rr = 0; rr < L.T; rr++) st |= tc::ld_cluster_s32(tc::mapa(base, (uint32_t)rr));
        if (p.status) p.status[em] = st;
        if (p.steps) p.steps[em] = step;
    }
    tc::cluster_sync();
}

template <class Kern>
cudaError_t tcc_prepare(Kern kern, const TccLayout &L, size_t smem)
{
    cudaError_t err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem);
    if (err == cudaSuccess && L.T > 8)
        err = cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
    return err;
}

template <class Kern, class... Args>
cudaError_t tcc_launch(Kern kern, const TccLayout &L, size_t smem, int threads, int64_t tiles,
                       cudaStream_t stream, Args... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(tiles * L.T));
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[2];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)L.T;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    // the stream's scheduling priority, carried into a captured graph node
    // (a batch gives its longest group the highest)
    int prio = 0;
    if (cudaStreamGetPriority(stream, &prio) != cudaSuccess) prio = 0;
    attr[1].id = cudaLaunchAttributePriority;
    attr[1].val.priority = prio;
    cfg.attrs = attr;
    cfg.numAttrs = 2;
    return cudaLaunchKernelEx(&cfg, kern, args...);
}

}  // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
bool tcc_supported(int n) { return n > 64 && n <= PPC * TCC_MAX_T; }

bool tcc_implicit_supported(int n) { return n >= 2 && n <= PPC * TCC_MAX_T; }

int tcc_members_per_cluster(int members_per_warp_hint)
{
    return members_per_warp_hint == 32 ? 32 : 64;
}

size_t tcc_d_elems(int n)
{
    const TccLayout L = tcc_layout(n, 64);
    return (size_t)RT * L.T * L.K * 2;
}

size_t tcc_b_elems(int n, int64_t E, int nb)
{
    const TccLayout L = tcc_layout(n, nb);
    const int64_t tiles = (E + nb - 1) / nb;
    return (size_t)2 * tiles * L.K * 2 * nb;
}

cudaError_t tcc_build_d(const double *pt, const double *rt, int n, __half *d, cudaStream_t stream)
{
    const TccLayout L = tcc_layout(n, 64);
    const int64_t tot = (int64_t)RT * L.T * L.K;
    tcc_build_d_kernel<<<(unsigned)((tot + 255) / 256), 256, 0, stream>>>(pt, rt, n, L.T, L.K, d);
    return cudaGetLastError();
}

// Raises the shared-memory limit (and allows clusters above 8 CTAs) of the
// kernels, once per device, and checks that a cluster of the largest size
// this n needs can be resident.  Called when a plan is created, so that
// launches made while a stream is being captured need no set-up call.
cudaError_t tcc_init(int n, int nb, int *max_clusters)
{
    static bool done[64][3] = {};
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    if (nb != 32 && nb != 40 && nb != 64) return cudaErrorInvalidValue;
    const int w = nb == 32 ? 0 : (nb == 64 ? 1 : 2);  // 2: the 40-member implicit form
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    const TccLayout Lmax = tcc_layout(PPC * TCC_MAX_T, nb);
    const size_t imp = tcc_imp_smem(Lmax);
    if (!done[dev][w] && nb == 40) {
        err = tcc_prepare(sllg_tcc_implicit_kernel<40>, Lmax, imp);
        if (err == cudaSuccess) err = tcc_prepare(sllg_tcc_kernel<40, false>, Lmax, Lmax.total);
        if (err == cudaSuccess) err = tcc_prepare(sllg_tcc_kernel<40, true>, Lmax, Lmax.total);
        if (err != cudaSuccess) return err;
        done[dev][w] = true;
    }
    if (!done[dev][w]) {
        err = nb == 32 ? tcc_prepare(sllg_tcc_kernel<32, false>, Lmax, Lmax.total)
                       : tcc_prepare(sllg_tcc_kernel<64, false>, Lmax, Lmax.total);
        if (err == cudaSuccess)
            err = nb == 32 ? tcc_prepare(sllg_tcc_kernel<32, true>, Lmax, Lmax.total)
                           : tcc_prepare(sllg_tcc_kernel<64, true>, Lmax, Lmax.total);
        if (err == cudaSuccess && nb == 64) {  // the 48-member form, prepared alongside
            const TccLayout L48 = tcc_layout(PPC * TCC_MAX_T, 48);
            err = tcc_prepare(sllg_tcc_kernel<48, false>, L48, L48.total);
            if (err == cudaSuccess) err = tcc_prepare(sllg_tcc_kernel<48, true>, L48, L48.total);
        }
        if (err == cudaSuccess)
            err = nb == 32 ? tcc_prepare(tcc_dipolar_kernel<32>, Lmax, Lmax.total)
                           : tcc_prepare(tcc_dipolar_kernel<64>, Lmax, Lmax.total);
        if (err == cudaSuccess)
            err = nb == 32 ? tcc_prepare(sllg_tcc_implicit_kernel<32>, Lmax, imp)
                           : tcc_prepare(sllg_tcc_implicit_kernel<64>, Lmax, imp);
        if (err != cudaSuccess) return err;
        done[dev][w] = true;
    }
    // a cluster of this n, with the larger (implicit) footprint, must fit
    const TccLayout L = tcc_layout(n, nb);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)L.T);
    cfg.blockDim = dim3((unsigned)(nb == 32 ? Cfg<32>::THREADS
                                   : nb == 40 ? Cfg<40>::THREADS : Cfg<64>::THREADS));
    cfg.dynamicSmemBytes = tcc_imp_smem(L);
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)L.T;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int clusters = 0;
    err = nb == 32   ? cudaOccupancyMaxActiveClusters(&clusters, sllg_tcc_implicit_kernel<32>, &cfg)
          : nb == 40 ? cudaOccupancyMaxActiveClusters(&clusters, sllg_tcc_implicit_kernel<40>, &cfg)
                     : cudaOccupancyMaxActiveClusters(&clusters, sllg_tcc_implicit_kernel<64>, &cfg);
    if (err != cudaSuccess) return err;
    if (max_clusters) *max_clusters = clusters;
    return clusters > 0 ? cudaSuccess : cudaErrorNotSupported;
}

cudaError_t launch_tcc(const DevPlan &p, const __half *d, __half *b, int nb, cudaStream_t stream)
{
    if (p.E == 0) return cudaSuccess;
    const TccLayout L = tcc_layout(p.n, nb);
    const int64_t tiles = (p.E + nb - 1) / nb;
    if (p.use_implicit) {
        if (!tcc_implicit_supported(p.n) || !p.hj) return cudaErrorNotSupported;
        const size_t smem = tcc_imp_smem(L);
        if (nb == 32)
            return tcc_launch(sllg_tcc_implicit_kernel<32>, L, smem, Cfg<32>::THREADS, tiles,
                              stream, p, d, b, tiles);
        if (nb == 40)
            return tcc_launch(sllg_tcc_implicit_kernel<40>, L, smem, Cfg<40>::THREADS, tiles,
                              stream, p, d, b, tiles);
        return tcc_launch(sllg_tcc_implicit_kernel<64>, L, smem, Cfg<64>::THREADS, tiles, stream,
                          p, d, b, tiles);
    }
    if (!tcc_supported(p.n)) return cudaErrorNotSupported;
    const bool dres = tcc_acc_cols(nb) + L.K <= 512;
    if (nb == 40)
        return dres ? tcc_launch(sllg_tcc_kernel<40, true>, L, L.total, Cfg<40>::THREADS, tiles,
                                 stream, p, d, b, tiles)
                    : tcc_launch(sllg_tcc_kernel<40, false>, L, L.total, Cfg<40>::THREADS, tiles,
                                 stream, p, d, b, tiles);
    if (nb == 48)
        return dres ? tcc_launch(sllg_tcc_kernel<48, true>, L, L.total, Cfg<48>::THREADS, tiles,
                                 stream, p, d, b, tiles)
                    : tcc_launch(sllg_tcc_kernel<48, false>, L, L.total, Cfg<48>::THREADS, tiles,
                                 stream, p, d, b, tiles);
    if (nb == 32)
        return dres ? tcc_launch(sllg_tcc_kernel<32, true>, L, L.total, Cfg<32>::THREADS, tiles,
                                 stream, p, d, b, tiles)
                    : tcc_launch(sllg_tcc_kernel<32, false>, L, L.total, Cfg<32>::THREADS, tiles,
                                 stream, p, d, b, tiles);
    return dres ? tcc_launch(sllg_tcc_kernel<64, true>, L, L.total, Cfg<64>::THREADS, tiles,
                             stream, p, d, b, tiles)
                : tcc_launch(sllg_tcc_kernel<64, false>, L, L.total, Cfg<64>::THREADS, tiles,
                             stream, p, d, b, tiles);
}

cudaError_t launch_tcc_dipolar(const __half *d, __half *b, int n, int64_t E, const double *m,
                               double *h, int *flag, cudaStream_t stream)
{
    if (!tcc_implicit_supported(n)) return cudaErrorNotSupported;
    const int nb = 32;
    const TccLayout L = tcc_layout(n, nb);
    const int64_t tiles = (E + nb - 1) / nb;
    return tcc_launch(tcc_dipolar_kernel<32>, L, L.total, Cfg<32>::THREADS, tiles, stream, n, E, d,
                      b, m, h, flag);
}

}  // namespace magpy
