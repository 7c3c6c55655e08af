// common.cuh -- device-side data layout and helpers shared by the sLLG kernels.
//
// Data layout in HBM (all arrays device-resident, struct-of-arrays so that
// consecutive threads touch consecutive addresses):
//   particles, global index g over all members (member-major):
//     m0[3][P], axes[3][P], k_red[P], sr[P], hj_eff[9][P]
//   clusters (one per distinct geometry; members may share one):
//     pt[j][q]   = dipolar pair factor  pref * v_j / r_qj^3   (N x N, column-major)
//     rt[c][j][q] = unit vector r_qj component c               (3 x N x N)
//   members: MemberDev[E]; sample step table sched[S]
//   outputs: mx/my/mz[S][P] (sample-major), status[E], steps[E]
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace magpy {

// Per-member status bits (same meaning as the oracle's).
enum : int32_t {
    ST_OK = 0,
    ST_NEWTON_MAXITER = 1,
    ST_SINGULAR = 2,
    ST_NONFINITE = 4,
    ST_NOISE_EXHAUSTED = 8,
};

enum : int32_t { FIELD_SINE = 0, FIELD_SQUARE = 1, FIELD_CONSTANT = 2 };

struct MemberDev {
    double dt;         // reduced time step
    double sqrt_dt;    // sqrt(dt), correctly rounded on host and device alike
    double alpha;      // damping
    double happ, fapp; // reduced field amplitude and frequency
    double Ah;         // implicit-midpoint increment truncation sqrt(2000 |ln dt|)
    double eps;        // Newton relative tolerance
    int64_t max_iter;  // Newton iteration limit
    int64_t pbase;     // first global particle index of the member
    int64_t noise_off; // first injected increment of the member
    int64_t noise_len; // injected increments available to the member
    uint64_t seed;     // counter-based generator key
    int64_t sched_off; // offset of the member's sample-step table
    int64_t cluster_off; // offset of the member's pair tables (elements)
    int32_t n;         // particles in the member
    int32_t shape;     // field waveform
    int32_t renorm;
    int32_t interactions;
};

// ---------------------------------------------------------------------------
// Counter-based generator: Philox-4x32 with 10 rounds (Salmon, Moraes, Dror,
// Shaw, "Parallel random numbers: as easy as 1, 2, 3", SC'11).  A 128-bit
// counter and 64-bit key give four independent 32-bit words.
// ---------------------------------------------------------------------------
struct U4 { uint32_t x, y, z, w; };

__host__ __device__ inline U4 philox4x32_10(U4 c, uint32_t k0, uint32_t k1)
{
    const uint32_t M0 = 0xD2511F53u, M1 = 0xCD9E8D57u;
    const uint32_t W0 = 0x9E3779B9u, W1 = 0xBB67AE85u;
#pragma unroll
    for (int r = 0; r < 10; r++) {
        // one 32 x 32 -> 64-bit product gives both halves
        const uint64_t p0 = (uint64_t)M0 * c.x, p1 = (uint64_t)M1 * c.z;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        U4 n{hi1 ^ c.y ^ k0, lo1, hi0 ^ c.w ^ k1, lo0};
        c = n;
        k0 += W0;
        k1 += W1;
    }
    return c;
}

// Counter of the increments of particle q at step k (1-based) of a member:
// (k low word, k high word, q, 0x5d11 stream tag); key = member seed.
// Four words -> two Box-Muller pairs (radius sqrt(-2 ln u), angle uniform on
// (-pi, pi)) -> normals (n0, n1, n2, n3); the three Wiener increments of the
// particle are n0, n1, n2.
struct Normals4 { float a, b, c, d; };

__device__ inline float u24_open(uint32_t x)
{
    // uniform on (0, 1) from the top 24 bits, never 0 or 1
    return (float)(x >> 8) * 5.9604644775390625e-8f + 2.98023223876953125e-8f;
}

// -2 ln u for u = u24_open(x).  Near u = 1, where the small radii come from
// and an absolute error in the log would be a large relative error of the
// radius, the series -ln(1 - v) = v + v^2/2 + ... + v^5/5 with v = 1 - u < 1/32
// (exact subtraction; truncation below 1e-8 relative); elsewhere the hardware
// base-2 logarithm, whose absolute error (~1e-7) is there a relative error
// below 5e-6 of -2 ln u >= 0.063.
__device__ inline float neg2_log_u24(uint32_t x)
{
    const float u = u24_open(x);
    const float v = 1.0f - u;
    float l2;
    asm("lg2.approx.f32 %0, %1;" : "=f"(l2) : "f"(u));
    // explicit fused multiply-adds: the same rounding in every translation
    // unit (the FP64-faithful unit is compiled without contraction)
    float p = __fmaf_rn(v, 0.2f, 0.25f);
    p = __fmaf_rn(v, p, 0.333333333f);
    p = __fmaf_rn(v, p, 0.5f);
    p = __fmaf_rn(v, p, 1.0f);
    return v < 0.03125f ? 2.0f * (v * p) : -1.38629436f * l2;  // -2 ln 2 log2 u
}

__device__ inline Normals4 wiener_normals(uint64_t seed, uint64_t step, uint32_t q)
{
    U4 c{(uint32_t)step, (uint32_t)(step >> 32), q, 0x5d11u};
    U4 r = philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
    // radius: -2 ln u accurate near u = 1, hardware square root (relative
    // error ~2^-22, far below anything the increments need)
    const float t0 = neg2_log_u24(r.x), t1 = neg2_log_u24(r.z);
    float r0, r1;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r0) : "f"(t0));
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r1) : "f"(t1));
    // angle uniform on (-pi, pi): the hardware sine/cosine is accurate to
    // ~2^-21 absolute on that range
    const float twopi = 6.2831853071795864769f, pi = 3.14159265358979323846f;
    float s0, c0, s1, c1;
    // explicit fused multiply-add: the same rounding in every translation unit
    // (the FP64-faithful unit is compiled without contraction)
    __sincosf(__fmaf_rn(twopi, u24_open(r.y), -pi), &s0, &c0);
    __sincosf(__fmaf_rn(twopi, u24_open(r.w), -pi), &s1, &c1);
    return Normals4{r0 * c0, r0 * s0, r1 * c1, r1 * s1};
}

// Member-level barrier: a warp subset when members are packed into warps,
// the whole CTA when one member spans several warps.
struct MemberSync {
    unsigned mask;
    bool cta;
    __device__ inline void sync() const
    {
        if (cta) __syncthreads();
        else __syncwarp(mask);
    }
};

}  // namespace magpy
