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
#ifdef __CUDA_ARCH__
#pragma unroll
#endif
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

// Wiener increments of a member at step k (1-based): the particles are taken
// in pairs (2p, 2p + 1), and one Philox call on the counter (k low word,
// k high word, p, 0x5d12 stream tag), keyed by the member seed, gives the six
// normals of a pair.  Its 128 bits make six uniforms -- four of 21 bits (the
// top of each word) and two of 22 bits (the low 11 bits of words 0 and 1, and
// of words 2 and 3) -- that feed three Box-Muller pairs (radius
// sqrt(-2 ln u), angle uniform on (-pi, pi)):
//   pair A (top of words 0, 1)  -> components 0, 1 of particle 2p,
//   pair B (top of words 2, 3)  -> components 0, 1 of particle 2p + 1,
//   pair C (the two low parts)  -> component 2 of 2p (cosine), of 2p + 1 (sine).
// A uniform of b bits is (x + 1/2) 2^-b, never 0 or 1, so the radius never
// exceeds 5.52 (21 bits) or 5.65 (22 bits): tails beyond are cut (3e-8 and
// 2e-8 per normal).
struct Normals4 { float a, b, c, d; };   // one particle: components a, b, c
struct PairNormals { float n[6]; };      // particle 2p: n[0..2], 2p + 1: n[3..5]

__device__ inline float u21_open(uint32_t w) { return (float)(w >> 11) * 4.76837158203125e-7f + 2.384185791015625e-7f; }
__device__ inline float u22_open(uint32_t x22) { return (float)x22 * 2.384185791015625e-7f + 1.1920928955078125e-7f; }
__device__ inline uint32_t low22(uint32_t w_hi, uint32_t w_lo) { return ((w_hi & 0x7ffu) << 11) | (w_lo & 0x7ffu); }

// -2 ln u for u in (0, 1).  Near u = 1, where the small radii come from and
// an absolute error in the log would be a large relative error of the radius,
// the series -ln(1 - v) = v + v^2/2 + ... + v^5/5 with v = 1 - u < 1/32
// (exact subtraction; truncation below 1e-8 relative); elsewhere the hardware
// base-2 logarithm, whose absolute error (~1e-7) is there a relative error
// below 5e-6 of -2 ln u >= 0.063.
__device__ inline float neg2_log(float u)
{
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

// Box-Muller: (r cos t, r sin t) for radius uniform ur and angle uniform ut.
// Hardware square root (relative error ~2^-22) and sine/cosine (~2^-21
// absolute on (-pi, pi)); the angle's fused multiply-add is explicit for the
// same rounding in every translation unit.
__device__ inline void box_muller(float ur, float ut, float &x, float &y)
{
    const float twopi = 6.2831853071795864769f, pi = 3.14159265358979323846f;
    float r, s, c;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(neg2_log(ur)));
    __sincosf(__fmaf_rn(twopi, ut, -pi), &s, &c);
    x = r * c;
    y = r * s;
}

__device__ inline U4 wiener_words(uint64_t seed, uint64_t step, uint32_t p)
{
    const U4 c{(uint32_t)step, (uint32_t)(step >> 32), p, 0x5d12u};
    return philox4x32_10(c, (uint32_t)seed, (uint32_t)(seed >> 32));
}

// The six normals of particles 2p and 2p + 1.
__device__ inline PairNormals wiener_pair(uint64_t seed, uint64_t step, uint32_t p)
{
    const U4 r = wiener_words(seed, step, p);
    PairNormals o;
    box_muller(u21_open(r.x), u21_open(r.y), o.n[0], o.n[1]);
    box_muller(u21_open(r.z), u21_open(r.w), o.n[3], o.n[4]);
    box_muller(u22_open(low22(r.x, r.y)), u22_open(low22(r.z, r.w)), o.n[2], o.n[5]);
    return o;
}

// The three normals of particle q alone (the same numbers as wiener_pair).
__device__ inline Normals4 wiener_normals(uint64_t seed, uint64_t step, uint32_t q)
{
    const U4 r = wiener_words(seed, step, q >> 1);
    const bool odd = (q & 1u) != 0;
    Normals4 o;
    box_muller(u21_open(odd ? r.z : r.x), u21_open(odd ? r.w : r.y), o.a, o.b);
    float c0, c1;
    box_muller(u22_open(low22(r.x, r.y)), u22_open(low22(r.z, r.w)), c0, c1);
    o.c = odd ? c1 : c0;
    o.d = 0.f;
    return o;
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
