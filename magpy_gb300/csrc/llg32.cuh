// llg32.cuh -- the FP32 LLG stage map and the float-float state update
// shared by the tensor-core kernels (sllg_tc.cu, sllg_tcc.cu).
//
// Stage increment: the reference's drift a = -m x h - alpha m x (m x h)
// (lib/llg.cpp:14-29) and diffusion B(m) w = sr (-m x w - alpha m x (m x w))
// (lib/llg.cpp:92-106, the same form with w in place of h), so
//     dt a + sqrt(dt) B w = F(m, dt h + sqrt(dt) sr w),
//     F(m, v) = -(m x v) - alpha (m (m.v) - v |m|^2),
// one evaluation of a map that is linear in v.
#pragma once

namespace magpy {

struct DDf { float hi, lo; };

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

// ---- two items per instruction (packed FP32: fma/add/mul .rn.f32x2, sm_100+) ----
// The same operations as llg_F and dd_add_ts on a pair of items held as the
// .x and .y halves of float2 values.
__device__ inline float2 f2(float a) { return make_float2(a, a); }
__device__ inline float2 neg2(float2 a) { return make_float2(-a.x, -a.y); }
__device__ inline float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ inline float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ inline float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }

__device__ inline void llg_F2(float2 o[3], const float2 m[3], float2 alpha, const float2 v[3])
{
    const float2 c0 = fma2(m[1], v[2], neg2(mul2(m[2], v[1])));
    const float2 c1 = fma2(m[2], v[0], neg2(mul2(m[0], v[2])));
    const float2 c2 = fma2(m[0], v[1], neg2(mul2(m[1], v[0])));
    const float2 mv = fma2(m[2], v[2], fma2(m[1], v[1], mul2(m[0], v[0])));
    const float2 mm = fma2(m[2], m[2], fma2(m[1], m[1], mul2(m[0], m[0])));
    o[0] = fma2(alpha, fma2(v[0], mm, neg2(mul2(m[0], mv))), neg2(c0));
    o[1] = fma2(alpha, fma2(v[1], mm, neg2(mul2(m[1], mv))), neg2(c1));
    o[2] = fma2(alpha, fma2(v[2], mm, neg2(mul2(m[2], mv))), neg2(c2));
}

// (hi, lo) + d for two float-float items.
__device__ inline void dd_add_ts2(float2 &hi, float2 &lo, float2 d)
{
    const float2 y = add2(d, lo);
    const float2 s = add2(hi, y);
    const float2 bb = add2(s, neg2(hi));
    lo = add2(add2(hi, neg2(add2(s, neg2(bb)))), add2(y, neg2(bb)));
    hi = s;
}

}  // namespace magpy
