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

}  // namespace magpy
