// llg64.cuh -- FP64 LLG arithmetic for the faithful kernel.
//
// Every expression keeps the association of the reference's C++ (lib/llg.cpp,
// lib/field.cpp) and the translation unit that includes this header is
// compiled with -fmad=false, so each product and sum rounds separately as in
// the reference's x86-64 build: the FP64 kernel reproduces the reference's
// trajectories bit for bit when both consume the same increments.
#pragma once
#include <cmath>
#include <cstdint>

namespace magpy {
namespace f64 {

// llg::drift, lib/llg.cpp:14-29
__host__ __device__ inline void drift(double d[3], const double m[3], double alpha,
                                      const double h[3])
{
    d[0] = m[2] * h[1] - m[1] * h[2]
        + alpha * (h[0] * (m[1] * m[1] + m[2] * m[2]) - m[0] * (m[1] * h[1] + m[2] * h[2]));
    d[1] = m[0] * h[2] - m[2] * h[0]
        + alpha * (h[1] * (m[0] * m[0] + m[2] * m[2]) - m[1] * (m[0] * h[0] + m[2] * h[2]));
    d[2] = m[1] * h[0] - m[0] * h[1]
        + alpha * (h[2] * (m[0] * m[0] + m[1] * m[1]) - m[2] * (m[0] * h[0] + m[1] * h[1]));
}

// llg::diffusion, lib/llg.cpp:92-106 (row-major 3x3)
__host__ __device__ inline void diffusion(double b[9], const double m[3], double sr,
                                          double alpha)
{
    b[0] = alpha * sr * (m[1] * m[1] + m[2] * m[2]);
    b[1] = sr * (m[2] - alpha * m[0] * m[1]);
    b[2] = -sr * (m[1] + alpha * m[0] * m[2]);
    b[3] = -sr * (m[2] + alpha * m[0] * m[1]);
    b[4] = alpha * sr * (m[0] * m[0] + m[2] * m[2]);
    b[5] = sr * (m[0] - alpha * m[1] * m[2]);
    b[6] = sr * (m[1] - alpha * m[0] * m[2]);
    b[7] = -sr * (m[0] + alpha * m[1] * m[2]);
    b[8] = alpha * sr * (m[0] * m[0] + m[1] * m[1]);
}

// llg::drift_jacobian, lib/llg.cpp:68-81
// (templated: the implicit solve of the mixed-precision mode evaluates the
// Jacobians and the 3x3 solve in FP32; T = double is the reference's arithmetic)
template <class T>
__host__ __device__ inline void drift_jacobian(T j[9], const T m[3], T a, const T h[3],
                                               const T hj[9])
{
    j[0] =  m[2]*hj[3] - m[1]*hj[6] + a*( -m[1]*h[1] - m[2]*h[2] + ( m[1]*m[1] + m[2]*m[2] )*hj[0] - m[0]*( m[1]*hj[3] + m[2]*hj[6] ) );
    j[1] = -h[2] + m[2]*hj[4] - m[1]*hj[7] + a*( 2*m[1]*h[0] + ( m[1]*m[1] + m[2]*m[2] )*hj[1] - m[0]*( h[1] + m[1]*hj[4] + m[2]*hj[7] ) );
    j[2] =  h[1] + m[2]*hj[5] - m[1]*hj[8] + a*( 2*m[2]*h[0] + ( m[1]*m[1] + m[2]*m[2] )*hj[2] - m[0]*( h[2] + m[1]*hj[5] + m[2]*hj[8] ) );
    j[3] =  h[2] - m[2]*hj[0] + m[0]*hj[6] + a*( 2*m[0]*h[1] + ( m[0]*m[0] + m[2]*m[2] )*hj[3] - m[1]*( h[0] + m[0]*hj[0] + m[2]*hj[6] ) );
    j[4] = -m[2]*hj[1] + m[0]*hj[7] + a*( -m[0]*h[0] - m[2]*h[2] + ( m[0]*m[0] + m[2]*m[2] )*hj[4] - m[1]*( m[0]*hj[1] + m[2]*hj[7] ) );
    j[5] = -h[0] - m[2]*hj[2] + m[0]*hj[8] + a*( 2*m[2]*h[1] + ( m[0]*m[0] + m[2]*m[2] )*hj[5] - m[1]*( h[2] + m[0]*hj[2] + m[2]*hj[8] ) );
    j[6] = -h[1] + m[1]*hj[0] - m[0]*hj[3] + a*( 2*m[0]*h[2] + ( m[0]*m[0] + m[1]*m[1] )*hj[6] - m[2]*( h[0] + m[0]*hj[0] + m[1]*hj[3] ) );
    j[7] =  h[0] + m[1]*hj[1] - m[0]*hj[4] + a*( 2*m[1]*h[2] + ( m[0]*m[0] + m[1]*m[1] )*hj[7] - m[2]*( h[1] + m[0]*hj[1] + m[1]*hj[4] ) );
    j[8] =  m[1]*hj[2] - m[0]*hj[5] + a*( -m[0]*h[0] - m[1]*h[1] + ( m[0]*m[0] + m[1]*m[1] )*hj[8] - m[2]*( m[0]*hj[2] + m[1]*hj[5] ) );
}

// llg::diffusion_jacobian, lib/llg.cpp:118-158, index 9*row + 3*wiener + deriv.
// Entries [4] and [25] are as the reference writes them (m[2] in place of
// the analytic m[0] and m[1]); they only steer the Newton iteration.
template <class T>
__host__ __device__ inline void diffusion_jacobian(T j[27], const T m[3], T sr, T alpha)
{
    j[0] = 0;
    j[1] = 2 * alpha * sr * m[1];
    j[2] = 2 * alpha * sr * m[2];
    j[3] = -alpha * sr * m[1];
    j[4] = -alpha * sr * m[2];
    j[5] = sr;
    j[6] = -alpha * sr * m[2];
    j[7] = -sr;
    j[8] = -alpha * sr * m[0];
    j[9] = -alpha * sr * m[1];
    j[10] = -alpha * sr * m[0];
    j[11] = -sr;
    j[12] = 2 * alpha * sr * m[0];
    j[13] = 0;
    j[14] = 2 * alpha * sr * m[2];
    j[15] = sr;
    j[16] = -alpha * sr * m[2];
    j[17] = -alpha * sr * m[1];
    j[18] = -alpha * sr * m[2];
    j[19] = sr;
    j[20] = -alpha * sr * m[0];
    j[21] = -sr;
    j[22] = -alpha * sr * m[2];
    j[23] = -alpha * sr * m[1];
    j[24] = 2 * alpha * sr * m[0];
    j[25] = 2 * alpha * sr * m[2];
    j[26] = 0;
}

// field::uniaxial_anisotropy, lib/field.cpp:97-105
__host__ __device__ inline void uniaxial(double h[3], const double m[3], const double ax[3])
{
    double dot = m[0] * ax[0] + m[1] * ax[1] + m[2] * ax[2];
    h[0] = dot * ax[0];
    h[1] = dot * ax[1];
    h[2] = dot * ax[2];
}

// Applied-field waveforms, lib/field.cpp:23-54
__host__ __device__ inline double field_value(int shape, double t, double h, double f)
{
    if (shape == 2) return h;
    if (shape == 0) return h * sin(2 * M_PI * f * t);
    return h * (int(t * f * 2) % 2 ? -1 : 1);
}

// Applied field of Heun step k (1-based) at t = k dt (second = 0) or at
// t + dt (second = 1) -- the times of the two stages, lib/integrators.cpp:386,
// :394 with t = step dt, lib/simulation.cpp:355 -- rounded to FP32.  The
// mixed-precision kernels take it from here, from a per-step table or
// computed in the kernel, so every form gets the same values.
__host__ __device__ inline float heun_field_f32(int shape, double dt, double h, double f,
                                                int64_t k, int second)
{
    const double t = (double)k * dt;
    return (float)field_value(shape, second ? t + dt : t, h, f);
}

// 3x3 solve with the arithmetic of the project BLAS/LAPACK shim's dgesv
// (partial pivoting, first maximal |a| wins; division multipliers; forward
// then column-oriented back substitution).  Returns 0 or the 1-based index
// of the first exactly-zero pivot, in which case b is left unchanged.
template <class T>
__host__ __device__ inline int solve3(T a[9], T b[3])
{
    int piv[3];
    int info = 0;
    for (int k = 0; k < 3; k++) {
        int p = k;
        T vmax = fabs(a[k * 3 + k]);
        for (int i = k + 1; i < 3; i++) {
            T v = fabs(a[i * 3 + k]);
            if (v > vmax) { vmax = v; p = i; }
        }
        piv[k] = p;
        if (a[p * 3 + k] != T(0)) {
            if (p != k)
                for (int c = 0; c < 3; c++) {
                    T tmp = a[k * 3 + c];
                    a[k * 3 + c] = a[p * 3 + c];
                    a[p * 3 + c] = tmp;
                }
            T pivot = a[k * 3 + k];
            for (int i = k + 1; i < 3; i++) {
                T l = a[i * 3 + k] / pivot;
                a[i * 3 + k] = l;
                for (int c = k + 1; c < 3; c++) a[i * 3 + c] = a[i * 3 + c] - l * a[k * 3 + c];
            }
        } else if (info == 0) {
            info = k + 1;
        }
    }
    if (info != 0) return info;
    for (int k = 0; k < 3; k++)
        if (piv[k] != k) {
            T tmp = b[k];
            b[k] = b[piv[k]];
            b[piv[k]] = tmp;
        }
    for (int k = 0; k < 3; k++)
        for (int i = k + 1; i < 3; i++) b[i] = b[i] - b[k] * a[i * 3 + k];
    for (int k = 2; k >= 0; k--) {
        b[k] = b[k] / a[k * 3 + k];
        for (int i = 0; i < k; i++) b[i] = b[i] - b[k] * a[i * 3 + k];
    }
    return 0;
}

}  // namespace f64
}  // namespace magpy
