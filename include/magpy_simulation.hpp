/* magpy_simulation.hpp -- the reference's C++ simulation entry point over the
 * C-ABI of libmagpy_gpu.so (header-only).
 *
 * Replaces: simulation::full_dynamics, physical units (lib/simulation.cpp:476-624),
 * declared at include/simulation.hpp:74-94 with the results struct of
 * include/simulation.hpp:32-48 and the field::options enum of
 * include/field.hpp:95-97.  The signature, argument meanings, defaults and the
 * returned std::vector<simulation::results> (one per particle, max_samples
 * values each, SI units) are the reference's, so a caller written against
 * simulation.hpp -- magpy/core.pyx's `cdef extern from "simulation.hpp"` block
 * (core.pyx:72-93) -- compiles against this header unchanged but for its name.
 * The run is the FP64-faithful GPU kernel (the reference's arithmetic) with
 * increments from the library's counter-based generator keyed by `seed`.
 *
 * Errors: the reference throws std::invalid_argument for an unknown field
 * option (simulation.cpp:571); this adapter throws std::invalid_argument for
 * every argument the library rejects and std::runtime_error for a CUDA
 * failure, with the library's message.  A member status other than zero (the
 * implicit solver's Newton limit or a singular block, which the reference
 * drops silently at simulation.cpp:368-369) is not an error: it is available
 * from last_status().
 *
 * Link with -lmagpy_gpu (magpy_gb300/_lib).
 */
#ifndef MAGPY_SIMULATION_HPP
#define MAGPY_SIMULATION_HPP

#include <array>
#include <cstddef>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "magpy_gpu.h"

using d3 = std::array<double, 3>;

namespace field {
// include/field.hpp:95-97; the same codes as MAGPY_FIELD_SINE/SQUARE/CONSTANT
enum options { SINE, SQUARE, CONSTANT };
}  // namespace field

namespace simulation {

// include/simulation.hpp:32-48: one particle's trajectory, N samples.
struct results {
    std::unique_ptr<double[]> mx;
    std::unique_ptr<double[]> my;
    std::unique_ptr<double[]> mz;
    std::unique_ptr<double[]> field;
    std::unique_ptr<double[]> time;
    size_t N;

    explicit results(size_t _N)
        : mx(new double[_N]), my(new double[_N]), mz(new double[_N]), field(new double[_N]),
          time(new double[_N]), N(_N)
    {
    }
};

// MAGPY_STATUS_* bits of the last full_dynamics call in this thread.
inline int32_t &last_status()
{
    static thread_local int32_t s = 0;
    return s;
}

inline std::vector<results> full_dynamics(
    const std::vector<double> radius,
    const std::vector<double> anisotropy,
    const std::vector<d3> anisotropy_axes,
    const std::vector<d3> magnetisation_direction,
    const std::vector<d3> location,
    const double magnetisation,
    const double damping,
    const double temperature,
    const bool renorm,
    const bool interactions,
    const bool use_implicit,
    const double eps,
    const double time_step,
    const double end_time,
    const size_t max_samples,
    const long seed,
    const field::options field_option = field::CONSTANT,
    const double field_amplitude = 0.0,
    const double field_frequency = 0.0)
{
    const size_t n = radius.size();
    if (anisotropy.size() != n || anisotropy_axes.size() != n ||
        magnetisation_direction.size() != n || location.size() != n)
        throw std::invalid_argument("per-particle inputs differ in length");
    if (field_option != field::SINE && field_option != field::SQUARE &&
        field_option != field::CONSTANT)
        throw std::invalid_argument("Unknown field option");
    const size_t S = max_samples;
    // d3 is three contiguous doubles: the vectors are the [n][3] arrays the
    // C-ABI takes
    static_assert(sizeof(d3) == 3 * sizeof(double), "d3 must be three packed doubles");
    std::vector<double> mx(n * S), my(n * S), mz(n * S), fld(S), tim(S);
    int32_t status = 0;
    const int rc = magpy_full_dynamics(
        (int64_t)n, radius.data(), anisotropy.data(), (const double *)anisotropy_axes.data(),
        (const double *)magnetisation_direction.data(), (const double *)location.data(),
        magnetisation, damping, temperature, renorm ? 1 : 0, interactions ? 1 : 0,
        use_implicit ? 1 : 0, eps, time_step, end_time, (int64_t)max_samples, (int64_t)seed,
        (int32_t)field_option, field_amplitude, field_frequency, nullptr, 0,
        MAGPY_PRECISION_FP64, mx.data(), my.data(), mz.data(), fld.data(), tim.data(), &status);
    if (rc == MAGPY_ERR_INVALID_ARGUMENT || rc == MAGPY_ERR_NOISE_TOO_SHORT ||
        rc == MAGPY_ERR_UNSUPPORTED)
        throw std::invalid_argument(magpy_last_error_string());
    if (rc != MAGPY_SUCCESS) throw std::runtime_error(magpy_last_error_string());
    last_status() = status;
    std::vector<results> out;
    out.reserve(n);
    for (size_t i = 0; i < n; i++) {
        results r(S);
        for (size_t s = 0; s < S; s++) {
            r.mx[s] = mx[i * S + s];
            r.my[s] = my[i * S + s];
            r.mz[s] = mz[i * S + s];
            r.field[s] = fld[s];
            r.time[s] = tim[s];
        }
        out.push_back(std::move(r));
    }
    return out;
}

}  // namespace simulation

#endif
