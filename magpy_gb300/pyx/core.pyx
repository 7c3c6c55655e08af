# distutils: language = c++
# cython: language_level=3
"""magpy.core.simulate on the GPU library.

The reference's Cython entry (magpy/core.pyx:128-203) with its Python
signature and result dictionary kept, calling simulation::full_dynamics
declared as the reference declares it (include/simulation.hpp:74-94), here
from include/magpy_simulation.hpp: the reference's C++ entry point over the
C-ABI of libmagpy_gpu.so.  Differences from the shipped binding: C++
exceptions become Python exceptions (``except +``; the reference's extern
block lets them terminate the process), the GIL is released during the run,
and the result arrays are copied in one pass per component instead of
element by element.

Built by magpy_gb300/pyx/build_pyx.py (Cython and a C++ compiler; the GPU
library itself comes from magpy_gb300/build.py).
"""
import numpy as np

cimport numpy as cnp
from libcpp cimport bool as cbool
from libcpp.vector cimport vector

cnp.import_array()


cdef extern from "magpy_simulation.hpp":
    cdef cppclass d3:
        double &operator[](size_t)


cdef extern from "<memory>" namespace "std":
    cdef cppclass darray "std::unique_ptr<double[]>":
        double &operator[](size_t)


cdef extern from "magpy_simulation.hpp" namespace "field":
    cdef enum options:
        SINE
        SQUARE
        CONSTANT


cdef extern from "magpy_simulation.hpp" namespace "simulation":
    cdef cppclass results:
        darray mx
        darray my
        darray mz
        darray field
        darray time
        size_t N

    vector[results] full_dynamics(
        const vector[double] radius,
        const vector[double] anisotropy,
        const vector[d3] anisotropy_axes,
        const vector[d3] magnetisation_direction,
        const vector[d3] location,
        const double magnetisation,
        const double damping,
        const double temperature,
        const cbool renorm,
        const cbool interactions,
        const cbool use_implicit,
        const double eps,
        const double time_step,
        const double end_time,
        const size_t max_samples,
        const long seed,
        const options field_option,
        const double field_amplitude,
        const double field_frequency) except + nogil


cdef vector[double] _vec(double[::1] a):
    cdef vector[double] v
    cdef Py_ssize_t i
    v.resize(a.shape[0])
    for i in range(a.shape[0]):
        v[i] = a[i]
    return v


cdef vector[d3] _vec3(double[:, ::1] a):
    cdef vector[d3] v
    cdef Py_ssize_t i
    cdef int c
    if a.shape[1] != 3:
        raise ValueError("expected an [N][3] array")
    v.resize(a.shape[0])
    for i in range(a.shape[0]):
        for c in range(3):
            v[i][c] = a[i, c]
    return v


cdef cnp.ndarray _copy(double *p, Py_ssize_t n):
    return np.asarray(<double[:n]> p).copy()


_FIELD_CODES = {'constant': CONSTANT, 'sine': SINE, 'square': SQUARE}


cpdef simulate(
        cnp.ndarray[double, ndim=1, mode='c'] radius,
        cnp.ndarray[double, ndim=1, mode='c'] anisotropy,
        cnp.ndarray[double, ndim=2, mode='c'] anisotropy_axis,
        cnp.ndarray[double, ndim=2, mode='c'] magnetisation_direction,
        cnp.ndarray[double, ndim=2, mode='c'] location,
        double magnetisation,
        double damping,
        double temperature,
        cbool renorm,
        cbool interactions,
        cbool use_implicit,
        double time_step,
        double end_time,
        int max_samples,
        int seed,
        str field_shape='constant',
        double field_amplitude=0.0,
        double field_frequency=0.0,
        double implicit_tol=1e-9):
    """One cluster: the dictionary {'N', 'time', 'field', 'x', 'y', 'z'} of
    magpy/core.pyx:186-202, x/y/z mapping each particle to its samples (A/m)."""
    cdef options code = _FIELD_CODES[field_shape]  # KeyError as the reference's lookup
    if max_samples < 1:
        raise ValueError("max_samples must be >= 1")
    cdef vector[double] c_radius = _vec(radius)
    cdef vector[double] c_anisotropy = _vec(anisotropy)
    cdef vector[d3] c_axis = _vec3(anisotropy_axis)
    cdef vector[d3] c_m0 = _vec3(magnetisation_direction)
    cdef vector[d3] c_loc = _vec3(location)
    cdef vector[results] res
    cdef size_t S = <size_t> max_samples
    cdef long c_seed = seed
    with nogil:
        res = full_dynamics(c_radius, c_anisotropy, c_axis, c_m0, c_loc, magnetisation, damping,
                            temperature, renorm, interactions, use_implicit, implicit_tol,
                            time_step, end_time, S, c_seed, code, field_amplitude,
                            field_frequency)
    n = radius.shape[0]
    return {
        'N': n,
        'time': _copy(&res[0].time[0], max_samples),
        'field': _copy(&res[0].field[0], max_samples),
        'x': {i: _copy(&res[i].mx[0], max_samples) for i in range(n)},
        'y': {i: _copy(&res[i].my[0], max_samples) for i in range(n)},
        'z': {i: _copy(&res[i].mz[0], max_samples) for i in range(n)},
    }
