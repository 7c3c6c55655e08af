"""ctypes binding of libmagpy_gpu.so (include/magpy_gpu.h).

The library is the product: there is no CPU fallback.  Loading fails with an
ImportError when the shared library is missing and cannot be built.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build as _build

SUCCESS = 0
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "noise too short", -4: "unsupported",
          -5: "out of memory", -6: "I/O error"}
STATUS_NEWTON_MAXITER = 1
STATUS_SINGULAR = 2
STATUS_NONFINITE = 4
STATUS_NOISE_EXHAUSTED = 8
STATUS_WATCHDOG = 16
STATUS_STEP_LIMIT = 32
NOALLOC_SCRATCH_BYTES = 32 * 1024 * 1024
FIELD_SHAPES = {"sine": 0, "square": 1, "constant": 2}
DOM_FIELD_SHAPES = {"sine": 0, "square": 1, "constant": 2, "square_f": 3}
PRECISIONS = {"fp64": 0, "mixed": 1, "mixed_tc": 2}

_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)


class EnsembleDesc(C.Structure):
    _fields_ = [
        ("n_members", C.c_int64), ("n_particles", C.c_int64),
        ("per_member_geometry", C.c_int32),
        ("radius", C.c_void_p), ("anisotropy", C.c_void_p), ("anisotropy_axis", C.c_void_p),
        ("magnetisation_direction", C.c_void_p), ("location", C.c_void_p),
        ("magnetisation", C.c_double), ("damping", C.c_double), ("temperature", C.c_double),
        ("field_amplitude", C.c_double), ("field_frequency", C.c_double),
        ("field_shape", C.c_int32),
        ("magnetisation_per_member", C.c_void_p), ("damping_per_member", C.c_void_p),
        ("temperature_per_member", C.c_void_p), ("field_amplitude_per_member", C.c_void_p),
        ("field_frequency_per_member", C.c_void_p),
        ("renorm", C.c_int32), ("interactions", C.c_int32), ("use_implicit", C.c_int32),
        ("eps", C.c_double), ("max_iter", C.c_int64), ("time_step", C.c_double),
        ("end_time", C.c_double), ("max_samples", C.c_int64), ("seeds", C.c_void_p),
        ("noise", C.c_void_p), ("noise_per_member", C.c_int64), ("precision", C.c_int32),
        ("buffers_on_device", C.c_int32),
    ]


class EnsembleOut(C.Structure):
    _fields_ = [("mx", C.c_void_p), ("my", C.c_void_p), ("mz", C.c_void_p),
                ("time", C.c_void_p), ("field", C.c_void_p), ("status", C.c_void_p),
                ("steps", C.c_void_p)]


class DomDesc(C.Structure):
    """magpy_dom_desc of include/magpy_gpu.h."""
    _fields_ = [("n_particles", C.c_int64), ("volume", C.c_void_p), ("anisotropy", C.c_void_p),
                ("temperature", C.c_void_p), ("magnetisation", C.c_void_p),
                ("damping", C.c_void_p), ("initial_probabilities", C.c_void_p),
                ("field_amplitude", C.c_void_p), ("field_frequency", C.c_void_p),
                ("field_shape", C.c_int32), ("field_n_components", C.c_int64),
                ("time_step", C.c_double), ("end_time", C.c_double),
                ("max_samples", C.c_int64), ("max_steps", C.c_int64)]


class GeoDesc(C.Structure):
    """magpy_geometry_desc of include/magpy_gpu.h."""
    _fields_ = [("n_members", C.c_int64), ("n_particles", C.c_int64), ("layout", C.c_int32),
                ("moments", C.c_int32), ("median_radius", C.c_double),
                ("sigma_log_radius", C.c_double), ("spacing", C.c_double),
                ("packing_fraction", C.c_double), ("max_rounds", C.c_int64),
                ("seeds", C.c_void_p), ("buffers_on_device", C.c_int32)]


SYMBOLS = [
    "magpy_ensemble_dynamics", "magpy_full_dynamics", "magpy_full_dynamics_reduced",
    "magpy_llg_components", "magpy_wiener_increments", "magpy_step_count",
    "magpy_last_error_string", "magpy_version", "magpy_plan_create", "magpy_plan_run",
    "magpy_plan_device_outputs", "magpy_plan_copy_out", "magpy_plan_shape", "magpy_plan_destroy",
    "magpy_ensemble_dynamics_noalloc", "magpy_dipolar_field_tc",
    "magpy_plan_ensemble_magnetisation", "magpy_plan_energy_dissipated",
    "magpy_batch_create", "magpy_batch_run", "magpy_batch_group_plan", "magpy_batch_group_choice",
    "magpy_batch_destroy", "magpy_plan_set_launch", "magpy_adjoint_create",
    "magpy_adjoint_forward", "magpy_adjoint_plan", "magpy_adjoint_backward",
    "magpy_adjoint_destroy", "magpy_save_results", "magpy_plan_save_results",
    "magpy_dom_dynamics", "magpy_generate_clusters", "magpy_plan_set_wait_limit",
]

_LIB = None


def lib() -> C.CDLL:
    """Load (building first if needed) and return the CUDA library."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path):
        try:
            path = _build.build()
        except Exception as exc:  # no toolkit: fail loudly, never fall back
            raise ImportError(f"libmagpy_gpu.so is not built and cannot be built: {exc}")
    L = C.CDLL(path)
    L.magpy_ensemble_dynamics.restype = C.c_int
    L.magpy_ensemble_dynamics.argtypes = [C.POINTER(EnsembleDesc), C.POINTER(EnsembleOut),
                                          C.c_void_p]
    L.magpy_full_dynamics.restype = C.c_int
    L.magpy_full_dynamics.argtypes = (
        [C.c_int64] + [_dp] * 5 + [C.c_double] * 3 + [C.c_int32] * 3 + [C.c_double] * 3 +
        [C.c_int64, C.c_int64, C.c_int32, C.c_double, C.c_double, _dp, C.c_int64, C.c_int32] +
        [_dp] * 5 + [_i32p])
    L.magpy_full_dynamics_reduced.restype = C.c_int
    L.magpy_full_dynamics_reduced.argtypes = (
        [C.c_int64] + [_dp] * 7 + [C.c_int32] + [C.c_double] * 8 + [_dp, C.c_int64] +
        [C.c_int32] * 3 + [C.c_double, C.c_int64, C.c_int64, C.c_int32] + [_dp] * 5 +
        [_i32p, _i64p])
    L.magpy_llg_components.restype = C.c_int
    L.magpy_llg_components.argtypes = [C.c_int64] + [_dp] * 11
    L.magpy_wiener_increments.restype = C.c_int
    L.magpy_wiener_increments.argtypes = [C.c_int64, C.c_int64, C.c_int64, _dp]
    L.magpy_step_count.restype = C.c_int
    L.magpy_step_count.argtypes = [C.c_double, C.c_double, C.c_int64, _i64p]
    L.magpy_plan_create.restype = C.c_int
    L.magpy_plan_create.argtypes = [C.POINTER(EnsembleDesc), C.POINTER(C.c_void_p), C.c_void_p]
    L.magpy_plan_run.restype = C.c_int
    L.magpy_plan_run.argtypes = [C.c_void_p, C.c_void_p]
    L.magpy_plan_device_outputs.restype = C.c_int
    L.magpy_plan_device_outputs.argtypes = [C.c_void_p] + [C.POINTER(C.c_void_p)] * 5
    L.magpy_plan_copy_out.restype = C.c_int
    L.magpy_plan_copy_out.argtypes = [C.c_void_p, C.POINTER(EnsembleOut), C.c_void_p]
    L.magpy_plan_shape.restype = C.c_int
    L.magpy_plan_shape.argtypes = [C.c_void_p] + [_i64p] * 4
    L.magpy_plan_destroy.restype = C.c_int
    L.magpy_plan_destroy.argtypes = [C.c_void_p]
    L.magpy_ensemble_dynamics_noalloc.restype = C.c_int
    L.magpy_ensemble_dynamics_noalloc.argtypes = [C.POINTER(EnsembleDesc),
                                                  C.POINTER(EnsembleOut), C.c_void_p]
    L.magpy_dipolar_field_tc.restype = C.c_int
    L.magpy_dipolar_field_tc.argtypes = [C.c_int64, C.c_int64, C.c_double, C.c_double] + [_dp] * 5
    L.magpy_plan_ensemble_magnetisation.restype = C.c_int
    L.magpy_plan_ensemble_magnetisation.argtypes = [C.c_void_p, C.c_int32, _dp, C.c_void_p]
    L.magpy_plan_energy_dissipated.restype = C.c_int
    L.magpy_plan_energy_dissipated.argtypes = [C.c_void_p, C.c_double, C.c_double, _dp,
                                               C.c_void_p]
    L.magpy_batch_create.restype = C.c_int
    L.magpy_batch_create.argtypes = [C.POINTER(EnsembleDesc), C.c_int64, C.c_int32,
                                     C.POINTER(C.c_void_p), C.c_void_p]
    L.magpy_batch_run.restype = C.c_int
    L.magpy_batch_run.argtypes = [C.c_void_p, C.c_void_p]
    L.magpy_batch_group_plan.restype = C.c_int
    L.magpy_batch_group_plan.argtypes = [C.c_void_p, C.c_int64, C.POINTER(C.c_void_p)]
    L.magpy_batch_group_choice.restype = C.c_int
    L.magpy_batch_group_choice.argtypes = [C.c_void_p, C.c_int64, _i32p, _i32p, _i32p,
                                           C.POINTER(C.c_double)]
    L.magpy_plan_set_launch.restype = C.c_int
    L.magpy_plan_set_launch.argtypes = [C.c_void_p, C.c_int32, C.c_int32]
    L.magpy_plan_set_wait_limit.restype = C.c_int
    L.magpy_plan_set_wait_limit.argtypes = [C.c_void_p, C.c_int64]
    L.magpy_batch_destroy.restype = C.c_int
    L.magpy_batch_destroy.argtypes = [C.c_void_p]
    L.magpy_adjoint_create.restype = C.c_int
    L.magpy_adjoint_create.argtypes = [C.POINTER(EnsembleDesc), C.c_int64,
                                       C.POINTER(C.c_void_p), C.c_void_p]
    L.magpy_adjoint_forward.restype = C.c_int
    L.magpy_adjoint_forward.argtypes = [C.c_void_p, C.c_void_p]
    L.magpy_adjoint_plan.restype = C.c_int
    L.magpy_adjoint_plan.argtypes = [C.c_void_p, C.POINTER(C.c_void_p)]
    L.magpy_adjoint_backward.restype = C.c_int
    L.magpy_adjoint_backward.argtypes = [C.c_void_p, _dp, _dp, _dp, C.c_void_p]
    L.magpy_adjoint_destroy.restype = C.c_int
    L.magpy_adjoint_destroy.argtypes = [C.c_void_p]
    L.magpy_dom_dynamics.restype = C.c_int
    L.magpy_dom_dynamics.argtypes = [C.POINTER(DomDesc), _dp, _dp, _dp, _i32p, _i64p,
                                     C.c_void_p]
    L.magpy_generate_clusters.restype = C.c_int
    L.magpy_generate_clusters.argtypes = [C.POINTER(GeoDesc), C.c_void_p, C.c_void_p,
                                          C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
    L.magpy_save_results.restype = C.c_int
    L.magpy_save_results.argtypes = [C.c_char_p] + [_dp] * 5 + [C.c_int64]
    L.magpy_plan_save_results.restype = C.c_int
    L.magpy_plan_save_results.argtypes = [C.c_void_p, C.c_char_p, C.c_int64, C.c_int64,
                                          C.c_void_p]
    L.magpy_last_error_string.restype = C.c_char_p
    L.magpy_version.restype = C.c_char_p
    _LIB = L
    return L


class MagpyError(RuntimeError):
    pass


def check(rc: int) -> None:
    if rc != SUCCESS:
        msg = lib().magpy_last_error_string().decode()
        raise MagpyError(f"{ERRORS.get(rc, rc)}: {msg}")


def dptr(a: np.ndarray | None):
    return None if a is None else a.ctypes.data_as(_dp)


def vptr(a) -> int | None:
    """Address of a numpy array or a torch tensor (device or host)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    return a.data_ptr()  # torch.Tensor


def f64(x, size=None) -> np.ndarray:
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    if size is not None and a.size != size:
        raise ValueError(f"expected {size} values, got {a.size}")
    return a
