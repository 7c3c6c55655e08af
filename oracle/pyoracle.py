"""ctypes bindings for the CPU checkers.  TEST INFRASTRUCTURE ONLY.

* ``Oracle``     -- oracle/_build/liboracle.so, the FP64 CPU restatement of
                    magpy's sLLG path (oracle/sllg_oracle.cpp).
* ``Reference``  -- oracle/_ref/libmagpy_ref.so, the reference's own lib/*.cpp
                    behind oracle/ref_harness.cpp (only where the reference
                    checkout was present when it was built).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline legs of bench.py
import this module.  The product (magpy_gb300) never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libmagpy_ref.so")

FIELD_SHAPES = {"sine": 0, "square": 1, "constant": 2}
DOM_FIELD_SHAPES = {"sine": 0, "square": 1, "constant": 2, "square_f": 3}

_dp = C.POINTER(C.c_double)
_i64p = C.POINTER(C.c_int64)
_i32p = C.POINTER(C.c_int32)


def _d(a):
    return a.ctypes.data_as(_dp) if a is not None else None


def build(ref: bool = False) -> None:
    """Compile the oracle (and, when asked and possible, the reference)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def reference_available() -> bool:
    return os.path.exists(REF_SO)


class _Reduced(C.Structure):
    _fields_ = [
        ("n", C.c_int64), ("sr", _dp), ("k_red", _dp), ("v_red", _dp), ("axes", _dp),
        ("m0", _dp), ("unit_dist", _dp), ("dist_mag", _dp), ("field_shape", C.c_int32),
        ("happ", C.c_double), ("fapp", C.c_double), ("k_av", C.c_double),
        ("v_av", C.c_double), ("alpha", C.c_double), ("ms", C.c_double), ("dt", C.c_double),
        ("end_time", C.c_double), ("renorm", C.c_int32), ("interactions", C.c_int32),
        ("use_implicit", C.c_int32), ("eps", C.c_double), ("max_iter", C.c_int64),
        ("max_samples", C.c_int64),
    ]


SDE_CB = C.CFUNCTYPE(None, _dp, _dp, _dp, C.c_double, C.c_void_p)
SDE_JAC_CB = C.CFUNCTYPE(None, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_double, C.c_void_p)
FJ_CB = C.CFUNCTYPE(None, _dp, _dp, _dp, C.c_void_p)


def _f64(x, n=None):
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float64))
    if n is not None:
        assert a.size == n, (a.size, n)
    return a


def reduced_inputs(rng: np.random.Generator, n: int, *, interactions=True, spacing=2.2):
    """Seeded reduced-unit inputs for a random cluster (parity cases)."""
    axes = rng.normal(size=(n, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    m0 = rng.normal(size=(n, 3))
    m0 /= np.linalg.norm(m0, axis=1, keepdims=True)
    # particles on a jittered cubic lattice, reduced distance >= ~spacing
    side = int(np.ceil(n ** (1 / 3)))
    grid = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    pts = grid * spacing + rng.uniform(-0.1, 0.1, size=(n, 3))
    vec = pts[None, :, :] - pts[:, None, :]
    mag = np.sqrt((vec ** 2).sum(-1))
    with np.errstate(invalid="ignore", divide="ignore"):
        unit = vec / mag[..., None]
    return dict(
        n=n, sr=rng.uniform(0.05, 0.3, n), k_red=rng.uniform(0.8, 1.2, n),
        v_red=rng.uniform(0.7, 1.3, n), axes=axes, m0=m0, unit_dist=unit, dist_mag=mag,
    )


class Oracle:
    """FP64 CPU restatement (oracle/sllg_oracle.cpp)."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build()
        self.lib = L = C.CDLL(path)
        L.oracle_full_dynamics_reduced.restype = C.c_int
        L.oracle_full_dynamics_reduced.argtypes = [
            C.POINTER(_Reduced), _dp, C.c_int64, C.c_uint64, _dp, _dp, _dp, _dp, _dp, _i64p]
        L.oracle_full_dynamics.restype = C.c_int
        L.oracle_full_dynamics.argtypes = [
            C.c_int64, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_double, C.c_double,
            C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double, C.c_int64,
            C.c_int64, C.c_int32, C.c_double, C.c_double, C.c_int64, _dp, C.c_int64,
            _dp, _dp, _dp, _dp, _dp, _i64p]
        L.oracle_ensemble.restype = C.c_int
        L.oracle_ensemble.argtypes = [
            C.c_int64, C.c_int64, _dp, _dp, _dp, _dp, _dp, C.c_double, C.c_double,
            C.c_double, C.c_int32, C.c_int32, C.c_int32, C.c_double, C.c_double, C.c_double,
            C.c_int64, _i64p, C.c_int32, C.c_double, C.c_double, C.c_int64, _dp, C.c_int64,
            C.c_int32, _dp, _dp, _dp, _dp, _dp, _i32p]
        L.oracle_reduce_parameters.restype = None
        L.oracle_reduce_parameters.argtypes = [
            C.c_int64, _dp, _dp, _dp, C.c_double, C.c_double, C.c_double, C.c_double,
            C.c_double, C.c_double, C.c_double, _dp, _dp, _dp, _dp, _dp, _dp]
        for name, nargs in [("oracle_llg_drift", None), ("oracle_llg_diffusion", None)]:
            pass
        L.oracle_llg_drift.argtypes = [_dp, _dp, C.c_double, _dp]
        L.oracle_llg_diffusion.argtypes = [_dp, _dp, C.c_double, C.c_double]
        L.oracle_llg_drift_jacobian.argtypes = [_dp, _dp, C.c_double, _dp, _dp]
        L.oracle_llg_diffusion_jacobian.argtypes = [_dp, _dp, C.c_double, C.c_double]
        L.oracle_uniaxial_anisotropy.argtypes = [_dp, _dp, _dp]
        L.oracle_uniaxial_anisotropy_jacobian.argtypes = [_dp, _dp]
        L.oracle_multi_add_uniaxial_anisotropy_jacobian.argtypes = [_dp, _dp, _dp, C.c_int64]
        L.oracle_dipolar_prefactor.restype = C.c_double
        L.oracle_dipolar_prefactor.argtypes = [C.c_double, C.c_double]
        L.oracle_dipolar_p2p.argtypes = [_dp, C.c_double, C.c_double, _dp, _dp, C.c_double]
        L.oracle_multi_add_dipolar.argtypes = [_dp, C.c_double, C.c_double, _dp, _dp, _dp, _dp,
                                               C.c_int64]
        L.oracle_pairwise_geometry.argtypes = [_dp, C.c_int64, _dp, _dp, _dp]
        L.oracle_field_value.restype = C.c_double
        L.oracle_field_value.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double]
        L.oracle_nrm2.restype = C.c_double
        L.oracle_nrm2.argtypes = [_dp, C.c_int64]
        L.oracle_dgesv.restype = C.c_int64
        L.oracle_dgesv.argtypes = [C.c_int64, _dp, _dp]
        L.oracle_heun_dense.argtypes = [_dp, _dp, _dp, SDE_CB, C.c_void_p, C.c_int64,
                                        C.c_int64, C.c_double, C.c_double]
        L.oracle_heun_driver.argtypes = [_dp, _dp, _dp, SDE_CB, C.c_void_p, C.c_int64,
                                         C.c_int64, C.c_int64, C.c_double]
        L.oracle_newton_noinv.restype = C.c_int
        L.oracle_newton_noinv.argtypes = [_dp, FJ_CB, C.c_void_p, _dp, C.c_int64, C.c_double,
                                          C.c_int64, _i64p]
        L.oracle_implicit_midpoint_dense.restype = C.c_int
        L.oracle_implicit_midpoint_dense.argtypes = [
            _dp, _dp, _dp, SDE_JAC_CB, C.c_void_p, C.c_int64, C.c_int64, C.c_double,
            C.c_double, C.c_double, C.c_int64]
        L.oracle_implicit_driver.argtypes = [
            _dp, _dp, _dp, SDE_JAC_CB, C.c_void_p, C.c_int64, C.c_int64, C.c_int64,
            C.c_double, C.c_double, C.c_double, C.c_int64, _i32p]
        L.oracle_mt_norm.argtypes = [C.c_uint64, C.c_double, C.c_int64, _dp]
        L.oracle_dom_transition_matrix.argtypes = [_dp] + [C.c_double] * 6
        L.oracle_max_threads.restype = C.c_int
        L.oracle_dom_field.restype = C.c_double
        L.oracle_dom_field.argtypes = [C.c_int, C.c_double, C.c_double, C.c_double, C.c_int64]
        L.oracle_master_equation.argtypes = [_dp, _dp, _dp, C.c_int64]
        L.oracle_rk45_tests_ode.restype = C.c_int
        L.oracle_rk45_tests_ode.argtypes = [_dp, _dp, _dp, _dp, _dp, C.c_double]
        L.oracle_dom_dynamics.restype = C.c_int
        L.oracle_dom_dynamics.argtypes = (
            [C.c_double] * 5 + [C.c_int32, C.c_double, C.c_double, C.c_int64, _dp, C.c_double,
                                C.c_double, C.c_int64, C.c_int64, C.c_int64, _dp, _dp, _dp,
                                _i64p])
        L.oracle_dom_batch.restype = C.c_int
        L.oracle_dom_batch.argtypes = (
            [C.c_int64] + [_dp] * 6 + [C.c_int32, _dp, _dp, C.c_int64, C.c_double, C.c_double,
                                       C.c_int64, C.c_int64, C.c_int64, C.c_int32, _dp, _dp,
                                       _dp, _i32p, _i64p])
        L.oracle_const_kb.restype = C.c_double
        L.oracle_const_mu0.restype = C.c_double
        L.oracle_const_gyromag.restype = C.c_double

    # ---- simulation ----
    def full_dynamics_reduced(self, inp: dict, *, field_shape="constant", happ=0.0, fapp=0.0,
                              k_av=2e4, v_av=1.0, alpha=0.1, ms=4e5, dt=1e-3, end_time=0.1,
                              renorm=False, interactions=True, use_implicit=False, eps=1e-9,
                              max_iter=1000, max_samples=11, noise=None, seed=1001):
        n = inp["n"]
        arrs = {k: _f64(inp[k]) for k in ("sr", "k_red", "v_red", "axes", "m0", "unit_dist",
                                          "dist_mag")}
        p = _Reduced(n, _d(arrs["sr"]), _d(arrs["k_red"]), _d(arrs["v_red"]), _d(arrs["axes"]),
                     _d(arrs["m0"]), _d(arrs["unit_dist"]), _d(arrs["dist_mag"]),
                     FIELD_SHAPES[field_shape], happ, fapp, k_av, v_av, alpha, ms, dt,
                     end_time, int(renorm), int(interactions), int(use_implicit), eps,
                     max_iter, max_samples)
        S = max_samples
        mx, my, mz = (np.zeros((n, S)) for _ in range(3))
        field, time = np.zeros(S), np.zeros(S)
        steps = C.c_int64(0)
        nz = _f64(noise) if noise is not None else None
        st = self.lib.oracle_full_dynamics_reduced(
            C.byref(p), _d(nz), 0 if nz is None else nz.size, seed, _d(mx), _d(my), _d(mz),
            _d(field), _d(time), C.byref(steps))
        return dict(x=mx, y=my, z=mz, field=field, time=time, status=st, steps=steps.value)

    def full_dynamics(self, radius, anisotropy, axes, m0, location, ms, damping, temperature,
                      *, renorm=False, interactions=True, use_implicit=False, eps=1e-9,
                      time_step=1e-13, end_time=1e-11, max_samples=11, seed=1001,
                      field_shape="constant", field_amplitude=0.0, field_frequency=0.0,
                      max_iter=1000, noise=None):
        radius = _f64(radius)
        n = radius.size
        S = max_samples
        mx, my, mz = (np.zeros((n, S)) for _ in range(3))
        field, time = np.zeros(S), np.zeros(S)
        steps = C.c_int64(0)
        nz = _f64(noise) if noise is not None else None
        st = self.lib.oracle_full_dynamics(
            n, _d(radius), _d(_f64(anisotropy, n)), _d(_f64(axes, 3 * n)), _d(_f64(m0, 3 * n)),
            _d(_f64(location, 3 * n)), ms, damping, temperature, int(renorm),
            int(interactions), int(use_implicit), eps, time_step, end_time, S, seed,
            FIELD_SHAPES[field_shape], field_amplitude, field_frequency, max_iter, _d(nz),
            0 if nz is None else nz.size, _d(mx), _d(my), _d(mz), _d(field), _d(time),
            C.byref(steps))
        return dict(x=mx, y=my, z=mz, field=field, time=time, status=st, steps=steps.value)

    def ensemble(self, seeds, radius, anisotropy, axes, m0, location, ms, damping, temperature,
                 *, renorm=False, interactions=True, use_implicit=False, eps=1e-9,
                 time_step=1e-13, end_time=1e-11, max_samples=11, field_shape="constant",
                 field_amplitude=0.0, field_frequency=0.0, max_iter=1000, noise=None,
                 n_threads=0):
        seeds = np.ascontiguousarray(seeds, dtype=np.int64)
        E = seeds.size
        radius = _f64(radius)
        n = radius.size
        S = max_samples
        mx, my, mz = (np.zeros((E, n, S)) for _ in range(3))
        field, time = np.zeros(S), np.zeros(S)
        status = np.zeros(E, dtype=np.int32)
        nz = _f64(noise) if noise is not None else None
        per = 0 if nz is None else nz.size // E
        self.lib.oracle_ensemble(
            E, n, _d(radius), _d(_f64(anisotropy, n)), _d(_f64(axes, 3 * n)),
            _d(_f64(m0, 3 * n)), _d(_f64(location, 3 * n)), ms, damping, temperature,
            int(renorm), int(interactions), int(use_implicit), eps, time_step, end_time, S,
            seeds.ctypes.data_as(_i64p), FIELD_SHAPES[field_shape], field_amplitude,
            field_frequency, max_iter, _d(nz), per, n_threads, _d(mx), _d(my), _d(mz),
            _d(field), _d(time), status.ctypes.data_as(_i32p))
        return dict(x=mx, y=my, z=mz, field=field, time=time, status=status)

    def reduce_parameters(self, radius, anisotropy, location, ms, damping, temperature,
                          time_step, end_time, field_amplitude=0.0, field_frequency=0.0):
        radius = _f64(radius)
        n = radius.size
        sr, k_red, v_red = np.zeros(n), np.zeros(n), np.zeros(n)
        unit, mag, sc = np.zeros((n, n, 3)), np.zeros((n, n)), np.zeros(8)
        self.lib.oracle_reduce_parameters(
            n, _d(radius), _d(_f64(anisotropy, n)), _d(_f64(location, 3 * n)), ms, damping,
            temperature, time_step, end_time, field_amplitude, field_frequency, _d(sr),
            _d(k_red), _d(v_red), _d(unit), _d(mag), _d(sc))
        keys = ["k_av", "v_av", "H_k", "time_factor", "dt", "end_time", "happ", "fapp"]
        out = dict(zip(keys, sc.tolist()))
        out.update(n=n, sr=sr, k_red=k_red, v_red=v_red, unit_dist=unit, dist_mag=mag)
        return out

    # ---- components ----
    def drift(self, m, alpha, h):
        d = np.zeros(3)
        self.lib.oracle_llg_drift(_d(d), _d(_f64(m)), alpha, _d(_f64(h)))
        return d

    def diffusion(self, m, sr, alpha):
        b = np.zeros(9)
        self.lib.oracle_llg_diffusion(_d(b), _d(_f64(m)), sr, alpha)
        return b

    def drift_jacobian(self, m, alpha, h, hj):
        j = np.zeros(9)
        self.lib.oracle_llg_drift_jacobian(_d(j), _d(_f64(m)), alpha, _d(_f64(h)), _d(_f64(hj)))
        return j

    def diffusion_jacobian(self, m, sr, alpha):
        j = np.zeros(27)
        self.lib.oracle_llg_diffusion_jacobian(_d(j), _d(_f64(m)), sr, alpha)
        return j

    def multi_add_dipolar(self, field, ms, k_av, v_red, mag, dists, dist_cubes):
        field = _f64(field).copy()
        n = field.size // 3
        self.lib.oracle_multi_add_dipolar(_d(field), ms, k_av, _d(_f64(v_red)), _d(_f64(mag)),
                                          _d(_f64(dists)), _d(_f64(dist_cubes)), n)
        return field

    def mt_norm(self, seed, std, count):
        out = np.zeros(count)
        self.lib.oracle_mt_norm(seed, std, count, _d(out))
        return out

    def nrm2(self, x):
        x = _f64(x)
        return self.lib.oracle_nrm2(_d(x), x.size)

    def dgesv(self, a, b):
        a = _f64(a).copy()
        b = _f64(b).copy()
        info = self.lib.oracle_dgesv(b.size, _d(a), _d(b))
        return info, b

    def transition_matrix(self, k, v, T, h, ms, alpha):
        W = np.zeros(4)
        self.lib.oracle_dom_transition_matrix(_d(W), k, v, T, h, ms, alpha)
        return W

    # ---- two-state master equation (DOModel) ----
    def dom_field(self, shape, t, h, f, n_components=1):
        return self.lib.oracle_dom_field(DOM_FIELD_SHAPES[shape], t, h, f, n_components)

    def master_equation(self, W, x):
        x = _f64(x)
        y = np.zeros_like(x)
        self.lib.oracle_master_equation(_d(y), _d(_f64(W)), _d(x), x.size)
        return y

    def rk45_tests_ode(self, x1, h, t, tol):
        x2, k = np.zeros(2), np.zeros(12)
        hh, tt = np.array([h], dtype=np.float64), np.array([t], dtype=np.float64)
        self.lib.oracle_rk45_tests_ode(_d(x2), _d(k), _d(hh), _d(tt), _d(_f64(x1)), tol)
        return x2, k.reshape(6, 2), hh[0], tt[0]

    def dom_dynamics(self, volume, anisotropy, temperature, ms, alpha, shape, h_red, f, ncomp,
                     p0, time_step, end_time, max_samples, max_steps=1 << 40,
                     max_attempts=4096):
        N = int(end_time / time_step) + 1 if max_samples == -1 else max_samples
        mz, field, time = np.zeros(N), np.zeros(N), np.zeros(N)
        steps = C.c_int64(0)
        st = self.lib.oracle_dom_dynamics(volume, anisotropy, temperature, ms, alpha,
                                          DOM_FIELD_SHAPES[shape], h_red, f, ncomp,
                                          _d(_f64(p0)), time_step, end_time, max_samples,
                                          max_steps, max_attempts, _d(mz), _d(field), _d(time),
                                          C.byref(steps))
        return dict(mz=mz, field=field, time=time, status=st, steps=steps.value)

    def dom_batch(self, volume, anisotropy, temperature, ms, alpha, p0, shape, amplitude,
                  frequency, ncomp, time_step, end_time, max_samples, max_steps=1 << 40,
                  max_attempts=4096, n_threads=0):
        volume = _f64(volume)
        E = volume.size
        per = [_f64(np.broadcast_to(np.asarray(a, dtype=np.float64), (E,)))
               for a in (anisotropy, temperature, ms, alpha, amplitude, frequency)]
        p0 = _f64(np.broadcast_to(np.asarray(p0, dtype=np.float64), (E, 2)))
        N = int(end_time / time_step) + 1 if max_samples == -1 else max_samples
        mz, field, time = (np.zeros((E, N)) for _ in range(3))
        status, steps = np.zeros(E, dtype=np.int32), np.zeros(E, dtype=np.int64)
        self.lib.oracle_dom_batch(E, _d(volume), _d(per[0]), _d(per[1]), _d(per[2]), _d(per[3]),
                                  _d(p0), DOM_FIELD_SHAPES[shape], _d(per[4]), _d(per[5]), ncomp,
                                  time_step, end_time, max_samples, max_steps, max_attempts,
                                  n_threads, _d(mz), _d(field), _d(time),
                                  status.ctypes.data_as(_i32p), steps.ctypes.data_as(_i64p))
        return dict(mz=mz, field=field, time=time, status=status, steps=steps)


class Reference:
    """The reference's own lib/*.cpp behind oracle/ref_harness.cpp."""

    def __init__(self, path: str = REF_SO):
        self.lib = L = C.CDLL(path)
        L.ref_full_dynamics_reduced.restype = C.c_int
        L.ref_full_dynamics_reduced.argtypes = (
            [C.c_int64] + [_dp] * 7 + [C.c_int32] + [C.c_double] * 8 + [C.c_int32] * 3 +
            [C.c_double, C.c_int64, _dp, C.c_int64] + [_dp] * 5)
        L.ref_full_dynamics.restype = C.c_int
        L.ref_full_dynamics.argtypes = (
            [C.c_int64] + [_dp] * 5 + [C.c_double] * 3 + [C.c_int32] * 3 + [C.c_double] * 3 +
            [C.c_int64, C.c_int64, C.c_int32, C.c_double, C.c_double] + [_dp] * 5)
        L.ref_ensemble.restype = C.c_int
        L.ref_ensemble.argtypes = (
            [C.c_int64, C.c_int64] + [_dp] * 5 + [C.c_double] * 3 + [C.c_int32] * 3 +
            [C.c_double] * 3 + [C.c_int64, _i64p, C.c_int32, C.c_double, C.c_double,
                                C.c_int32] + [_dp] * 3)
        L.ref_llg_drift.argtypes = [_dp, _dp, C.c_double, _dp]
        L.ref_llg_diffusion.argtypes = [_dp, _dp, C.c_double, C.c_double]
        L.ref_llg_drift_jacobian.argtypes = [_dp, _dp, C.c_double, _dp, _dp]
        L.ref_llg_diffusion_jacobian.argtypes = [_dp, _dp, C.c_double, C.c_double]
        L.ref_multi_add_dipolar.argtypes = [_dp, C.c_double, C.c_double, _dp, _dp, _dp, _dp,
                                            C.c_int64]
        L.ref_mt_norm.argtypes = [C.c_uint64, C.c_double, C.c_int64, _dp]
        L.ref_dom_transition_matrix.argtypes = [_dp] + [C.c_double] * 6
        L.ref_save_results.argtypes = [C.c_char_p] + [_dp] * 5 + [C.c_int64]
        L.ref_dom_dynamics.restype = C.c_int
        L.ref_dom_dynamics.argtypes = (
            [C.c_double] * 5 + [C.c_int32, C.c_double, C.c_double, C.c_int64, _dp, C.c_double,
                                C.c_double, C.c_int64, _dp, _dp, _dp])
        L.ref_rk45_tests_ode.argtypes = [_dp, _dp, _dp, _dp, _dp, C.c_double]

    def full_dynamics_reduced(self, inp: dict, *, field_shape="constant", happ=0.0, fapp=0.0,
                              k_av=2e4, v_av=1.0, alpha=0.1, ms=4e5, dt=1e-3, end_time=0.1,
                              renorm=False, interactions=True, use_implicit=False, eps=1e-9,
                              max_samples=11, noise=None):
        n = inp["n"]
        a = {k: _f64(inp[k]) for k in ("sr", "k_red", "v_red", "axes", "m0", "unit_dist",
                                       "dist_mag")}
        S = max_samples
        mx, my, mz = (np.zeros((n, S)) for _ in range(3))
        field, time = np.zeros(S), np.zeros(S)
        nz = _f64(noise)
        st = self.lib.ref_full_dynamics_reduced(
            n, _d(a["sr"]), _d(a["k_red"]), _d(a["v_red"]), _d(a["axes"]), _d(a["m0"]),
            _d(a["unit_dist"]), _d(a["dist_mag"]), FIELD_SHAPES[field_shape], happ, fapp,
            k_av, v_av, alpha, ms, dt, end_time, int(renorm), int(interactions),
            int(use_implicit), eps, S, _d(nz), nz.size, _d(mx), _d(my), _d(mz), _d(field),
            _d(time))
        return dict(x=mx, y=my, z=mz, field=field, time=time, status=st)

    def full_dynamics(self, radius, anisotropy, axes, m0, location, ms, damping, temperature,
                      *, renorm=False, interactions=True, use_implicit=False, eps=1e-9,
                      time_step=1e-13, end_time=1e-11, max_samples=11, seed=1001,
                      field_shape="constant", field_amplitude=0.0, field_frequency=0.0):
        radius = _f64(radius)
        n = radius.size
        S = max_samples
        mx, my, mz = (np.zeros((n, S)) for _ in range(3))
        field, time = np.zeros(S), np.zeros(S)
        self.lib.ref_full_dynamics(
            n, _d(radius), _d(_f64(anisotropy, n)), _d(_f64(axes, 3 * n)), _d(_f64(m0, 3 * n)),
            _d(_f64(location, 3 * n)), ms, damping, temperature, int(renorm),
            int(interactions), int(use_implicit), eps, time_step, end_time, S, seed,
            FIELD_SHAPES[field_shape], field_amplitude, field_frequency, _d(mx), _d(my),
            _d(mz), _d(field), _d(time))
        return dict(x=mx, y=my, z=mz, field=field, time=time)

    def ensemble(self, seeds, radius, anisotropy, axes, m0, location, ms, damping, temperature,
                 *, renorm=False, interactions=True, use_implicit=False, eps=1e-9,
                 time_step=1e-13, end_time=1e-11, max_samples=11, field_shape="constant",
                 field_amplitude=0.0, field_frequency=0.0, n_threads=0, keep=True):
        seeds = np.ascontiguousarray(seeds, dtype=np.int64)
        E = seeds.size
        radius = _f64(radius)
        n = radius.size
        S = max_samples
        if keep:
            mx, my, mz = (np.zeros((E, n, S)) for _ in range(3))
        else:
            mx = my = mz = None
        self.lib.ref_ensemble(
            E, n, _d(radius), _d(_f64(anisotropy, n)), _d(_f64(axes, 3 * n)),
            _d(_f64(m0, 3 * n)), _d(_f64(location, 3 * n)), ms, damping, temperature,
            int(renorm), int(interactions), int(use_implicit), eps, time_step, end_time, S,
            seeds.ctypes.data_as(_i64p), FIELD_SHAPES[field_shape], field_amplitude,
            field_frequency, n_threads, _d(mx), _d(my), _d(mz))
        return dict(x=mx, y=my, z=mz)

    def drift(self, m, alpha, h):
        d = np.zeros(3)
        self.lib.ref_llg_drift(_d(d), _d(_f64(m)), alpha, _d(_f64(h)))
        return d

    def diffusion(self, m, sr, alpha):
        b = np.zeros(9)
        self.lib.ref_llg_diffusion(_d(b), _d(_f64(m)), sr, alpha)
        return b

    def drift_jacobian(self, m, alpha, h, hj):
        j = np.zeros(9)
        self.lib.ref_llg_drift_jacobian(_d(j), _d(_f64(m)), alpha, _d(_f64(h)), _d(_f64(hj)))
        return j

    def diffusion_jacobian(self, m, sr, alpha):
        j = np.zeros(27)
        self.lib.ref_llg_diffusion_jacobian(_d(j), _d(_f64(m)), sr, alpha)
        return j

    def multi_add_dipolar(self, field, ms, k_av, v_red, mag, dists, dist_cubes):
        field = _f64(field).copy()
        n = field.size // 3
        self.lib.ref_multi_add_dipolar(_d(field), ms, k_av, _d(_f64(v_red)), _d(_f64(mag)),
                                       _d(_f64(dists)), _d(_f64(dist_cubes)), n)
        return field

    def mt_norm(self, seed, std, count):
        out = np.zeros(count)
        self.lib.ref_mt_norm(seed, std, count, _d(out))
        return out

    def transition_matrix(self, k, v, T, h, ms, alpha):
        W = np.zeros(4)
        self.lib.ref_dom_transition_matrix(_d(W), k, v, T, h, ms, alpha)
        return W

    def dom_dynamics(self, volume, anisotropy, temperature, ms, alpha, shape, h_red, f, ncomp,
                     p0, time_step, end_time, max_samples):
        """simulation::dom_ensemble_dynamics (lib/simulation.cpp:659-767)."""
        N = int(end_time / time_step) + 1 if max_samples == -1 else max_samples
        mz, field, time = np.zeros(N), np.zeros(N), np.zeros(N)
        rc = self.lib.ref_dom_dynamics(volume, anisotropy, temperature, ms, alpha,
                                       DOM_FIELD_SHAPES[shape], h_red, f, ncomp, _d(_f64(p0)),
                                       time_step, end_time, max_samples, _d(mz), _d(field),
                                       _d(time))
        assert rc == 0
        return dict(mz=mz, field=field, time=time)

    def rk45_tests_ode(self, x1, h, t, tol):
        x2, k = np.zeros(2), np.zeros(12)
        hh, tt = np.array([h], dtype=np.float64), np.array([t], dtype=np.float64)
        self.lib.ref_rk45_tests_ode(_d(x2), _d(k), _d(hh), _d(tt), _d(_f64(x1)), tol)
        return x2, k.reshape(6, 2), hh[0], tt[0]

    def save_results(self, prefix, mx, my, mz, field, time):
        """simulation::save_results (lib/simulation.cpp:38-63)."""
        arrs = [_f64(a) for a in (mx, my, mz, field, time)]
        self.lib.ref_save_results(str(prefix).encode(), *[_d(a) for a in arrs], arrs[0].size)
