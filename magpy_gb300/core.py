"""The GPU core: counterpart of magpy.core (magpy/core.pyx).

``simulate`` keeps the signature and the returned dictionary of
``magpy.core.simulate`` (magpy/core.pyx:128-203); ``simulate_ensemble`` runs
all members of an ensemble in one launch (the reference calls ``simulate``
once per member from joblib workers, magpy/model.py:204-207).
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, dptr, f64, vptr

# include/constants.hpp:10-12
KB = 1.38064852e-23
MU0 = 1.25663706e-6
GYROMAG = 1.76086e11


def get_KB():
    return KB


def get_mu0():
    return MU0


def get_gamma():
    return GYROMAG


def _shape_code(field_shape: str) -> int:
    # magpy/core.pyx:158-161 raises KeyError for unknown shapes
    return _lib.FIELD_SHAPES[field_shape]


def simulate(radius, anisotropy, anisotropy_axis, magnetisation_direction, location,
             magnetisation, damping, temperature, renorm, interactions, use_implicit, time_step,
             end_time, max_samples, seed, field_shape="constant", field_amplitude=0.0,
             field_frequency=0.0, implicit_tol=1e-9, *, precision="fp64", noise=None):
    """One cluster on the GPU; same arguments and result as magpy.core.simulate.

    Returns ``{'N', 'time', 'field', 'x', 'y', 'z'}`` with x/y/z dictionaries
    particle -> array of ``max_samples`` values (A/m).  ``noise`` optionally
    injects the Wiener increments (``[steps][3N]``); by default they come from
    the in-kernel counter-based generator keyed by ``seed``.
    """
    radius = f64(radius)
    n = radius.size
    S = int(max_samples)
    mx, my, mz = (np.empty((n, S)) for _ in range(3))
    field, time = np.empty(S), np.empty(S)
    status = C.c_int32(0)
    nz = f64(noise) if noise is not None else None
    rc = _lib.lib().magpy_full_dynamics(
        n, dptr(radius), dptr(f64(anisotropy, n)), dptr(f64(anisotropy_axis, 3 * n)),
        dptr(f64(magnetisation_direction, 3 * n)), dptr(f64(location, 3 * n)),
        float(magnetisation), float(damping), float(temperature), int(bool(renorm)),
        int(bool(interactions)), int(bool(use_implicit)), float(implicit_tol), float(time_step),
        float(end_time), S, int(seed), _shape_code(field_shape), float(field_amplitude),
        float(field_frequency), dptr(nz), 0 if nz is None else nz.size,
        _lib.PRECISIONS[precision], dptr(mx), dptr(my), dptr(mz), dptr(field), dptr(time),
        C.byref(status))
    check(rc)
    return {
        "N": n,
        "time": time,
        "field": field,
        "x": {i: mx[i] for i in range(n)},
        "y": {i: my[i] for i in range(n)},
        "z": {i: mz[i] for i in range(n)},
        "status": int(status.value),
    }


def simulate_reduced(n, thermal_field_strengths, reduced_anisotropy_constants,
                     reduced_particle_volumes, anisotropy_unit_axes, initial_magnetisations,
                     interparticle_unit_distances, interparticle_reduced_distance_magnitudes,
                     field_shape, reduced_field_amplitude, reduced_field_frequency,
                     average_anisotropy, average_volume, damping_constant,
                     saturation_magnetisation, time_step, end_time, noise, renorm,
                     interactions, use_implicit, eps, max_samples, *, max_iter=1000,
                     precision="fp64"):
    """Reduced-unit run with injected increments: simulation::full_dynamics
    (lib/simulation.cpp:132-429) driven by an RngArray (lib/rng.cpp:67-94)."""
    S = int(max_samples)
    mx, my, mz = (np.empty((n, S)) for _ in range(3))
    field, time = np.empty(S), np.empty(S)
    status, steps = C.c_int32(0), C.c_int64(0)
    nz = f64(noise)
    rc = _lib.lib().magpy_full_dynamics_reduced(
        n, dptr(f64(thermal_field_strengths, n)), dptr(f64(reduced_anisotropy_constants, n)),
        dptr(f64(reduced_particle_volumes, n)), dptr(f64(anisotropy_unit_axes, 3 * n)),
        dptr(f64(initial_magnetisations, 3 * n)), dptr(f64(interparticle_unit_distances, 3 * n * n)),
        dptr(f64(interparticle_reduced_distance_magnitudes, n * n)), _shape_code(field_shape),
        float(reduced_field_amplitude), float(reduced_field_frequency), float(average_anisotropy),
        float(average_volume), float(damping_constant), float(saturation_magnetisation),
        float(time_step), float(end_time), dptr(nz), nz.size, int(bool(renorm)),
        int(bool(interactions)), int(bool(use_implicit)), float(eps), int(max_iter), S,
        _lib.PRECISIONS[precision], dptr(mx), dptr(my), dptr(mz), dptr(field), dptr(time),
        C.byref(status), C.byref(steps))
    check(rc)
    return dict(x=mx, y=my, z=mz, field=field, time=time, status=int(status.value),
                steps=int(steps.value))


class EnsembleArrays:
    """Dense results of one batched run.

    ``mx, my, mz``: [S][E*N] sample-major (A/m); ``time, field``: [E][S];
    ``status``: [E] status bits; ``steps``: [E] integration steps.
    """

    def __init__(self, n_members, n_particles, mx, my, mz, time, field, status, steps):
        self.n_members = n_members
        self.n_particles = n_particles
        self.mx, self.my, self.mz = mx, my, mz
        self.time, self.field = time, field
        self.status, self.steps = status, steps

    def member(self, e: int) -> dict:
        """The reference's per-member result dict (magpy/core.pyx:186-202)."""
        n = self.n_particles
        sl = slice(e * n, (e + 1) * n)
        return {
            "N": n, "time": self.time[e], "field": self.field[e],
            "x": {i: self.mx[:, sl][:, i] for i in range(n)},
            "y": {i: self.my[:, sl][:, i] for i in range(n)},
            "z": {i: self.mz[:, sl][:, i] for i in range(n)},
        }


def _ensemble_desc(n_members, radius, anisotropy, anisotropy_axis, magnetisation_direction,
                   location, magnetisation, damping, temperature, renorm, interactions,
                   use_implicit, time_step, end_time, max_samples, seeds, field_shape,
                   field_amplitude, field_frequency, implicit_tol, per_member_geometry,
                   per_member, precision, noise, max_iter):
    """Builds the C descriptor; returns (desc, keep-alive dict, n)."""
    E = int(n_members)
    radius = f64(radius)
    rows = radius.size
    n = rows // E if per_member_geometry else rows
    seeds = np.ascontiguousarray(seeds, dtype=np.int64)
    if seeds.size != E:
        raise ValueError("need one seed per member")
    keep = {"seeds": seeds}
    d = _lib.EnsembleDesc()
    d.n_members, d.n_particles = E, n
    d.per_member_geometry = int(bool(per_member_geometry))
    for name, arr in (("radius", radius), ("anisotropy", f64(anisotropy, rows)),
                      ("anisotropy_axis", f64(anisotropy_axis, 3 * rows)),
                      ("magnetisation_direction", f64(magnetisation_direction, 3 * rows)),
                      ("location", f64(location, 3 * rows))):
        keep[name] = arr
        setattr(d, name, arr.ctypes.data)
    d.magnetisation, d.damping, d.temperature = float(magnetisation), float(damping), float(temperature)
    d.field_amplitude, d.field_frequency = float(field_amplitude), float(field_frequency)
    d.field_shape = _shape_code(field_shape)
    for k, v in (per_member or {}).items():
        arr = f64(v, E)
        keep["pm_" + k] = arr
        setattr(d, k + "_per_member", arr.ctypes.data)
    d.renorm, d.interactions, d.use_implicit = int(bool(renorm)), int(bool(interactions)), int(bool(use_implicit))
    d.eps, d.max_iter = float(implicit_tol), int(max_iter)
    d.time_step, d.end_time, d.max_samples = float(time_step), float(end_time), int(max_samples)
    d.seeds = seeds.ctypes.data
    if noise is not None:
        nz = f64(noise)
        keep["noise"] = nz
        d.noise = nz.ctypes.data
        d.noise_per_member = nz.size // max(E, 1)
    d.precision = _lib.PRECISIONS[precision]
    d.buffers_on_device = 0
    return d, keep, n


def _host_empty(shape):
    """Float64 host array for device results: page-locked memory from torch's
    caching host allocator when torch and a GPU are present (copied into at
    full link speed, and recycled across calls instead of being faulted in
    afresh), plain numpy otherwise.  The array keeps its backing alive."""
    try:
        import torch
        if torch.cuda.is_available():
            return torch.empty(shape, dtype=torch.float64, pin_memory=True).numpy()
    except ImportError:
        pass
    return np.empty(shape)


def simulate_ensemble(n_members, radius, anisotropy, anisotropy_axis, magnetisation_direction,
                      location, magnetisation, damping, temperature, renorm, interactions,
                      use_implicit, time_step, end_time, max_samples, seeds,
                      field_shape="constant", field_amplitude=0.0, field_frequency=0.0,
                      implicit_tol=1e-9, *, per_member_geometry=False, per_member=None,
                      precision="fp64", noise=None, max_iter=1000, keep_trajectories=True,
                      stream=None) -> EnsembleArrays:
    """All members in one GPU launch.

    Geometry arrays are one cluster ([N], [N][3]) shared by every member, or
    member-major ([E][N], [E][N][3]) with ``per_member_geometry=True``.
    ``per_member`` maps any of 'magnetisation', 'damping', 'temperature',
    'field_amplitude', 'field_frequency' to an [E] array overriding the scalar.
    ``noise``: optional injected increments [E][steps*3N].
    ``precision``: 'fp64' (the reference's arithmetic), 'mixed' (FP32 CUDA
    cores) or 'mixed_tc' (dipolar field on the tensor cores).
    """
    d, keep, n = _ensemble_desc(n_members, radius, anisotropy, anisotropy_axis,
                                magnetisation_direction, location, magnetisation, damping,
                                temperature, renorm, interactions, use_implicit, time_step,
                                end_time, max_samples, seeds, field_shape, field_amplitude,
                                field_frequency, implicit_tol, per_member_geometry, per_member,
                                precision, noise, max_iter)
    E, S = int(n_members), int(max_samples)
    P = E * n
    if keep_trajectories:
        mx, my, mz = _host_empty((3, S, P))
    else:
        mx = my = mz = None
    time, field = np.empty((E, S)), np.empty((E, S))
    status, steps = np.empty(E, dtype=np.int32), np.empty(E, dtype=np.int64)
    o = _lib.EnsembleOut(vptr(mx), vptr(my), vptr(mz), vptr(time), vptr(field), vptr(status),
                         vptr(steps))
    check(_lib.lib().magpy_ensemble_dynamics(C.byref(d), C.byref(o), stream))
    return EnsembleArrays(E, n, mx, my, mz, time, field, status, steps)


class EnsemblePlan:
    """A reusable device-resident ensemble run (magpy_plan_* of the C-ABI).

    Same arguments as ``simulate_ensemble``.  ``run()`` integrates on the GPU;
    trajectories stay on the device until ``arrays()`` copies them out;
    ``ensemble_magnetisation`` and ``energy_dissipated`` reduce them on the
    device in FP64.
    """

    def __init__(self, n_members, radius, anisotropy, anisotropy_axis, magnetisation_direction,
                 location, magnetisation, damping, temperature, renorm, interactions,
                 use_implicit, time_step, end_time, max_samples, seeds,
                 field_shape="constant", field_amplitude=0.0, field_frequency=0.0,
                 implicit_tol=1e-9, *, per_member_geometry=False, per_member=None,
                 precision="fp64", noise=None, max_iter=1000):
        d, self._keep, self.n_particles = _ensemble_desc(
            n_members, radius, anisotropy, anisotropy_axis, magnetisation_direction, location,
            magnetisation, damping, temperature, renorm, interactions, use_implicit, time_step,
            end_time, max_samples, seeds, field_shape, field_amplitude, field_frequency,
            implicit_tol, per_member_geometry, per_member, precision, noise, max_iter)
        self.handle = C.c_void_p()
        check(_lib.lib().magpy_plan_create(C.byref(d), C.byref(self.handle), None))
        E, n, S, K = (C.c_int64() for _ in range(4))
        _lib.lib().magpy_plan_shape(self.handle, C.byref(E), C.byref(n), C.byref(S), C.byref(K))
        self.n_members, self.n_samples, self.max_steps = E.value, S.value, K.value

    def run(self, stream=None):
        check(_lib.lib().magpy_plan_run(self.handle, stream))
        return self

    def set_launch(self, block_warps, members_per_warp=0):
        """Launch shape of the warp-packed kernels (clusters of <= 32 particles)."""
        check(_lib.lib().magpy_plan_set_launch(self.handle, int(block_warps),
                                               int(members_per_warp)))
        return self

    def set_wait_limit(self, polls):
        """Polls of the tensor-core kernel's MMA-completion waits before it
        gives up with MAGPY_STATUS_WATCHDOG (default 2^24; 0 gives up at the
        first wait)."""
        check(_lib.lib().magpy_plan_set_wait_limit(self.handle, int(polls)))
        return self

    def arrays(self) -> EnsembleArrays:
        E, n, S = self.n_members, self.n_particles, self.n_samples
        mx, my, mz = (np.empty((S, E * n)) for _ in range(3))
        time, field = np.empty((E, S)), np.empty((E, S))
        status, steps = np.empty(E, dtype=np.int32), np.empty(E, dtype=np.int64)
        o = _lib.EnsembleOut(vptr(mx), vptr(my), vptr(mz), vptr(time), vptr(field),
                             vptr(status), vptr(steps))
        check(_lib.lib().magpy_plan_copy_out(self.handle, C.byref(o), None))
        return EnsembleArrays(E, n, mx, my, mz, time, field, status, steps)

    def ensemble_magnetisation(self, direction="z"):
        out = np.empty(self.n_samples)
        check(_lib.lib().magpy_plan_ensemble_magnetisation(
            self.handle, "xyz".index(direction), dptr(out), None))
        return out

    def energy_dissipated(self, start_time=None, end_time=None):
        out = C.c_double(0.0)
        check(_lib.lib().magpy_plan_energy_dissipated(
            self.handle, float("nan") if start_time is None else float(start_time),
            float("nan") if end_time is None else float(end_time), C.byref(out), None))
        return out.value

    def save_results(self, prefix, member_begin=0, member_end=None, stream=None):
        """simulation::save_results files (lib/simulation.cpp:38-63) for every
        particle of members [member_begin, member_end): '<prefix>_<e>_<i>.mx' etc."""
        end = self.n_members if member_end is None else int(member_end)
        check(_lib.lib().magpy_plan_save_results(self.handle, str(prefix).encode(),
                                                 int(member_begin), end, stream))

    def close(self):
        if getattr(self, "handle", None):
            _lib.lib().magpy_plan_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class _GroupPlan(EnsemblePlan):
    """A plan owned by an EnsembleBatch (not destroyed by this object)."""

    def __init__(self, handle, n_particles):  # noqa: D401 - no EnsemblePlan.__init__
        self.handle = handle
        self.n_particles = n_particles
        E, n, S, K = (C.c_int64() for _ in range(4))
        _lib.lib().magpy_plan_shape(self.handle, C.byref(E), C.byref(n), C.byref(S), C.byref(K))
        self.n_members, self.n_samples, self.max_steps = E.value, S.value, K.value

    def close(self):
        self.handle = None


class EnsembleBatch:
    """Ensembles of uneven cluster sizes run as one CUDA-graph launch.

    ``groups`` is a list of dictionaries holding the arguments of
    ``simulate_ensemble`` (as keywords; 'n_members' ... 'seeds' plus the
    optional ones).  With ``autotune`` the kernel and the CTA shape of each
    group are chosen by timing them on the group's own ensemble.
    """

    _POS = ("n_members", "radius", "anisotropy", "anisotropy_axis", "magnetisation_direction",
            "location", "magnetisation", "damping", "temperature", "renorm", "interactions",
            "use_implicit", "time_step", "end_time", "max_samples", "seeds")
    _OPT = (("field_shape", "constant"), ("field_amplitude", 0.0), ("field_frequency", 0.0),
            ("implicit_tol", 1e-9), ("per_member_geometry", False), ("per_member", None),
            ("precision", "mixed"), ("noise", None), ("max_iter", 1000))

    def __init__(self, groups, autotune=True, stream=None):
        descs = (_lib.EnsembleDesc * len(groups))()
        self._keep = []
        self._n = []
        for i, g in enumerate(groups):
            args = [g[k] for k in self._POS] + [g.get(k, v) for k, v in self._OPT]
            d, keep, n = _ensemble_desc(*args)
            descs[i] = d
            self._keep.append(keep)
            self._n.append(n)
        self.handle = C.c_void_p()
        check(_lib.lib().magpy_batch_create(descs, len(groups), int(bool(autotune)),
                                            C.byref(self.handle), stream))
        self.groups = [_GroupPlan(self._plan_handle(i), self._n[i]) for i in range(len(groups))]

    def _plan_handle(self, i):
        h = C.c_void_p()
        check(_lib.lib().magpy_batch_group_plan(self.handle, i, C.byref(h)))
        return h

    def choice(self, i):
        """(precision name, warps per CTA, members per warp, tuned ms per step) of group i."""
        p, w, m, ms = C.c_int32(), C.c_int32(), C.c_int32(), C.c_double()
        check(_lib.lib().magpy_batch_group_choice(self.handle, i, C.byref(p), C.byref(w),
                                                  C.byref(m), C.byref(ms)))
        name = {v: k for k, v in _lib.PRECISIONS.items()}[p.value]
        return name, w.value, m.value, ms.value

    def run(self, stream=None):
        check(_lib.lib().magpy_batch_run(self.handle, stream))
        return self

    def close(self):
        if getattr(self, "handle", None):
            _lib.lib().magpy_batch_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def simulate_dom_batch(initial_probabilities, volume, anisotropy, temperature, magnetisation,
                       alpha, time_step, end_time, max_samples, field_shape="constant",
                       field_amplitude=0.0, field_frequency=0.0, field_n_components=1,
                       max_steps=0) -> dict:
    """Two-state master equation for a batch of independent particles in one
    GPU launch (simulate_dom of magpy/core.pyx:205-278, per particle).

    Every argument but the integration settings may be a scalar or an array
    of one value per particle (initial_probabilities: [2] or [E][2]).
    Returns arrays [E][S]: ``mz`` (p0 - p1), ``field`` (A/m), ``time`` (s),
    and ``status`` / ``steps`` per particle.
    """
    cols = [volume, anisotropy, temperature, magnetisation, alpha, field_amplitude,
            field_frequency]
    E = max(np.size(c) for c in cols)
    p0 = np.asarray(initial_probabilities, dtype=np.float64)
    if p0.ndim == 2:
        E = max(E, p0.shape[0])
    keep = [np.ascontiguousarray(np.broadcast_to(np.asarray(c, dtype=np.float64), (E,)))
            for c in cols]
    p0 = np.ascontiguousarray(np.broadcast_to(p0.reshape(-1, 2), (E, 2)))
    if field_shape not in _lib.DOM_FIELD_SHAPES:
        raise KeyError(field_shape)  # as the reference's string dispatch fails
    S = int(end_time / time_step) + 1 if max_samples == -1 else int(max_samples)
    d = _lib.DomDesc(E, *[vptr(a) for a in keep[:5]], vptr(p0), vptr(keep[5]), vptr(keep[6]),
                     _lib.DOM_FIELD_SHAPES[field_shape], int(field_n_components),
                     float(time_step), float(end_time), int(max_samples), int(max_steps))
    mz, field, time = (np.empty((E, max(S, 0))) for _ in range(3))
    status, steps = np.empty(E, dtype=np.int32), np.empty(E, dtype=np.int64)
    check(_lib.lib().magpy_dom_dynamics(C.byref(d), dptr(mz), dptr(field), dptr(time),
                                        status.ctypes.data_as(C.POINTER(C.c_int32)),
                                        steps.ctypes.data_as(C.POINTER(C.c_int64)), None))
    return dict(mz=mz, field=field, time=time, status=status, steps=steps)


def simulate_dom(initial_probabilities, volume, anisotropy, temperature, magnetisation, alpha,
                 time_step, end_time, max_samples, field_shape, field_amplitude,
                 field_frequency, field_n_components):
    """magpy/core.pyx:205-278 simulate_dom: one particle; the reference's
    result dictionary (N, time, field, x, y, z)."""
    r = simulate_dom_batch(initial_probabilities, volume, anisotropy, temperature,
                           magnetisation, alpha, time_step, end_time, max_samples, field_shape,
                           field_amplitude, field_frequency, field_n_components)
    S = r["mz"].shape[1]
    return {"N": 1, "time": r["time"][0], "field": r["field"][0],
            "x": {0: np.zeros(S)}, "y": {0: np.zeros(S)}, "z": {0: r["mz"][0]},
            "status": int(r["status"][0])}


def generate_clusters(n_members, n_particles, seeds, median_radius=8e-9, sigma=0.2,
                      spacing=2.2, packing_fraction=0.3, layout="sphere", moments="axes",
                      max_rounds=0, device=None, stream=None) -> dict:
    """Seeded cluster geometries drawn on the GPU (magpy_generate_clusters).

    Returns member-major arrays -- ``radius`` [E][N], ``anisotropy_axis``,
    ``magnetisation_direction``, ``location`` [E][N][3] -- ready for
    ``simulate_ensemble(..., per_member_geometry=True)``, and ``status`` [E].
    With ``device`` set (a torch device), the arrays are torch tensors on it
    and never leave the GPU.
    """
    E, n = int(n_members), int(n_particles)
    lay = {"sphere": 0, "chain": 1}[layout]
    mom = {"axes": 0, "random": 1}[moments]
    if device is None:
        sd = np.ascontiguousarray(seeds, dtype=np.int64)
        if sd.size != E:
            raise ValueError("one seed per member")
        out = dict(radius=np.empty((E, n)), anisotropy_axis=np.empty((E, n, 3)),
                   magnetisation_direction=np.empty((E, n, 3)), location=np.empty((E, n, 3)),
                   status=np.empty(E, dtype=np.int32))
        ptr = {k: v.ctypes.data for k, v in out.items()}
        seed_ptr = sd.ctypes.data
        on_dev = 0
    else:
        import torch
        sd = torch.as_tensor(np.asarray(seeds, dtype=np.int64), device=device)
        if sd.numel() != E:
            raise ValueError("one seed per member")
        f = dict(dtype=torch.float64, device=device)
        out = dict(radius=torch.empty((E, n), **f), anisotropy_axis=torch.empty((E, n, 3), **f),
                   magnetisation_direction=torch.empty((E, n, 3), **f),
                   location=torch.empty((E, n, 3), **f),
                   status=torch.empty(E, dtype=torch.int32, device=device))
        ptr = {k: v.data_ptr() for k, v in out.items()}
        seed_ptr = sd.data_ptr()
        on_dev = 1
    d = _lib.GeoDesc(E, n, lay, mom, float(median_radius), float(sigma), float(spacing),
                     float(packing_fraction), int(max_rounds), seed_ptr, on_dev)
    check(_lib.lib().magpy_generate_clusters(
        C.byref(d), ptr["radius"], ptr["anisotropy_axis"], ptr["magnetisation_direction"],
        ptr["location"], ptr["status"], stream))
    return out


def save_results(prefix, mx, my, mz, field, time) -> None:
    """Write one particle's trajectory in the format of simulation::save_results
    (lib/simulation.cpp:38-63): prefix.mx, .my, .mz, .field, .time, each the
    raw native-endian doubles of the array."""
    arrs = [np.ascontiguousarray(a, dtype=np.float64) for a in (mx, my, mz, field, time)]
    n = arrs[0].size
    if any(a.size != n for a in arrs):
        raise ValueError("the five arrays must have the same length")
    check(_lib.lib().magpy_save_results(str(prefix).encode(), *[dptr(a) for a in arrs], n))


def load_results(prefix) -> dict:
    """Read the five files written by ``save_results`` (or by the reference)."""
    return {k: np.fromfile(f"{prefix}.{k}", dtype=np.float64)
            for k in ("mx", "my", "mz", "field", "time")}


def step_count(time_step, end_time, max_samples) -> int:
    """Integration steps taken by full_dynamics (reduced units)."""
    k = C.c_int64(0)
    check(_lib.lib().magpy_step_count(float(time_step), float(end_time), int(max_samples),
                                      C.byref(k)))
    return int(k.value)


def wiener_increments(seed, n_particles, n_steps) -> np.ndarray:
    """The in-kernel generator's increments for one member, [n_steps][3N]."""
    out = np.empty((int(n_steps), 3 * int(n_particles)))
    check(_lib.lib().magpy_wiener_increments(int(seed), int(n_particles), int(n_steps),
                                             dptr(out)))
    return out


def llg_components(m, h, hj, axis, alpha, sr) -> dict:
    """Device evaluation of drift, diffusion, their Jacobians and the
    anisotropy field for a batch of states (see magpy_llg_components)."""
    m = f64(m).reshape(-1, 3)
    n = m.shape[0]
    out = {k: np.empty((n, w)) for k, w in (("drift", 3), ("diffusion", 9), ("drift_jac", 9),
                                             ("diff_jac", 27), ("anis", 3))}
    check(_lib.lib().magpy_llg_components(
        n, dptr(m), dptr(f64(h, 3 * n)), dptr(f64(hj, 9 * n)), dptr(f64(axis, 3 * n)),
        dptr(f64(alpha, n)), dptr(f64(sr, n)), dptr(out["drift"]), dptr(out["diffusion"]),
        dptr(out["drift_jac"]), dptr(out["diff_jac"]), dptr(out["anis"])))
    return out
