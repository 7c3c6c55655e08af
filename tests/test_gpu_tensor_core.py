"""Tensor-core dipolar path (tcgen05, FP16 hi/lo split, FP32 accumulation)."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cluster(rng, n, spacing=2.3):
    from oracle.pyoracle import reduced_inputs
    return reduced_inputs(rng, n, spacing=spacing)


@pytest.mark.parametrize("n,E", [(2, 3), (5, 33), (16, 40), (27, 64), (43, 37), (64, 70)])
def test_dipolar_field_matches_fp64(gpu_lib, oracle, n, E):
    """magpy_dipolar_field_tc == field::multi_add_dipolar (FP64 oracle) to ~1e-6 of |h|."""
    from magpy_gb300 import _lib
    from oracle.pyoracle import _f64
    rng = np.random.default_rng(n)
    inp = _cluster(rng, n)
    cubes = inp["dist_mag"] ** 3
    np.fill_diagonal(cubes, 0.0)
    unit = np.nan_to_num(inp["unit_dist"])
    mag = rng.normal(size=(E, n, 3))
    mag /= np.linalg.norm(mag, axis=2, keepdims=True)
    field = np.zeros((E, n, 3))
    _lib.check(gpu_lib.magpy_dipolar_field_tc(n, E, 4e5, 2e4, _lib.dptr(_f64(inp["v_red"])),
                                              _lib.dptr(_f64(unit)), _lib.dptr(_f64(cubes)),
                                              _lib.dptr(_f64(mag)), _lib.dptr(field)))
    ref = np.stack([oracle.multi_add_dipolar(np.zeros(3 * n), 4e5, 2e4, inp["v_red"], mag[e],
                                             unit, cubes).reshape(n, 3) for e in range(E)])
    scale = np.max(np.abs(ref))
    err = np.max(np.abs(field - ref))
    assert err <= 2e-6 * scale, (err, scale)


@pytest.mark.parametrize("n", [2, 8, 27, 42, 43, 50, 64])
def test_tc_integrator_strong_error_vs_oracle(gpu_lib, oracle, n):
    """One member through the reduced entry point in tensor-core mode against the
    FP64 oracle on identical injected increments: strong error <= 1e-5."""
    from magpy_gb300 import core
    rng = np.random.default_rng(500 + n)
    inp = _cluster(rng, n)
    dt, end, S = 8.7e-4, 8.7e-4 * 2000, 9
    K = core.step_count(dt, end, S)
    noise = rng.normal(size=K * 3 * n)
    kw = dict(field_shape="sine", happ=0.12, fapp=1e-3, dt=dt, end_time=end, max_samples=S,
              interactions=True)
    a = core.simulate_reduced(n, inp["sr"], inp["k_red"], inp["v_red"], inp["axes"], inp["m0"],
                              inp["unit_dist"], inp["dist_mag"], "sine", 0.12, 1e-3, 2e4, 1.0,
                              0.1, 4e5, dt, end, noise, False, True, False, 1e-9, S,
                              precision="mixed_tc")
    b = oracle.full_dynamics_reduced(inp, noise=noise, **kw)
    assert a["status"] == 0 and a["steps"] == b["steps"] == K
    for s in range(S):
        mT = np.stack([a[c][:, s] for c in "xyz"], 1)
        oT = np.stack([b[c][:, s] for c in "xyz"], 1)
        err = np.max(np.linalg.norm(mT - oT, axis=1) / np.linalg.norm(oT, axis=1))
        assert err <= 1e-5, (s, err)
    np.testing.assert_array_equal(a["time"], b["time"])


@pytest.mark.parametrize("n,E,renorm", [(8, 70, False), (43, 17, False), (64, 40, False),
                                         (64, 129, False), (27, 45, True), (64, 40, True)])
def test_tc_ensemble_matches_fp64_kernel(gpu_lib, n, E, renorm):
    """Ensemble in tensor-core mode (partial last CTA; odd N leaves the last
    particle pair half empty) against the FP64 kernel with the same in-kernel
    increments, with and without renormalisation."""
    from magpy_gb300 import core
    rng = np.random.default_rng(n + E)
    side = int(np.ceil(n ** (1 / 3)))
    grid = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    radius = rng.uniform(6e-9, 9e-9, n)
    axes = rng.normal(size=(n, 3)); axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    loc = grid * 20e-9
    seeds = rng.integers(0, 2**31 - 1, size=E)
    args = (E, radius, np.full(n, 2e4), axes, axes, loc, 4e5, 0.1, 300.0, renorm, True, False,
            5e-14, 5e-14 * 400, 5, seeds, "sine", 1e4, 3e8)
    a = core.simulate_ensemble(*args, precision="mixed_tc")
    b = core.simulate_ensemble(*args, precision="fp64")
    assert np.all(a.status == 0) and np.all(b.status == 0)
    assert np.array_equal(a.steps, b.steps)
    for m1, m2 in ((a.mx, b.mx), (a.my, b.my), (a.mz, b.mz)):
        assert np.max(np.abs(m1 - m2)) <= 1e-5 * 4e5
    np.testing.assert_array_equal(a.time, b.time)


def test_tc_headline_window_strong_error_vs_fp64_kernel(gpu_lib):
    """The benchmark's headline workload (N = 64 sphere cluster, E = 4096
    members sharing it, AC 10 kA/m at 300 kHz, dt = 5e-14 s) over its timed
    2001-step window: the tensor-core form against the FP64-faithful kernel
    on identical in-kernel increments, every particle of every member within
    1e-5 relative strong error at the end of the window."""
    from bench import workload
    from magpy_gb300 import core
    wl = workload(4096, 64, 2000, 11)
    g = wl["geo"]
    args = (wl["E"], g["radius"], g["anisotropy"], g["anisotropy_axis"],
            g["magnetisation_direction"], g["location"], wl["ms"], wl["damping"],
            wl["temperature"], False, True, False, wl["dt"], wl["end_time"], wl["samples"],
            wl["seeds"], wl["field_shape"], wl["field_amplitude"], wl["field_frequency"])
    a = core.simulate_ensemble(*args, precision="mixed_tc")
    b = core.simulate_ensemble(*args, precision="fp64")
    assert np.all(a.status == 0) and np.all(b.status == 0)
    assert np.all(a.steps == 2001) and np.array_equal(a.steps, b.steps)
    ma = np.stack([a.mx[-1], a.my[-1], a.mz[-1]], 1)
    mb = np.stack([b.mx[-1], b.my[-1], b.mz[-1]], 1)
    err = np.linalg.norm(ma - mb, axis=1) / np.linalg.norm(mb, axis=1)
    assert err.size == 4096 * 64
    assert err.max() <= 1e-5, err.max()


def test_tc_watchdog_gives_up_and_leaves_the_context_usable(gpu_lib):
    """A phase-wait limit of 0 polls makes the tensor-core kernel's first wait
    for its MMAs run out: every member reports MAGPY_STATUS_WATCHDOG, stops
    at step 0 with NaN samples after the initial one, and the kernel frees its
    tensor memory after draining the MMAs in flight with the long bound.  The
    same plan, run again with the default limit, then matches the FP64
    kernel (the context and the tensor memory are intact)."""
    from magpy_gb300 import _lib, core
    rng = np.random.default_rng(16)
    n, E = 27, 70
    grid = np.stack(np.meshgrid(*[np.arange(3)] * 3, indexing="ij"), -1).reshape(-1, 3)
    axes = rng.normal(size=(n, 3)); axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    seeds = rng.integers(0, 2**31 - 1, size=E)
    args = (E, rng.uniform(6e-9, 9e-9, n), np.full(n, 2e4), axes, axes, grid * 20e-9, 4e5, 0.1,
            300.0, False, True, False, 5e-14, 5e-14 * 300, 5, seeds, "sine", 1e4, 3e8)
    plan = core.EnsemblePlan(*args, precision="mixed_tc")
    try:
        plan.set_wait_limit(0).run()
        a = plan.arrays()
        assert np.all(a.status & _lib.STATUS_WATCHDOG)
        assert np.all(a.steps == 0)
        assert np.all(np.isfinite(a.mz[0])) and np.all(np.isnan(a.mz[1:]))
        plan.set_wait_limit(1 << 24).run()
        b = plan.arrays()
        assert np.all(b.status == 0)
        ref = core.simulate_ensemble(*args, precision="fp64")
        assert np.array_equal(b.steps, ref.steps)
        for m1, m2 in ((b.mx, ref.mx), (b.my, ref.my), (b.mz, ref.mz)):
            assert np.max(np.abs(m1 - m2)) <= 1e-5 * 4e5
    finally:
        plan.close()


@pytest.mark.parametrize("n,shape", [(64, "square"), (64, "sine"), (70, "square"),
                                     (125, "sine")])
def test_tc_fast_field_matches_fp64_kernel(gpu_lib, n, shape):
    """The tensor-core kernels compute the applied field themselves (the
    single-CTA kernel for n <= 64, the cluster kernel above).  A strong field
    (2e5 A/m, about 2.5 anisotropy fields) with a period of ten steps makes a
    misplaced field step visible: a field one step off changes the torque by
    ~4e-3 per affected step, while the tensor-core form stays within ~1e-6 of
    the FP64-faithful kernel (which evaluates the FP64 waveform itself) on
    the same in-kernel increments.  300 steps, 1e-4 relative."""
    from magpy_gb300 import core
    rng = np.random.default_rng(n + 5)
    E = 40
    side = int(np.ceil(n ** (1 / 3)))
    grid = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    axes = rng.normal(size=(n, 3)); axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    seeds = rng.integers(0, 2**31 - 1, size=E)
    dt = 5e-14
    args = (E, rng.uniform(6e-9, 8e-9, n), np.full(n, 2e4), axes, axes, grid * 20e-9, 4e5, 0.1,
            300.0, False, True, False, dt, dt * 299.5, 7, seeds, shape, 2e5, 1 / (10 * dt))
    a = core.simulate_ensemble(*args, precision="mixed_tc")
    b = core.simulate_ensemble(*args, precision="fp64")
    assert np.all(a.status == 0) and np.all(b.status == 0)
    np.testing.assert_array_equal(a.field, b.field)
    for m1, m2 in ((a.mx, b.mx), (a.my, b.my), (a.mz, b.mz)):
        assert np.max(np.abs(m1 - m2)) <= 1e-4 * 4e5
