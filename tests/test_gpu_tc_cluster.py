"""Tensor-core dipolar path for clusters of more than 64 particles: D split
over a thread-block cluster of ceil(n/42) CTAs, streamed with bulk copies
(sllg_tcc.cu).  Checked against the FP64 oracle (field::multi_add_dipolar and
the reduced full_dynamics on injected increments) and against the
FP64-faithful kernel on in-kernel increments."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _cluster(rng, n, spacing=2.3):
    from oracle.pyoracle import reduced_inputs
    return reduced_inputs(rng, n, spacing=spacing)


@pytest.mark.parametrize("n,E", [(65, 3), (84, 33), (85, 40), (125, 70), (300, 5), (512, 33),
                                 (672, 2)])
def test_cluster_dipolar_field_matches_fp64(gpu_lib, oracle, n, E):
    """magpy_dipolar_field_tc for n > 64 == field::multi_add_dipolar (FP64
    oracle) to 2e-6 sqrt(n / 64) of the largest |h|: each of the 3n products
    carries the ~2^-22 relative error of the FP16 hi/lo split and FP32
    accumulation, and independent roundings of a 3n-term sum grow as its
    square root (the n <= 64 kernel is held to 2e-6)."""
    from magpy_gb300 import _lib
    from oracle.pyoracle import _f64
    rng = np.random.default_rng(n + 7)
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
    assert err <= 2e-6 * max(1.0, np.sqrt(n / 64)) * scale, (err, scale)


@pytest.mark.parametrize("n,steps", [(65, 2000), (125, 2000), (512, 300)])
def test_cluster_integrator_strong_error_vs_oracle(gpu_lib, oracle, n, steps):
    """One member through the reduced entry point in tensor-core mode against
    the FP64 oracle on identical injected increments: strong error <= 1e-5 at
    every sample."""
    from magpy_gb300 import core
    rng = np.random.default_rng(900 + n)
    inp = _cluster(rng, n)
    dt, S = 8.7e-4, 7
    end = dt * steps
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


def _lattice_ensemble(rng, n, E, renorm=False):
    side = int(np.ceil(n ** (1 / 3)))
    grid = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    radius = rng.uniform(6e-9, 9e-9, n)
    axes = rng.normal(size=(n, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    seeds = rng.integers(0, 2**31 - 1, size=E)
    return (E, radius, np.full(n, 2e4), axes, axes, grid * 20e-9, 4e5, 0.1, 300.0, renorm, True,
            False, 5e-14, 5e-14 * 400, 5, seeds, "sine", 1e4, 3e8)


@pytest.mark.parametrize("n,E,nb,renorm", [(65, 70, 64, False), (125, 130, 64, False),
                                           (125, 45, 32, True), (170, 33, 32, False),
                                           (343, 20, 64, False), (125, 100, 48, False),
                                           (216, 50, 48, True), (125, 90, 40, False),
                                           (170, 41, 40, True)])
def test_cluster_ensemble_matches_fp64_kernel(gpu_lib, n, E, nb, renorm):
    """Ensembles in tensor-core mode (partial last member tile; odd n leaves
    the last pair half empty) against the FP64 kernel with the same in-kernel
    increments, 64, 48 or 32 members per thread-block cluster (chosen explicitly;
    by default the plan picks the fewer member-waves), with and without
    renormalisation."""
    from magpy_gb300 import core
    rng = np.random.default_rng(n * 3 + E)
    args = _lattice_ensemble(rng, n, E, renorm)
    plan = core.EnsemblePlan(*args, precision="mixed_tc")
    try:
        plan.set_launch(4, nb)
        a = plan.run().arrays()
    finally:
        plan.close()
    b = core.simulate_ensemble(*args, precision="fp64")
    assert np.all(a.status == 0) and np.all(b.status == 0)
    assert np.array_equal(a.steps, b.steps)
    for m1, m2 in ((a.mx, b.mx), (a.my, b.my), (a.mz, b.mz)):
        assert np.max(np.abs(m1 - m2)) <= 1e-5 * 4e5
    np.testing.assert_array_equal(a.time, b.time)


def test_cluster_watchdog_gives_up_and_leaves_the_context_usable(gpu_lib):
    """A phase-wait limit of 0 polls: every CTA's first wait runs out, the
    cluster stops together at its first check, every member reports
    MAGPY_STATUS_WATCHDOG, the copies and MMAs in flight are drained before
    the tensor memory is freed, and the same plan then runs correctly."""
    from magpy_gb300 import _lib, core
    rng = np.random.default_rng(5)
    args = _lattice_ensemble(rng, 125, 70)
    plan = core.EnsemblePlan(*args, precision="mixed_tc")
    try:
        a = plan.set_wait_limit(0).run().arrays()
        assert np.all(a.status & _lib.STATUS_WATCHDOG)
        b = plan.set_wait_limit(1 << 24).run().arrays()
        assert np.all(b.status == 0)
    finally:
        plan.close()
    ref = core.simulate_ensemble(*args, precision="fp64")
    for m1, m2 in ((b.mx, ref.mx), (b.my, ref.my), (b.mz, ref.mz)):
        assert np.max(np.abs(m1 - m2)) <= 1e-5 * 4e5


# ---- implicit midpoint with the dipolar field on the tensor cores ----

@pytest.mark.parametrize("n,steps,shape", [(27, 60, "sine"), (65, 40, "square"),
                                           (125, 30, "constant"), (512, 8, "sine")])
def test_cluster_implicit_strong_error_vs_oracle(gpu_lib, oracle, n, steps, shape):
    """Implicit midpoint in tensor-core mode (FP64 state, residual and norms;
    dipolar field ~22 bits; FP32 quasi-Jacobian) for one member through the
    reduced entry point, against the FP64 oracle on identical injected
    increments: strong error <= 1e-5 at every sample, Newton converged."""
    from magpy_gb300 import core
    from oracle.pyoracle import reduced_inputs
    from test_gpu_parity import _gpu_reduced
    rng = np.random.default_rng(1300 + n)
    inp = reduced_inputs(rng, n)
    dt, S = 1.3e-3, 5
    end = dt * steps
    K = core.step_count(dt, end, S)
    noise = rng.normal(size=K * 3 * n)
    kw = dict(field_shape=shape, happ=0.3, fapp=3.0, dt=dt, end_time=end, max_samples=S,
              use_implicit=True, renorm=False, interactions=True)
    a = _gpu_reduced(core, inp, kw, noise, precision="mixed_tc")
    b = oracle.full_dynamics_reduced(inp, noise=noise, **kw)
    assert a["status"] == 0 and b["status"] == 0
    for s in range(S):
        mT = np.stack([a[c][:, s] for c in "xyz"], 1)
        oT = np.stack([b[c][:, s] for c in "xyz"], 1)
        err = np.max(np.linalg.norm(mT - oT, axis=1) / np.linalg.norm(oT, axis=1))
        assert err <= 1e-5, (s, err)


@pytest.mark.parametrize("n,E,steps,nb", [(64, 70, 100, 64), (125, 45, 60, 32),
                                          (512, 66, 20, 64), (125, 90, 60, 40),
                                          (300, 50, 30, 40), (125, 45, 40, 40)])
def test_cluster_implicit_ensemble_matches_fp64_kernel(gpu_lib, n, E, steps, nb):
    """Sphere clusters (alpha = 0.01, dt = 2e-13 s, AC field, as the large
    implicit workload) in tensor-core mode against the FP64-faithful kernel on
    the same in-kernel increments: strong error <= 1e-5, the same steps.  64,
    40 or 32 members per thread-block cluster (40: the correction MMA runs at
    N = 48 and the epilogue reads member halves of 20 columns; E = 90, 50 and
    45 leave partial last tiles, and at E = 45 the 40-member layout needs the
    largest B buffer of all member counts)."""
    from magpy_gb300 import core
    from test_gpu_large_clusters import _sphere_cluster
    radius, loc, axes = _sphere_cluster(n, n + 1)
    dt = 2e-13
    seeds = np.arange(E) + 31
    args = (E, radius, np.full(n, 2e4), axes, axes.copy(), loc, 4e5, 0.01, 300.0, False, True,
            True, dt, dt * (steps - 0.5), 3, seeds, "sine", 1e4, 3e5, 1e-9)
    a64 = core.simulate_ensemble(*args, precision="fp64")
    plan = core.EnsemblePlan(*args, precision="mixed_tc")
    try:
        plan.set_launch(4, nb)
        atc = plan.run().arrays()
    finally:
        plan.close()
    assert np.all(a64.status == 0) and np.all(atc.status == 0)
    assert np.array_equal(atc.steps, a64.steps)
    m64 = np.stack([a64.mx[-1], a64.my[-1], a64.mz[-1]], 1)
    mtc = np.stack([atc.mx[-1], atc.my[-1], atc.mz[-1]], 1)
    err = np.linalg.norm(mtc - m64, axis=1) / np.linalg.norm(m64, axis=1)
    assert err.max() < 1e-5, err.max()


def test_cluster_implicit_newton_limit_status(gpu_lib):
    """max_iter = 1: every member's Newton iteration stops at its limit and
    reports MAGPY_STATUS_NEWTON_MAXITER, as the FP64 kernel does."""
    from magpy_gb300 import _lib, core
    from test_gpu_large_clusters import _sphere_cluster
    n, E = 80, 9
    radius, loc, axes = _sphere_cluster(n, 5)
    args = (E, radius, np.full(n, 2e4), axes, axes.copy(), loc, 4e5, 0.01, 300.0, False, True,
            True, 2e-13, 2e-13 * 5.5, 3, np.arange(E) + 1, "sine", 1e4, 3e5, 1e-9)
    a = core.simulate_ensemble(*args, precision="mixed_tc", max_iter=1)
    b = core.simulate_ensemble(*args, precision="fp64", max_iter=1)
    assert np.all(b.status & _lib.STATUS_NEWTON_MAXITER)
    assert np.all(a.status & _lib.STATUS_NEWTON_MAXITER)
    assert np.array_equal(a.steps, b.steps)


def test_cluster_implicit_renorm_square_field_matches_fp64_kernel(gpu_lib):
    """Implicit midpoint with renormalisation and a square field, 96 members
    (three 32-member clusters or two of 64, by the wave rule), against the
    FP64 kernel on the same in-kernel increments."""
    from magpy_gb300 import core
    from test_gpu_large_clusters import _sphere_cluster
    n, E, steps = 125, 96, 30
    radius, loc, axes = _sphere_cluster(n, 17)
    args = (E, radius, np.full(n, 2e4), axes, axes.copy(), loc, 4e5, 0.05, 300.0, True, True,
            True, 2e-13, 2e-13 * (steps - 0.5), 4, np.arange(E) + 7, "square", 8e3, 1e9, 1e-9)
    a = core.simulate_ensemble(*args, precision="mixed_tc")
    b = core.simulate_ensemble(*args, precision="fp64")
    assert np.all(a.status == 0) and np.all(b.status == 0)
    assert np.array_equal(a.steps, b.steps)
    ma = np.stack([a.mx[-1], a.my[-1], a.mz[-1]], 1)
    mb = np.stack([b.mx[-1], b.my[-1], b.mz[-1]], 1)
    err = np.linalg.norm(ma - mb, axis=1) / np.linalg.norm(mb, axis=1)
    assert err.max() < 1e-5, err.max()
    assert np.allclose(np.linalg.norm(ma, axis=1), 4e5, rtol=1e-12)


def test_cluster_heun_constant_field_matches_fp64_kernel(gpu_lib):
    """A constant applied field (no per-step field table) on the cluster
    kernel against the FP64 kernel."""
    from magpy_gb300 import core
    rng = np.random.default_rng(23)
    args = list(_lattice_ensemble(rng, 100, 50))
    args[16], args[17], args[18] = "constant", 6e3, 0.0
    a = core.simulate_ensemble(*args, precision="mixed_tc")
    b = core.simulate_ensemble(*args, precision="fp64")
    assert np.all(a.status == 0) and np.all(b.status == 0)
    for m1, m2 in ((a.mx, b.mx), (a.my, b.my), (a.mz, b.mz)):
        assert np.max(np.abs(m1 - m2)) <= 1e-5 * 4e5


def test_cluster_mode_refuses_per_member_geometries(gpu_lib):
    """D is one matrix for the launch: members with their own geometries are
    refused with a message, not integrated with the wrong D."""
    from magpy_gb300 import core
    from magpy_gb300._lib import MagpyError
    n, E = 80, 3
    rng = np.random.default_rng(2)
    side = int(np.ceil(n ** (1 / 3)))
    grid = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    loc = np.concatenate([grid * 20e-9 * (1 + 0.01 * e) for e in range(E)])
    axes = np.tile([0, 0, 1.0], (E * n, 1))
    with pytest.raises(MagpyError, match="share one geometry"):
        core.simulate_ensemble(E, np.full(E * n, 7e-9), np.full(E * n, 2e4), axes, axes, loc,
                               4e5, 0.1, 300.0, False, True, False, 1e-13, 1e-11, 3,
                               np.arange(E), per_member_geometry=True, precision="mixed_tc")
