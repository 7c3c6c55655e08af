"""CUDA path against the oracle and the reference's fixtures, through the C-ABI."""
import os

import numpy as np
import pytest

from conftest import golden_files, load_reduced_case

pytestmark = pytest.mark.gpu
FIELDS = ("x", "y", "z", "field", "time")


def _gpu_reduced(core, inp, kw, noise, precision="fp64", max_iter=1000):
    return core.simulate_reduced(
        inp["n"], inp["sr"], inp["k_red"], inp["v_red"], inp["axes"], inp["m0"],
        inp["unit_dist"], inp["dist_mag"], kw.get("field_shape", "constant"),
        kw.get("happ", 0.0), kw.get("fapp", 0.0), kw.get("k_av", 2e4), kw.get("v_av", 1.0),
        kw.get("alpha", 0.1), kw.get("ms", 4e5), kw["dt"], kw["end_time"], noise,
        kw.get("renorm", False), kw.get("interactions", True), kw.get("use_implicit", False),
        kw.get("eps", 1e-9), kw["max_samples"], max_iter=max_iter, precision=precision)


def _assert_close(a, b, exact, rtol=1e-12):
    for k in FIELDS:
        if exact:
            assert np.array_equal(a[k], b[k]), (k, np.max(np.abs(a[k] - b[k])))
        else:
            np.testing.assert_allclose(a[k], b[k], rtol=rtol, atol=rtol, err_msg=k)


@pytest.mark.parametrize("path", golden_files("reduced_"), ids=os.path.basename)
def test_fp64_kernel_matches_reference_fixture(gpu_lib, path):
    """FP64 kernel == the reference's own output on the same injected increments.
    Bit-exact except with a sine field, where CUDA's sin differs from glibc's by
    <= 2 ulp (tolerance 1e-12, relative and absolute)."""
    from magpy_gb300 import core
    inp, kw, z = load_reduced_case(path)
    out = _gpu_reduced(core, inp, kw, z["noise"])
    assert out["status"] == 0
    _assert_close(out, z, exact=kw["field_shape"] != "sine")


@pytest.mark.parametrize("n", [1, 2, 3, 5, 8, 16, 27, 31, 32, 33, 64, 100])
@pytest.mark.parametrize("implicit", [False, True])
def test_fp64_kernel_matches_oracle(gpu_lib, oracle, n, implicit):
    from magpy_gb300 import core
    from oracle.pyoracle import reduced_inputs
    rng = np.random.default_rng(1000 + n + 7 * implicit)
    inp = reduced_inputs(rng, n)
    dt, end, S = 1.3e-3, (0.06 if n > 30 else 0.15), 7
    K = core.step_count(dt, end, S)
    noise = rng.normal(size=K * 3 * n)
    kw = dict(field_shape="square", happ=0.3, fapp=3.0, dt=dt, end_time=end, max_samples=S,
              use_implicit=implicit, renorm=(n % 2 == 1), interactions=True)
    a = _gpu_reduced(core, inp, kw, noise)
    b = oracle.full_dynamics_reduced(inp, noise=noise, **kw)
    assert a["status"] == b["status"] == 0
    assert a["steps"] == b["steps"] == K
    _assert_close(a, b, exact=True)


@pytest.mark.parametrize("path", golden_files("physical_"), ids=os.path.basename)
def test_physical_api_matches_oracle_with_injected_noise(gpu_lib, oracle, path):
    """magpy_full_dynamics (physical units, SI output) == the oracle's physical path
    on the same increments (the reference's RngMtNorm draws, replayed)."""
    from magpy_gb300 import core
    z = np.load(path)
    kw = {k[3:]: z[k].item() for k in z.files if k.startswith("kw_")}
    n = z["radius"].size
    K = core.step_count(kw["time_step"] * 1.0, kw["end_time"], kw["max_samples"])  # upper bound
    noise = oracle.mt_norm(kw["seed"], 1.0, 3 * n * (int(kw["end_time"] / kw["time_step"]) + 10))
    o = oracle.full_dynamics(z["radius"], z["anisotropy"], z["axes"], z["m0"], z["location"],
                             4e5, 0.1, 300.0, noise=noise, **kw)
    # with the reference's own draws the oracle reproduces the fixture exactly
    for k in FIELDS:
        assert np.array_equal(o[k], z[k]), k
    g = core.simulate(z["radius"], z["anisotropy"], z["axes"], z["m0"], z["location"], 4e5, 0.1,
                      300.0, kw["renorm"], kw["interactions"], kw["use_implicit"],
                      kw["time_step"], kw["end_time"], kw["max_samples"], kw["seed"],
                      kw["field_shape"], kw["field_amplitude"], kw["field_frequency"],
                      kw["eps"], noise=noise)
    assert g["status"] == 0
    for i in range(n):
        for c in "xyz":
            np.testing.assert_allclose(g[c][i], z[c][i], rtol=1e-12, atol=1e-12 * 4e5)
    np.testing.assert_array_equal(g["time"], z["time"])
    np.testing.assert_array_equal(g["field"], z["field"])


def test_components_match_reference(gpu_lib):
    from magpy_gb300 import core
    z = np.load(golden_files("components")[0])
    n = z["m"].shape[0]
    out = core.llg_components(z["m"], z["h"], z["hj"], np.tile([0, 0, 1.0], (n, 1)), z["alpha"],
                              z["sr"])
    assert np.array_equal(out["drift"], z["drift"])
    assert np.array_equal(out["diffusion"], z["diffusion"])
    assert np.array_equal(out["drift_jac"], z["drift_jac"])
    assert np.array_equal(out["diff_jac"], z["diff_jac"])
    # tests.cpp:23-52 goldens
    g = core.llg_components([[2, 3, 4]], [[1, 2, 3]], np.zeros(9), [[1.0, 2.0, 1.5]], [3.0], [2.0])
    assert list(g["drift"][0]) == [-34, -4, 20]
    assert list(g["diffusion"][0]) == [150, -28, -54, -44, 120, -68, -42, -76, 78]


def test_generator_matches_its_numpy_statement(gpu_lib):
    from magpy_gb300 import core
    from philox_ref import wiener
    for seed in (0, 1001, 2**31 - 5, 2**40 + 17):
        g = core.wiener_increments(seed, 7, 50)
        r = wiener(seed, 7, 50)
        np.testing.assert_allclose(g, r, rtol=0, atol=5e-6)


def test_generator_statistics(gpu_lib):
    from magpy_gb300 import core
    w = core.wiener_increments(12345, 64, 4000).ravel()
    assert abs(w.mean()) < 5e-3
    assert abs(w.var() - 1) < 5e-3
    assert abs(np.mean(w ** 4) - 3) < 0.05
    # independent streams for different seeds / particles / steps
    a = core.wiener_increments(1, 4, 2000)
    b = core.wiener_increments(2, 4, 2000)
    assert abs(np.corrcoef(a.ravel(), b.ravel())[0, 1]) < 0.02
    assert abs(np.corrcoef(a[:-1, 0], a[1:, 0])[0, 1]) < 0.05


@pytest.mark.parametrize("n,implicit", [(1, False), (3, True), (40, False)])
def test_in_kernel_generator_replays_exactly(gpu_lib, oracle, n, implicit):
    """The in-kernel generator run == the oracle fed with the generator's increments."""
    from magpy_gb300 import core
    from oracle.pyoracle import reduced_inputs
    rng = np.random.default_rng(n)
    radius = rng.uniform(6e-9, 8e-9, n)
    K = rng.uniform(1.5e4, 2.5e4, n)
    axes = rng.normal(size=(n, 3)); axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    m0 = rng.normal(size=(n, 3)); m0 /= np.linalg.norm(m0, axis=1, keepdims=True)
    loc = rng.uniform(0, 1, size=(n, 3)) * 20e-9 * n ** (1 / 3)
    loc += np.arange(n)[:, None] * np.array([25e-9, 0, 0])
    kw = dict(renorm=False, interactions=True, use_implicit=implicit, eps=1e-9, time_step=1e-13,
              end_time=2e-11, max_samples=9, seed=4242, field_shape="square",
              field_amplitude=5e3, field_frequency=1e9)
    g = core.simulate(radius, K, axes, m0, loc, 4e5, 0.1, 300.0, kw["renorm"], kw["interactions"],
                      kw["use_implicit"], kw["time_step"], kw["end_time"], kw["max_samples"],
                      kw["seed"], kw["field_shape"], kw["field_amplitude"], kw["field_frequency"],
                      kw["eps"])
    steps = 260
    w = core.wiener_increments(kw["seed"], n, steps).ravel()
    o = oracle.full_dynamics(radius, K, axes, m0, loc, 4e5, 0.1, 300.0, noise=w, **kw)
    assert o["status"] == 0
    for i in range(n):
        for c in "xyz":
            assert np.array_equal(g[c][i], o[c][i])


@pytest.mark.parametrize("n,renorm", [(1, False), (8, False), (64, False), (8, True),
                                      (27, True)])
def test_mixed_precision_strong_error(gpu_lib, oracle, n, renorm):
    """Mixed form vs the FP64 oracle on identical increments: strong error
    max_member |m_T - m_T^oracle| / |m_T^oracle| <= 1e-5, with and without
    renormalisation (lib/simulation.cpp:379-387)."""
    from magpy_gb300 import core
    from oracle.pyoracle import reduced_inputs
    rng = np.random.default_rng(77 + n)
    inp = reduced_inputs(rng, n)
    dt, end, S = 8.7e-4, 8.7e-4 * 3000, 11
    K = core.step_count(dt, end, S)
    noise = rng.normal(size=K * 3 * n)
    kw = dict(field_shape="sine", happ=0.12, fapp=1e-3, dt=dt, end_time=end, max_samples=S,
              interactions=True, renorm=renorm)
    a = _gpu_reduced(core, inp, kw, noise, precision="mixed")
    b = oracle.full_dynamics_reduced(inp, noise=noise, **kw)
    mT = np.stack([a[c][:, -1] for c in "xyz"], 1)
    oT = np.stack([b[c][:, -1] for c in "xyz"], 1)
    err = np.max(np.linalg.norm(mT - oT, axis=1) / np.linalg.norm(oT, axis=1))
    assert err <= 1e-5, err


def test_status_bits(gpu_lib):
    from magpy_gb300 import core
    from magpy_gb300._lib import MagpyError
    from oracle.pyoracle import reduced_inputs
    inp = reduced_inputs(np.random.default_rng(5), 4)
    kw = dict(dt=1e-3, end_time=0.02, max_samples=5, use_implicit=True)
    K = core.step_count(1e-3, 0.02, 5)
    noise = np.random.default_rng(6).normal(size=K * 12)
    # Newton limit reached (MAX_ITERATIONS_ERR, optimisation.cpp:147)
    out = _gpu_reduced(core, inp, kw, noise, max_iter=1)
    assert out["status"] & 1
    # injected increments shorter than the run (RngArray out_of_range)
    with pytest.raises(MagpyError, match="noise"):
        _gpu_reduced(core, inp, kw, noise[:-1])
    # a non-finite initial state is reported, not hidden
    bad = dict(inp)
    bad["m0"] = inp["m0"].copy()
    bad["m0"][2, 1] = np.nan
    out = _gpu_reduced(core, bad, dict(kw, use_implicit=False), noise)
    assert out["status"] & 4


def test_ensemble_model_matches_single_models(gpu_lib):
    """EnsembleModel (one launch) == Model.simulate per member with the seeds of
    magpy/model.py:202-203."""
    import magpy_gb300 as mp
    base = mp.Model([7e-9, 6e-9], [2e4, 2.2e4], [[0, 0, 1], [0, 1, 0]], [[0, 0, 1], [1, 0, 0]],
                    [[0, 0, 0], [20e-9, 0, 0]], 4e5, 0.1, 300, field_shape="sine",
                    field_frequency=3e9, field_amplitude=5e3)
    ens = mp.EnsembleModel(5, base, damping=[0.1, 0.05, 0.2, 0.1, 0.3])
    r = ens.simulate(1e-11, 1e-13, 11, 42, implicit_solve=False)
    seeds = ens.seeds(42)
    for e in range(5):
        single = ens.models[e].simulate(1e-11, 1e-13, 11, seed=int(seeds[e]), implicit_solve=False)
        for i in range(2):
            np.testing.assert_array_equal(r.results[e].z[i], single.z[i])
    assert r.ensemble_magnetisation().shape == (11,)


@pytest.mark.parametrize("precision", ["fp64", "mixed_tc"])
def test_device_statistics_match_host(gpu_lib, precision):
    """EnsemblePlan statistics (FP64 device reductions) == EnsembleResults on the
    copied trajectories (magpy/results.py:134-191 as the reference writes it)."""
    from magpy_gb300 import core
    from magpy_gb300.results import EnsembleResults
    rng = np.random.default_rng(3)
    n, E = 8, 64
    axes = rng.normal(size=(n, 3)); axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    loc = np.stack([np.arange(n) * 20e-9, np.zeros(n), np.zeros(n)], 1)
    plan = core.EnsemblePlan(E, rng.uniform(6e-9, 8e-9, n), np.full(n, 2e4), axes, axes, loc,
                             4e5, 0.1, 300.0, False, True, False, 5e-14, 5e-14 * 600, 31,
                             rng.integers(0, 2**31 - 1, size=E), "sine", 1e4, 1e9,
                             precision=precision)
    plan.run()
    arr = plan.arrays()
    host = EnsembleResults(arrays=arr)
    for c in "xyz":
        np.testing.assert_allclose(plan.ensemble_magnetisation(c), host.ensemble_magnetisation(c),
                                   rtol=1e-12, atol=1e-9)
    e_dev = plan.energy_dissipated()
    e_host = host.energy_dissipated()
    assert abs(e_dev - e_host) <= 1e-10 * max(1.0, abs(e_host))
    t = arr.time[0]
    e_dev = plan.energy_dissipated(t[5], t[20])
    e_host = host.energy_dissipated(t[5], t[20])
    assert abs(e_dev - e_host) <= 1e-10 * max(1.0, abs(e_host))
    plan.close()
