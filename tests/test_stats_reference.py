"""Ensemble statistics against the reference's own magpy/results.py.

tests/golden/stats_reference.npz holds trajectories of a small interacting
ensemble in an AC field produced by the reference's simulation::full_dynamics
(its own RngMtNorm noise per member seed) and the statistics the reference's
Results / EnsembleResults (magpy/results.py:61-217) compute from them:
member and ensemble magnetisation, energy dissipated over the run, over a
window and over the final field cycle (tests/golden/make_stats_golden.py).

The CPU tests put the same trajectories through this package's results
module (both the list-of-Results form and the dense-array form).  The GPU
test replays the reference's noise through the FP64 kernel and reduces the
device trajectories on the device (stats.cu).
"""
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "stats_reference.npz")


def _gold():
    z = np.load(GOLD)
    kw = {k[3:]: z[k].item() for k in z.files if k.startswith("kw_")}
    return z, kw


def _check(ens, z, kw, rtol):
    for c in "xyz":
        np.testing.assert_allclose(ens.ensemble_magnetisation(c), z["ensemble_magnetisation_" + c],
                                   rtol=rtol, atol=rtol * 4e5)
    np.testing.assert_allclose(np.array(ens.magnetisation("z")), z["member_magnetisation_z"],
                               rtol=rtol, atol=rtol * 4e5)
    scale = abs(float(z["energy_dissipated"].ravel()[0]))
    assert abs(ens.energy_dissipated() - float(z["energy_dissipated"].ravel()[0])) <= rtol * scale
    w = z["window"]
    assert abs(ens.energy_dissipated(w[0], w[1]) - float(z["energy_dissipated_window"])) <= \
        rtol * scale
    assert abs(ens.final_cycle_energy_dissipated(kw["field_frequency"]) -
               float(z["final_cycle_energy_dissipated"])) <= rtol * scale


def test_results_list_form_matches_reference_results_module():
    from magpy_gb300.results import EnsembleResults, Results
    z, kw = _gold()
    E, N, S = z["x"].shape
    members = [Results(z["time"], z["field"], {i: z["x"][e, i] for i in range(N)},
                       {i: z["y"][e, i] for i in range(N)}, {i: z["z"][e, i] for i in range(N)}, N)
               for e in range(E)]
    _check(EnsembleResults(members), z, kw, 1e-13)


def test_results_dense_form_matches_reference_results_module():
    from magpy_gb300.core import EnsembleArrays
    from magpy_gb300.results import EnsembleResults
    z, kw = _gold()
    E, N, S = z["x"].shape
    # [E][N][S] -> sample-major [S][E*N]
    dense = [np.ascontiguousarray(z[c].reshape(E * N, S).T) for c in "xyz"]
    arr = EnsembleArrays(E, N, *dense, np.tile(z["time"], (E, 1)), np.tile(z["field"], (E, 1)),
                         np.zeros(E, dtype=np.int32), np.zeros(E, dtype=np.int64))
    _check(EnsembleResults(arrays=arr), z, kw, 1e-13)


@pytest.mark.gpu
def test_device_statistics_match_reference_results_module(gpu_lib, oracle):
    """FP64 kernel on the reference's own draws (RngMtNorm per member seed,
    replayed by the oracle's restatement of mt19937_64 and
    normal_distribution): trajectories within 1e-12 of the reference's (the
    device sine differs from glibc's by a few ulp), and the device
    reductions within 1e-10 of the reference's results.py on them."""
    from magpy_gb300 import core
    z, kw = _gold()
    E, N, S = z["x"].shape
    seeds = z["seeds"]
    K = core.step_count(kw["time_step"], kw["end_time"], S)
    npm = 3 * N * (K + 8)
    noise = np.stack([oracle.mt_norm(int(s), 1.0, npm) for s in seeds])
    plan = core.EnsemblePlan(E, z["radius"], z["anisotropy"], z["axes"], z["m0"], z["location"],
                             float(z["ms"]), float(z["damping"]), float(z["temperature"]),
                             kw["renorm"], kw["interactions"], kw["use_implicit"],
                             kw["time_step"], kw["end_time"], S, seeds, kw["field_shape"],
                             kw["field_amplitude"], kw["field_frequency"], kw["eps"],
                             precision="fp64", noise=noise)
    try:
        plan.run()
        arr = plan.arrays()
        assert np.all(arr.status == 0)
        for c, m in (("x", arr.mx), ("y", arr.my), ("z", arr.mz)):
            traj = m.T.reshape(E, N, S)
            np.testing.assert_allclose(traj, z[c], rtol=1e-12, atol=1e-12 * 4e5)
        np.testing.assert_array_equal(arr.time[0], z["time"])
        for c in "xyz":
            np.testing.assert_allclose(plan.ensemble_magnetisation(c),
                                       z["ensemble_magnetisation_" + c], rtol=1e-10,
                                       atol=1e-10 * 4e5)
        scale = abs(float(z["energy_dissipated"].ravel()[0]))
        assert abs(plan.energy_dissipated() - float(z["energy_dissipated"].ravel()[0])) <= \
            1e-10 * scale
        w = z["window"]
        assert abs(plan.energy_dissipated(w[0], w[1]) - float(z["energy_dissipated_window"])) <= \
            1e-10 * scale
        t_last = arr.time[0][-1]
        assert abs(plan.energy_dissipated(t_last - 1.0 / kw["field_frequency"]) -
                   float(z["final_cycle_energy_dissipated"])) <= 1e-10 * scale
    finally:
        plan.close()


def test_oracle_reproduces_the_fixture_trajectories(oracle):
    """The fixture's trajectories are the reference's own; the oracle fed the
    reference's draws (its restatement of RngMtNorm) reproduces them bit for
    bit, which is what the GPU test relies on when it replays those draws."""
    z, kw = _gold()
    E, N, S = z["x"].shape
    steps = int(kw["end_time"] / kw["time_step"]) + 10
    for e in range(E):
        noise = oracle.mt_norm(int(z["seeds"][e]), 1.0, 3 * N * steps)
        o = oracle.full_dynamics(z["radius"], z["anisotropy"], z["axes"], z["m0"], z["location"],
                                 float(z["ms"]), float(z["damping"]), float(z["temperature"]),
                                 noise=noise, seed=int(z["seeds"][e]), **kw)
        for c in "xyz":
            assert np.array_equal(o[c], z[c][e]), (e, c)
