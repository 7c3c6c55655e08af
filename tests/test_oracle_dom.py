"""The two-state master-equation oracle (oracle/dom_oracle.cpp).

* The known answers of test/tests.cpp: rk45 time_dependent_step (:566-590,
  ASSERT_DOUBLE_EQ = 4 ulp) and master_equation 3d_system (:592-603).
* simulation::dom_ensemble_dynamics of the compiled reference, bit for bit,
  for every field shape the DOModel offers (magpy/model.py:211-295).
"""
import numpy as np
import pytest

KB, MU0 = 1.38064852e-23, 1.25663706e-6


def _ulps(a, b):
    a, b = np.float64(a), np.float64(b)
    return abs(int(a.view(np.int64)) - int(b.view(np.int64)))


def test_rk45_known_answers(oracle):  # tests.cpp:566-590
    x2, k, h, t = oracle.rk45_tests_ode([1.0, 2.0], 0.01, 0.5, 1e-4)
    expect_k = [(1.0, -6.0), (0.997976, -6.002), (0.9969437365, -6.002995446),
                (0.993774919651888, -6.005981540838), (0.9893745618215710, -6.009947940975117),
                (0.99077120433373344621, -6.00871032589945830438)]
    for got, want in zip(k, expect_k):
        for g, w in zip(got, want):
            assert _ulps(g, w) <= 4, (g, w)
    assert _ulps(x2[0], 1.00994791563354557873) <= 4
    assert _ulps(x2[1], 1.93995017187702467609) <= 4
    assert t == 0.5 + 0.01  # the step was accepted at the given size


def test_rk45_matches_reference(oracle, reference):
    for x1, h, t, tol in [([1.0, 2.0], 0.01, 0.5, 1e-4), ([0.3, -2.0], 0.5, 0.0, 1e-9),
                          ([5.0, 1.0], 2.0, 3.0, 1e-2)]:
        a = oracle.rk45_tests_ode(x1, h, t, tol)
        b = reference.rk45_tests_ode(x1, h, t, tol)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
        assert a[2] == b[2] and a[3] == b[3]


def test_master_equation_known_answer(oracle):  # tests.cpp:592-603
    y = oracle.master_equation(np.arange(1.0, 10.0), [3.0, 2.0, 1.0])
    np.testing.assert_array_equal(y, [10.0, 28.0, 46.0])


CASES = [
    # volume, K, T, Ms, alpha, shape, H0 (A/m), f (Hz), ncomp, p0, dt, end, samples
    (4 / 3 * np.pi * 9e-9 ** 3, 2e4, 300.0, 4e5, 0.1, "sine", 5e3, 2e5, 1, (1.0, 0.0),
     1e-10, 2e-5, 201),
    (4 / 3 * np.pi * 8e-9 ** 3, 2e4, 300.0, 4e5, 0.1, "square", 4e3, 1e5, 1, (0.5, 0.5),
     1e-10, 3e-5, 101),
    (4 / 3 * np.pi * 10e-9 ** 3, 1.5e4, 310.0, 4.5e5, 0.05, "constant", 2e3, 0.0, 1,
     (0.2, 0.8), 1e-9, 1e-5, 51),
    (4 / 3 * np.pi * 9e-9 ** 3, 2e4, 300.0, 4e5, 0.1, "square_f", 5e3, 2e5, 5, (1.0, 0.0),
     1e-10, 2e-5, 201),
    (4 / 3 * np.pi * 9e-9 ** 3, 2e4, 300.0, 4e5, 0.1, "sine", 5e3, 2e5, 1, (1.0, 0.0),
     2e-7, 2e-5, -1),
]


def _hk(K, Ms):
    return 2.0 * K / MU0 / Ms  # magpy/core.pyx:226


@pytest.mark.parametrize("case", range(len(CASES)))
def test_dom_dynamics_matches_reference(oracle, reference, case):
    v, K, T, Ms, a, shape, H0, f, nc, p0, dt, end, S = CASES[case]
    h = H0 / _hk(K, Ms)
    o = oracle.dom_dynamics(v, K, T, Ms, a, shape, h, f, nc, p0, dt, end, S)
    r = reference.dom_dynamics(v, K, T, Ms, a, shape, h, f, nc, p0, dt, end, S)
    assert o["status"] == 0
    for key in ("mz", "field", "time"):
        np.testing.assert_array_equal(o[key], r[key])
    assert o["steps"] > 10


def test_dom_batch_is_per_member_dynamics(oracle):
    v, K, T, Ms, a, shape, H0, f, nc, p0, dt, end, S = CASES[0]
    vols = v * np.array([0.8, 1.0, 1.3])
    b = oracle.dom_batch(vols, K, T, Ms, a, p0, shape, H0, f, nc, dt, end, S)
    for e, ve in enumerate(vols):
        o = oracle.dom_dynamics(ve, K, T, Ms, a, shape, H0 / _hk(K, Ms), f, nc, p0, dt, end, S)
        np.testing.assert_array_equal(b["mz"][e], o["mz"])
        np.testing.assert_array_equal(b["field"][e], o["field"] * _hk(K, Ms))
        assert b["steps"][e] == o["steps"]


def test_dom_step_limit_is_reported(oracle):
    v, K, T, Ms, a, shape, H0, f, nc, p0, dt, end, S = CASES[0]
    o = oracle.dom_dynamics(v, K, T, Ms, a, shape, H0 / _hk(K, Ms), f, nc, p0, dt, end, S,
                            max_steps=50)
    assert o["status"] == 32 and o["steps"] == 50
    assert np.isnan(o["mz"][-1]) and np.isfinite(o["mz"][0])


def test_dom_relaxes_to_two_state_equilibrium(oracle):
    # constant field, dp/dt = W p with W = [[-r2, r1], [r2, -r1]] (lib/dom.cpp:55-56):
    # p -> (r1, r2) / (r1 + r2), so mz = p0 - p1 -> (r1 - r2) / (r1 + r2)
    v, K, T, Ms, a = 4 / 3 * np.pi * 7e-9 ** 3, 2e4, 300.0, 4e5, 0.1
    h = 2e3 / _hk(K, Ms)
    W = oracle.transition_matrix(K, v, T, h, Ms, a)
    r1, r2 = W[1], W[2]
    tau = 1.0 / (r1 + r2)
    o = oracle.dom_dynamics(v, K, T, Ms, a, "constant", h, 0.0, 1, (0.0, 1.0), tau * 1e-4,
                            8 * tau, 41)
    assert o["status"] == 0
    assert abs(o["mz"][-1] - (r1 - r2) / (r1 + r2)) < 1e-3
