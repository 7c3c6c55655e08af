"""The oracle against the reference's own known answers (test/tests.cpp)."""
import math

import numpy as np
import pytest

from oracle.pyoracle import FJ_CB, SDE_CB, SDE_JAC_CB

MU0 = 1.25663706e-6


def test_constants(oracle):
    # include/constants.hpp:10-12
    assert oracle.lib.oracle_const_kb() == 1.38064852e-23
    assert oracle.lib.oracle_const_mu0() == 1.25663706e-6
    assert oracle.lib.oracle_const_gyromag() == 1.76086e11


def test_llg_drift(oracle):  # tests.cpp:23-34
    d = oracle.drift([2, 3, 4], 3, [1, 2, 3])
    assert list(d) == [-34, -4, 20]


def test_llg_diffusion(oracle):  # tests.cpp:36-52
    b = oracle.diffusion([2, 3, 4], 2, 3)
    assert list(b) == [150, -28, -54, -44, 120, -68, -42, -76, 78]


def test_llg_drift_jacobian(oracle):  # tests.cpp:94-114
    j = oracle.drift_jacobian([1.0, 1.2, 2.2], 0.1, [6.7, 13.4, 10.05],
                              [1.0, 2.0, 1.5, 2.0, 4.0, 3.0, 1.5, 3.0, 2.25])
    want = [-1.161, -4.466, 19.33, 11.878, -2.977, -2.082, -14.046, 3.8, -4.051]
    for k, (a, b) in enumerate(zip(j, want)):
        if k == 5:
            assert abs(a - b) <= 1e-10
        else:
            assert a == pytest.approx(b, rel=4 * 2.2e-16, abs=0)


def test_uniaxial(oracle):  # tests.cpp:117-127
    h = np.zeros(3)
    from oracle.pyoracle import _d, _f64
    oracle.lib.oracle_uniaxial_anisotropy(_d(h), _d(_f64([1.0, 1.2, 2.2])), _d(_f64([1.0, 2.0, 1.5])))
    assert h == pytest.approx([6.7, 13.4, 10.05], rel=4e-16)


def test_uniaxial_jacobian(oracle):  # tests.cpp:132-146
    from oracle.pyoracle import _d, _f64
    j = np.zeros(9)
    oracle.lib.oracle_uniaxial_anisotropy_jacobian(_d(j), _d(_f64([1.0, 2.0, 1.5])))
    assert list(j) == [1.0, 2.0, 1.5, 2.0, 4.0, 3.0, 1.5, 3.0, 2.25]


def test_multi_uniaxial_jacobian(oracle):  # tests.cpp:842-904
    from oracle.pyoracle import _d, _f64
    jac = np.zeros(81)
    oracle.lib.oracle_multi_add_uniaxial_anisotropy_jacobian(
        _d(jac), _d(_f64([1, 2, 3, 4, 5, 6, 4, 2, 3])), _d(_f64([3.2, 5.2, 1.2])), 3)
    res = jac.reshape(9, 9)
    mask = np.kron(np.eye(3), np.ones((3, 3))) == 0
    assert np.all(res[mask] == 0)
    assert np.allclose(res[:3, :3], [[3.2, 6.4, 9.6], [6.4, 12.8, 19.2], [9.6, 19.2, 28.8]], rtol=1e-15, atol=0)
    assert np.allclose(res[3:6, 3:6], [[83.2, 104, 124.8], [104, 130, 156], [124.8, 156, 187.2]], rtol=1e-15, atol=0)
    assert np.allclose(res[6:, 6:], [[19.2, 9.6, 14.4], [9.6, 4.8, 7.2], [14.4, 7.2, 10.8]], rtol=1e-15, atol=0)


def test_heun_multiplicative(oracle):  # tests.cpp:148-181
    def sde(drift, diff, x, t, ctx):
        drift[0] = x[0] * x[1] * t
        drift[1] = 3 * x[0]
        diff[0] = t; diff[1] = x[0]; diff[2] = x[1]; diff[3] = x[1]; diff[4] = 4.0
        diff[5] = x[0] * x[1]
    cb = SDE_CB(sde)
    from oracle.pyoracle import _d, _f64
    dt = 0.1
    w = _f64([0.1, 0.01, 0.001]) / math.sqrt(dt)
    nxt = np.zeros(2)
    oracle.lib.oracle_heun_dense(_d(nxt), _d(_f64([1, 2])), _d(w), cb, None, 2, 3, 0.0, dt)
    assert nxt[0] == pytest.approx(1.03019352, rel=4 * 2.2e-16)
    assert nxt[1] == pytest.approx(2.571186252, rel=4 * 2.2e-16)


def test_heun_driver_ou(oracle):  # tests.cpp:183-227
    theta, mu, sigma = 10.0, -1.0, 0.8
    def sde(drift, diff, x, t, ctx):
        drift[0] = theta * (mu - x[0])
        diff[0] = sigma
    cb = SDE_CB(sde)
    n, dt = 5000, 1e-5
    w = oracle.mt_norm(1001, 1.0, n)
    from oracle.pyoracle import _d, _f64
    states = np.zeros(n + 1)
    oracle.lib.oracle_heun_driver(_d(states), _d(_f64([-3.0])), _d(w), cb, None, n, 1, 1, dt)
    true = -3.0
    for i in range(1, n + 1):
        true = (true * math.exp(-theta * dt) + mu * (1 - math.exp(-theta * dt)) +
                sigma * math.sqrt((1 - math.exp(-2 * theta * dt)) / (2 * theta)) * w[i - 1])
        assert abs(true - states[i]) <= 1e-8


def _newton_fj(sing=False):
    def fj(f, j, x, ctx):
        f[0] = -(x[0] - 2) * (x[0] - 2) - 2 * x[0] * x[1]
        if sing:
            f[1] = 2.0 * f[0]
            j[0] = -2 * x[0] - 2 * x[1] + 4; j[1] = -2 * x[0]
            j[2] = 2.0 * j[0]; j[3] = 2.0 * j[1]
        else:
            f[1] = -x[1] * (x[0] + 1) - 4 * x[1]
            j[0] = -2 * x[0] - 2 * x[1] + 4; j[1] = -2 * x[0]; j[2] = -x[1]; j[3] = -x[0] - 5
    return FJ_CB(fj)


def test_newton_two_solutions(oracle):  # tests.cpp:270-313
    import ctypes as C
    from oracle.pyoracle import _d, _f64
    cb = _newton_fj()
    x = np.zeros(2)
    info = C.c_int64(0)
    flag = oracle.lib.oracle_newton_noinv(_d(x), cb, None, _d(_f64([-5.2, -5.2])), 2, 1e-10, 100, C.byref(info))
    assert flag == 0
    tol = math.sqrt(2 * 5.2 * 5.2) * 1e-10
    assert abs(x[0] + 5) <= tol and abs(x[1] - 4.9) <= tol
    flag = oracle.lib.oracle_newton_noinv(_d(x), cb, None, _d(_f64([1.0, 1.0])), 2, 1e-10, 100, C.byref(info))
    assert flag == 0
    tol = math.sqrt(2.0) * 1e-10
    assert abs(x[0] - 2) <= tol and abs(x[1]) <= tol


def test_newton_singular(oracle):  # tests.cpp:315-344
    import ctypes as C
    from oracle.pyoracle import _d, _f64
    cb = _newton_fj(sing=True)
    x = np.zeros(2)
    info = C.c_int64(0)
    flag = oracle.lib.oracle_newton_noinv(_d(x), cb, None, _d(_f64([-5.2, -5.2])), 2, 1e-8, 100, C.byref(info))
    assert flag == 2 and info.value >= 0


def test_rng_mt_norm(oracle):  # tests.cpp:346-355
    v = oracle.mt_norm(999, 0.2, 5)
    want = [0.27100401702487437, -0.18950297511996847, -0.27620532277321042,
            -0.10214651921310165, -0.19125423381292103]
    for a, b in zip(v, want):
        assert a == pytest.approx(b, rel=4 * 2.2e-16)


def _stiff_sde(a=0.1, b=5.0):
    def sde(aout, bout, adash, bdash, x, ta, tb, ctx):
        aout[0] = a * (x[1] - x[0]) - 0.5 * b * b * x[0]
        aout[1] = a * (x[0] - x[1]) - 0.5 * b * b * x[1]
        adash[0] = -a - 0.5 * b * b; adash[1] = a; adash[2] = a; adash[3] = -a - 0.5 * b * b
        bout[0] = b * x[0]; bout[1] = b * x[1]
        bdash[0] = b; bdash[1] = 0; bdash[2] = 0; bdash[3] = b
    return SDE_JAC_CB(sde)


def test_implicit_midpoint_stiff(oracle):  # tests.cpp:434-481
    from oracle.pyoracle import _d, _f64
    cb = _stiff_sde()
    x = np.zeros(2)
    rc = oracle.lib.oracle_implicit_midpoint_dense(_d(x), _d(_f64([1.0, 2.0])), _d(_f64([0.25])),
                                                   cb, None, 2, 1, 0.0, 1e-4, 1e-6, 100)
    assert rc == 0
    assert abs(x[0] - 1.01132363) <= 5e-4 and abs(x[1] - 2.02261693) <= 5e-4


def test_implicit_driver_stiff(oracle):  # tests.cpp:483-539
    from oracle.pyoracle import _d, _f64, _i32p
    a, b, N, dt = 0.1, 5.0, 100, 1e-4
    cb = _stiff_sde(a, b)
    dw = oracle.mt_norm(1001, 1.0, N)
    Wt = np.concatenate([[0.0], np.cumsum(dw[:-1])])
    x = np.zeros(2 * N)
    codes = np.zeros(N - 1, dtype=np.int32)
    oracle.lib.oracle_implicit_driver(_d(x), _d(_f64([1.0, 2.0])), _d(dw), cb, None, 2, 1,
                                      N - 1, 0.0, dt, 1e-6, 500, codes.ctypes.data_as(_i32p))
    for i in range(1, N):
        rp = -0.5 * b * b * i * dt + b * Wt[i] * math.sqrt(dt)
        rm = (-2 * a - 0.5 * b * b) * i * dt + b * Wt[i] * math.sqrt(dt)
        on, off = math.exp(rp) + math.exp(rm), math.exp(rp) - math.exp(rm)
        assert abs(0.5 * (on * 1.0 + off * 2.0) - x[2 * i]) <= 0.002
        assert abs(0.5 * (off * 1.0 + on * 2.0) - x[2 * i + 1]) <= 0.002


def test_dom_transition_matrix(oracle):  # tests.cpp:609-620
    W = oracle.transition_matrix(1, 2e-21, 10, 0.5, 2.7, 0.1)
    want = [-0.00021827108536028533, 278104386.1896516, 0.00021827108536028533, -278104386.1896516]
    for a, b in zip(W, want):
        assert a == pytest.approx(b, rel=4 * 2.2e-16)


def test_dipolar_two_particles(oracle):  # tests.cpp:622-643
    ms = 1.0 / math.sqrt(MU0)
    f = oracle.multi_add_dipolar(np.zeros(6), ms, 0.5, [15 / 16, 17 / 16], [1, 0, 0, 0, 0, 1],
                                 [0, 0, 0, -0.5, 0, math.sqrt(3) / 2, 0.5, 0, -math.sqrt(3) / 2, 0, 0, 0],
                                 [0, 1, 1, 0])
    want = [-0.10983505338481014402, 0, 0.10568882939696175316, -0.01865096989358148646, 0,
            -0.09691328239836190239]
    for a, b in zip(f, want):
        assert a == pytest.approx(b, rel=4 * 2.2e-16, abs=0)


@pytest.mark.parametrize("r1,r2,k1,k2", [(2.5e-9, 2.5e-9, 6.33e4, 6.33e4), (2.5e-9, 3.0e-9, 5e4, 7e4)])
def test_dipolar_aligned_closed_form(oracle, r1, r2, k1, k2):  # tests.cpp:645-806
    v1, v2 = 4 / 3 * math.pi * r1 ** 3, 4 / 3 * math.pi * r2 ** 3
    vav, kav = 0.5 * (v1 + v2), 0.5 * (k1 + k2)
    R = 2.917e-9
    Rr = R / vav ** (1 / 3)
    ms = 400e3
    dists = [0, 0, 0, 0, 0, 1, 0, 0, -1, 0, 0, 0]
    cubes = [0, Rr ** 3, Rr ** 3, 0]
    Hk = 2 * kav / MU0 / ms
    rng = np.random.default_rng(0)
    for mag in ([1, 0, 0, 1, 0, 0], [0, 0, 1, 0, 0, 1], list(rng.normal(size=6))):
        f = oracle.multi_add_dipolar(np.zeros(6), ms, kav, [v1 / vav, v2 / vav], mag, dists, cubes)
        c1 = v2 * ms / (4 * math.pi * R ** 3)
        c2 = v1 * ms / (4 * math.pi * R ** 3)
        want = [c1 * -mag[3] / Hk, c1 * -mag[4] / Hk, c1 * 2 * mag[5] / Hk,
                c2 * -mag[0] / Hk, c2 * -mag[1] / Hk, c2 * 2 * mag[2] / Hk]
        assert np.allclose(f, want, rtol=0, atol=1e-14)


def test_dipolar_prefactor_and_p2p(oracle):  # tests.cpp:808-838
    from oracle.pyoracle import _d, _f64
    assert oracle.lib.oracle_dipolar_prefactor(1 / math.sqrt(MU0), 0.5) == pytest.approx(
        0.07957747154594767280, rel=4 * 2.2e-16)
    out = _f64([1.0, 1.5, 2.0]).copy()
    oracle.lib.oracle_dipolar_p2p(_d(out), 2.3, 1.2, _d(_f64([0.7, 0.2, 0.4])),
                                  _d(_f64([1.2, 1.1, 1.3])), 3.7)
    assert out == pytest.approx([36.37323333333333333333, 37.05761666666666666667,
                                 42.86218333333333333333], rel=4 * 2.2e-16)


def test_applied_field_and_waveforms(oracle):  # tests.cpp:826-840, field.cpp:23-54
    f = oracle.lib.oracle_field_value
    assert f(2, 3.0, 0.7, 9.0) == 0.7
    assert f(0, 0.1, 2.0, 1.5) == 2.0 * math.sin(2 * math.pi * 1.5 * 0.1)
    assert f(1, 0.1, 2.0, 1.5) == 2.0 and f(1, 0.4, 2.0, 1.5) == -2.0


def test_pairwise_geometry(oracle):  # tests.cpp:906-980
    from oracle.pyoracle import _d, _f64
    pts = _f64([[0, 0, 1], [3, 1, 0], [0.5, 0.5, 0.5]])
    vec, mag, unit = np.zeros((3, 3, 3)), np.zeros((3, 3)), np.zeros((3, 3, 3))
    oracle.lib.oracle_pairwise_geometry(_d(pts), 3, _d(vec), _d(mag), _d(unit))
    assert list(vec[0, 1]) == [3, 1, -1] and list(vec[1, 0]) == [-3, -1, 1]
    assert list(vec[1, 2]) == [-2.5, -0.5, 0.5] and list(vec[2, 1]) == [2.5, 0.5, -0.5]
    assert np.all(np.diag(mag) == 0)
    assert mag[0, 1] == pytest.approx(math.sqrt(11), rel=4e-16)
    assert unit[0, 1] == pytest.approx(vec[0, 1] / math.sqrt(11), rel=4e-16)


def test_nrm2_and_dgesv(oracle):
    x = np.array([3.0, 4.0, 12.0, 0.0, 0.0])
    assert oracle.nrm2(x) == 13.0
    rng = np.random.default_rng(3)
    A = rng.normal(size=(5, 5)) + 5 * np.eye(5)
    b = rng.normal(size=5)
    info, sol = oracle.dgesv(A, b)
    assert info == 0 and np.allclose(A @ sol, b, rtol=0, atol=1e-12)
    info, _ = oracle.dgesv(np.array([[1.0, 2.0], [2.0, 4.0]]), np.array([1.0, 1.0]))
    assert info == 2
