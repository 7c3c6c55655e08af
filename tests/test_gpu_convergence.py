"""Convergence of the FP64 kernel (the reference's test/convergence recipes).

* Deterministic LLG (test/convergence/task4.cpp): a single particle with no
  anisotropy and no noise in a constant field h along z, started along x,
  follows m_x = sech(a h t) cos(h t), m_y = sech(a h t) sin(h t),
  m_z = tanh(a h t) in reduced time; the Heun scheme's error must fall as dt^2.
* Stochastic LLG (test/convergence/task5.cpp): on the same Brownian paths
  (coarse increments summed from the fine ones), the strong error of the
  final state against a path computed with dt/16 must fall at least as fast as
  dt^(1/2), the order of the Stratonovich Heun scheme for multiplicative noise.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _run(core, dt, end, noise, *, sr=0.0, k=0.0, h=0.0, alpha=0.1, m0=(1.0, 0.0, 0.0), S=2):
    return core.simulate_reduced(1, [sr], [k], [1.0], [0.0, 0.0, 1.0], list(m0), [0.0, 0.0, 0.0],
                                 [0.0], "constant", h, 0.0, 1.0, 1.0, alpha, 1.0, dt, end,
                                 noise, False, False, False, 1e-9, S)


def _sample_times(dt, end, S):
    """Reduced time of each sample's state: after k_s - 1 steps, k_s the first
    step count with k dt > s T_s (lib/simulation.cpp:342-405)."""
    Ts = end / (S - 1)
    out = [0.0]
    for s in range(1, S):
        k = 0
        while not (k * dt > s * Ts):
            k += 1
        out.append((k - 1) * dt)
    return np.array(out)


def test_deterministic_llg_closed_form(gpu_lib):
    from magpy_gb300 import core
    h, alpha, end, S = 1.0, 0.1, 2.0, 5
    errs = []
    for dt in (2e-3, 1e-3, 5e-4):
        K = core.step_count(dt, end, S)
        r = _run(core, dt, end, np.zeros(3 * K), h=h, alpha=alpha, S=S)
        assert r["status"] == 0
        t = _sample_times(dt, end, S)
        want = np.stack([np.cos(h * t) / np.cosh(alpha * h * t),
                         np.sin(h * t) / np.cosh(alpha * h * t), np.tanh(alpha * h * t)])
        got = np.stack([r["x"][0], r["y"][0], r["z"][0]])
        errs.append(np.abs(got - want).max())
    assert errs[1] < 1e-5, errs
    for a, b in zip(errs, errs[1:]):
        assert 3.0 < a / b < 5.0, errs  # second order


def test_stochastic_llg_strong_order(gpu_lib):
    from magpy_gb300 import core
    rng = np.random.default_rng(55)
    end, sr, k, alpha = 1.0, 0.3, 1.0, 0.1
    fine = 2.0 ** -12
    levels = [2.0 ** -8, 2.0 ** -9, 2.0 ** -10]
    paths = 96
    errs = np.zeros(len(levels))
    for _ in range(paths):
        Kf = core.step_count(fine, end, 2)
        w = rng.normal(size=(Kf, 3))
        ref = _run(core, fine, end, w.ravel(), sr=sr, k=k, alpha=alpha, m0=(0.6, 0.0, 0.8))
        mref = np.array([ref["x"][0, -1], ref["y"][0, -1], ref["z"][0, -1]])
        for i, dt in enumerate(levels):
            r = int(round(dt / fine))
            Kc = core.step_count(dt, end, 2)
            # the coarse increment is the sum of r fine ones (standard normals
            # scaled by sqrt(dt) inside the step): (w_1 + ... + w_r) / sqrt(r)
            wc = np.zeros((Kc, 3))
            full = (Kf - 1) // r
            wc[:full] = w[:full * r].reshape(full, r, 3).sum(axis=1) / np.sqrt(r)
            c = _run(core, dt, end, wc.ravel(), sr=sr, k=k, alpha=alpha, m0=(0.6, 0.0, 0.8))
            m = np.array([c["x"][0, -1], c["y"][0, -1], c["z"][0, -1]])
            errs[i] += np.linalg.norm(m - mref) / paths
    slope = np.polyfit(np.log(levels), np.log(errs), 1)[0]
    assert 0.4 < slope < 1.6, (slope, errs)
    assert np.all(np.diff(errs) < 0), errs
