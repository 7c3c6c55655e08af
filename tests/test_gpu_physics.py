"""Ensemble statistics against physics known in closed form.

* Boltzmann equilibrium of a single uniaxial particle (the reference's
  docs/source/notebooks/single-particle-equilibrium.ipynb): with u = cos(theta)
  between moment and easy axis, p(u) is proportional to exp(sigma u^2) on [-1, 1],
  sigma = K V / (kB T).  Final states of independent members are binned and a
  chi-square statistic is required to stay below the 0.999 quantile.
* Neel relaxation: <m_z>(t) of members started along +z decays as exp(-t/tau)
  once the in-well relaxation (time scale tau_D) is over.  The fitted tau is
  compared with the exact relaxation time of Brown's Fokker-Planck equation
  for the polar angle (its smallest non-zero eigenvalue, computed below), to
  +-15 % (the statistical error of 4096 members over the fit window is ~5 %).
  The Neel-Brown asymptote the reference uses for its two-state model
  (lib/dom.cpp:33-59), tau_D sqrt(pi) e^sigma / (2 sigma^1.5), is 19 % below
  the exact value at sigma = 5.55 and is checked against it as a consistency
  statement of that formula's high-barrier accuracy.
"""
import numpy as np
import pytest
from scipy import stats
from scipy.linalg import eigh_tridiagonal

KB, MU0, GAMMA = 1.38064852e-23, 1.25663706e-6, 1.76086e11


def _single(E, radius, K, T, dt, end, samples, precision, seed=11):
    from magpy_gb300 import core
    seeds = np.random.default_rng(seed).integers(0, 2**31 - 1, size=E)
    return core.simulate_ensemble(E, [radius], [K], [[0, 0, 1.0]], [[0, 0, 1.0]], [[0, 0, 0.0]],
                                  4e5, 0.1, T, False, True, False, dt, end, samples, seeds,
                                  precision=precision)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_boltzmann_equilibrium_single_particle(gpu_lib, precision):
    radius, K, T = 4.5e-9, 2e4, 300.0
    V = 4 / 3 * np.pi * radius ** 3
    sigma = K * V / (KB * T)
    E = 8192 if precision == "mixed" else 4096
    arr = _single(E, radius, K, T, 5e-13, 4e-8, 3, precision)
    assert np.all(arr.status == 0)
    u = arr.mz[-1] / 4e5 / np.sqrt((arr.mx[-1] ** 2 + arr.my[-1] ** 2 + arr.mz[-1] ** 2) / 4e5 ** 2)
    edges = np.linspace(-1, 1, 21)
    counts, _ = np.histogram(u, edges)
    w = np.array([np.exp(sigma * np.linspace(a, b, 201) ** 2).mean() * (b - a)
                  for a, b in zip(edges[:-1], edges[1:])])
    expected = E * w / w.sum()
    chi2 = np.sum((counts - expected) ** 2 / expected)
    assert chi2 < stats.chi2.ppf(0.999, len(counts) - 1), (sigma, chi2, counts, expected)


def brown_tau(sigma, n=1600):
    """Exact uniaxial relaxation time in units of tau_D: 1 / (smallest non-zero
    eigenvalue) of  dW/dt = 1/(2 tau_D) d/du[(1-u^2)(dW/du - 2 sigma u W)],
    u = cos(theta) in [-1, 1], zero flux at the poles.  Finite volumes with
    Boltzmann-weighted face rates, symmetrised to a tridiagonal matrix."""
    u = np.linspace(-1, 1, n + 1)
    h = u[1] - u[0]
    phi = sigma * (0.5 * (u[1:] + u[:-1])) ** 2
    D = 1 - u[1:-1] ** 2
    kf = D / h ** 2 * np.exp((phi[1:] - phi[:-1]) / 2)
    kb = D / h ** 2 * np.exp((phi[:-1] - phi[1:]) / 2)
    diag = np.zeros(n)
    diag[:-1] -= kf
    diag[1:] -= kb
    w = eigh_tridiagonal(diag, D / h ** 2, eigvals_only=True, select="i",
                         select_range=(n - 2, n - 2))
    return 2.0 / abs(w[0])


def test_brown_tau_limits():
    # free rotational diffusion: <u> relaxes with tau_D exactly
    assert abs(brown_tau(1e-9) - 1.0) < 1e-3
    # high barrier: approaches the Neel-Brown asymptote
    s = 16.0
    asym = np.sqrt(np.pi) * np.exp(s) / (2 * s ** 1.5)
    assert 1.0 < brown_tau(s) / asym < 1.12


@pytest.mark.gpu
def test_neel_relaxation_time(gpu_lib):
    radius, K, T, alpha, Ms = 6.5e-9, 2e4, 300.0, 0.1, 4e5
    V = 4 / 3 * np.pi * radius ** 3
    sigma = K * V / (KB * T)
    tau_D = V * Ms * (1 + alpha ** 2) / (2 * GAMMA * alpha * KB * T)
    tau_N = tau_D * np.sqrt(np.pi) * np.exp(sigma) / (2 * sigma ** 1.5)  # lib/dom.cpp:33-59
    tau_B = tau_D * brown_tau(sigma)
    assert 1.1 < tau_B / tau_N < 1.3
    end = 2.0 * tau_N
    S = 81
    arr = _single(4096, radius, K, T, 5e-13, end, S, "mixed", seed=5)
    assert np.all(arr.status == 0)
    t = arr.time[0]
    mz = arr.mz.mean(axis=1) / Ms
    sel = (t > 0.2 * tau_N) & (t < 1.6 * tau_N)
    slope, _ = np.polyfit(t[sel], np.log(mz[sel]), 1)
    tau = -1.0 / slope
    assert 0.85 * tau_B < tau < 1.15 * tau_B, (sigma, tau, tau_B, tau_N)


def _metropolis_pair(sig, e, c, rhat, chains=16384, sweeps=1500, seed=3):
    """Samples of (m1, m2) from exp(-E/kT), E/kT = -sum_i sig_i (m_i.e_i)^2
    - c (3 (m1.r)(m2.r) - m1.m2): the anisotropy and dipolar energies whose
    gradients are the reference's reduced fields (lib/field.cpp:116-132,
    187-225)."""
    rng = np.random.default_rng(seed)

    def unit(v):
        return v / np.linalg.norm(v, axis=-1, keepdims=True)

    m = unit(rng.normal(size=(chains, 2, 3)))

    def energy(m):
        an = -(sig[0] * (m[:, 0] @ e[0]) ** 2 + sig[1] * (m[:, 1] @ e[1]) ** 2)
        dd = -c * (3 * (m[:, 0] @ rhat) * (m[:, 1] @ rhat) - np.sum(m[:, 0] * m[:, 1], -1))
        return an + dd

    E = energy(m)
    for sweep in range(sweeps):
        for i in (0, 1):
            trial = m.copy()
            trial[:, i] = unit(m[:, i] + 0.5 * rng.normal(size=(chains, 3)))
            Et = energy(trial)
            acc = rng.random(chains) < np.exp(np.minimum(0.0, E - Et))
            m[acc] = trial[acc]
            E[acc] = Et[acc]
    return m


@pytest.mark.gpu
def test_two_particle_equilibrium_matches_metropolis(gpu_lib):
    """Two interacting particles (the reference's
    docs/source/notebooks/two-particle-equilibrium.ipynb): the ensemble's
    final states against Metropolis samples of the Boltzmann distribution with
    the same anisotropy and dipolar energies; three observables agree within
    4 combined standard errors."""
    from magpy_gb300 import core
    r, K, T, Ms, alpha = 5e-9, 1.6e4, 300.0, 4e5, 0.1
    V = 4 / 3 * np.pi * r ** 3
    d = 2.2 * r
    rhat = np.array([0.0, 0.0, 1.0])
    axes = np.array([[0.0, 0.0, 1.0], [np.sin(0.6), 0.0, np.cos(0.6)]])
    sig = np.array([K * V / (KB * T)] * 2)
    c = MU0 * Ms ** 2 * V * V / (4 * np.pi * d ** 3) / (KB * T)
    E = 8192
    seeds = np.random.default_rng(8).integers(0, 2**31 - 1, size=E)
    arr = core.simulate_ensemble(E, [r, r], [K, K], axes, axes, [[0, 0, 0], [0, 0, d]], Ms, alpha,
                                 T, False, True, False, 5e-13, 4e-8, 2, seeds,
                                 precision="mixed")
    assert np.all(arr.status == 0)
    mm = np.stack([arr.mx[-1], arr.my[-1], arr.mz[-1]], 1).reshape(E, 2, 3) / Ms
    mm /= np.linalg.norm(mm, axis=2, keepdims=True)
    ref = _metropolis_pair(sig, axes, c, rhat)

    def observables(m):
        return np.stack([(m[:, 0] @ axes[0]) ** 2, np.sum(m[:, 0] * m[:, 1], -1),
                         (m[:, 0] @ rhat) * (m[:, 1] @ rhat)], 1)

    a, b = observables(mm), observables(ref)
    se = np.sqrt(a.var(0) / len(a) + b.var(0) / len(b))
    assert np.all(np.abs(a.mean(0) - b.mean(0)) < 4 * se), (a.mean(0), b.mean(0), se, c)
