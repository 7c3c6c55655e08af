"""Pathwise adjoint gradients against central finite differences.

The finite differences run the FP64 oracle (the reference's algorithm) at
theta +- h, h = 1e-4 relative, on the same increments the in-kernel generator
produced for the adjoint's forward run; the adjoint runs on the mixed-precision
trajectory.  Stated agreement: 1e-3 relative.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MU0 = 1.25663706e-6


def _cfg(n=8, E=32, steps=1200, f=5e9, H0=1e4):
    side = int(np.ceil(n ** (1 / 3)))
    grid = np.stack(np.meshgrid(*[np.arange(side)] * 3, indexing="ij"), -1).reshape(-1, 3)[:n]
    rng = np.random.default_rng(n)
    axes = rng.normal(size=(n, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    dt = 5e-14
    return dict(n_members=E, radius=np.full(n, 8e-9), anisotropy_axis=axes,
                magnetisation_direction=axes.copy(), location=grid * 20e-9, magnetisation=4e5,
                temperature=300.0, time_step=dt, end_time=dt * (steps - 0.5), max_samples=11,
                seeds=rng.integers(0, 2**31 - 1, size=E), field_shape="sine",
                field_frequency=f, H0=H0, K=2e4, alpha=0.1)


def _objectives(field, M):
    sar = -MU0 * np.sum((M[1:] - M[:-1]) * (field[1:] + field[:-1]) / 2.0)
    return np.array([sar, M[-1]])


def _oracle_J(oracle, cfg, noise, K, alpha, H0):
    n = cfg["radius"].size
    out = oracle.ensemble(cfg["seeds"], cfg["radius"], np.full(n, K), cfg["anisotropy_axis"],
                          cfg["magnetisation_direction"], cfg["location"], cfg["magnetisation"],
                          alpha, cfg["temperature"], interactions=True, use_implicit=False,
                          time_step=cfg["time_step"], end_time=cfg["end_time"],
                          max_samples=cfg["max_samples"], field_shape="sine",
                          field_amplitude=H0, field_frequency=cfg["field_frequency"],
                          noise=noise)
    assert np.all(out["status"] == 0)
    M = out["z"].sum(axis=1).mean(axis=0)
    return _objectives(out["field"], M)


def test_adjoint_matches_oracle_finite_differences(gpu_lib, oracle):
    from magpy_gb300 import core
    from magpy_gb300.adjoint import EnsembleAdjoint, sar_grad_M
    cfg = _cfg()
    n = cfg["radius"].size
    adj = EnsembleAdjoint(cfg["n_members"], cfg["radius"], np.full(n, cfg["K"]),
                          cfg["anisotropy_axis"], cfg["magnetisation_direction"],
                          cfg["location"], cfg["magnetisation"], cfg["alpha"],
                          cfg["temperature"], cfg["time_step"], cfg["end_time"],
                          cfg["max_samples"], cfg["seeds"], "sine", cfg["H0"],
                          cfg["field_frequency"], True, checkpoint_every=256)
    t, field, M = adj.forward()
    assert np.all(adj.status == 0)
    steps = adj.plan.max_steps
    noise = np.concatenate([core.wiener_increments(int(s), n, steps).ravel()
                            for s in cfg["seeds"]])
    J0 = _oracle_J(oracle, cfg, noise, cfg["K"], cfg["alpha"], cfg["H0"])
    # the mixed forward reproduces the FP64 objectives
    np.testing.assert_allclose(_objectives(field, M), J0, rtol=1e-5, atol=1e-6 * abs(J0).max())
    g_sar, _ = adj.backward(sar_grad_M(field))
    g_sar[2] += _objectives(field, M)[0] / cfg["H0"]  # direct field dependence of the SAR
    dM = np.zeros_like(M)
    dM[-1] = 1.0
    g_mz, _ = adj.backward(dM)
    adj.close()
    names = ("K", "alpha", "H0")
    for i, name in enumerate(names):
        th = [cfg["K"], cfg["alpha"], cfg["H0"]]
        h = 1e-4 * th[i]
        tp, tm = list(th), list(th)
        tp[i] += h
        tm[i] -= h
        fd = (_oracle_J(oracle, cfg, noise, *tp) - _oracle_J(oracle, cfg, noise, *tm)) / (2 * h)
        for k, (g, label) in enumerate(((g_sar, "SAR"), (g_mz, "M_T"))):
            rel = abs(g[i] - fd[k]) / max(abs(fd[k]), 1e-30)
            assert rel < 1e-3, (label, name, g[i], fd[k], rel)


def test_autograd_function(gpu_lib):
    torch = pytest.importorskip("torch")
    from magpy_gb300.adjoint import EnsembleAdjoint, sar_and_mz, sar_grad_M
    cfg = _cfg(n=4, E=16, steps=600)
    K = torch.tensor(cfg["K"], dtype=torch.float64, requires_grad=True)
    a = torch.tensor(cfg["alpha"], dtype=torch.float64, requires_grad=True)
    H0 = torch.tensor(cfg["H0"], dtype=torch.float64, requires_grad=True)
    c = {k: v for k, v in cfg.items() if k not in ("K", "alpha", "H0")}
    c["checkpoint_every"] = 100
    out = sar_and_mz(K, a, H0, c)
    (2.0 * out[0] + 3.0 * out[1]).backward()
    # the same through the explicit adjoint
    n = cfg["radius"].size
    adj = EnsembleAdjoint(cfg["n_members"], cfg["radius"], np.full(n, cfg["K"]),
                          cfg["anisotropy_axis"], cfg["magnetisation_direction"],
                          cfg["location"], cfg["magnetisation"], cfg["alpha"],
                          cfg["temperature"], cfg["time_step"], cfg["end_time"],
                          cfg["max_samples"], cfg["seeds"], "sine", cfg["H0"],
                          cfg["field_frequency"], True, checkpoint_every=100)
    t, field, M = adj.forward()
    dJ = 2.0 * sar_grad_M(field)
    dJ[-1] += 3.0
    g, _ = adj.backward(dJ)
    sar = -MU0 * np.sum((M[1:] - M[:-1]) * (field[1:] + field[:-1]) / 2.0)
    g[2] += 2.0 * sar / cfg["H0"]
    adj.close()
    np.testing.assert_allclose([K.grad.item(), a.grad.item(), H0.grad.item()], g, rtol=1e-12)
    assert out.shape == (2,)
