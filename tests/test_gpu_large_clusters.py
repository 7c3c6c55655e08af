"""Large clusters: the FP64 kernel beyond one warp-CTA's register budget and
the mixed-precision implicit-midpoint mode (FP64 Newton, FP32 dipolar sum).

* FP64 kernel, n = 600 (CTAs of 608 threads), Heun and implicit: bit for bit
  equal to the oracle on injected increments.
* Mixed Heun, n = 700 (CTAs above 640 threads use the 64-register variant):
  strong error against the oracle <= 1e-5.
* Mixed implicit, n = 64 and 512: strong error against the FP64 kernel on
  the same in-kernel increments <= 1e-5 (the stated bound), and Newton
  converges for every member.
"""
import numpy as np
import pytest

from test_gpu_parity import _assert_close, _gpu_reduced

pytestmark = pytest.mark.gpu


def _sphere_cluster(n, seed):
    rng = np.random.default_rng(seed)
    radius = 8e-9 * np.exp(0.2 * rng.normal(size=n))
    R = 1.1 * radius.mean() * (n / 0.3) ** (1 / 3)
    pts = []
    while len(pts) < n:
        p = rng.uniform(-R, R, 3)
        if p @ p > R * R:
            continue
        if all(np.linalg.norm(p - q) >= 2.2 * radius.mean() for q in pts):
            pts.append(p)
    axes = rng.normal(size=(n, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    return radius, np.array(pts), axes


@pytest.mark.parametrize("implicit", [False, True])
def test_fp64_kernel_n600_matches_oracle(gpu_lib, oracle, implicit):
    from magpy_gb300 import core
    from oracle.pyoracle import reduced_inputs
    n = 600
    rng = np.random.default_rng(600 + implicit)
    inp = reduced_inputs(rng, n)
    dt, end, S = 1.3e-3, 0.02, 4
    K = core.step_count(dt, end, S)
    noise = rng.normal(size=K * 3 * n)
    kw = dict(field_shape="sine", happ=0.3, fapp=3.0, dt=dt, end_time=end, max_samples=S,
              use_implicit=implicit, renorm=False, interactions=True)
    a = _gpu_reduced(core, inp, kw, noise)
    b = oracle.full_dynamics_reduced(inp, noise=noise, **kw)
    assert a["status"] == b["status"] == 0
    _assert_close(a, b, exact=False, rtol=1e-12)  # sine field: device sin within 2 ulp


def test_mixed_heun_n700(gpu_lib, oracle):
    from magpy_gb300 import core
    from oracle.pyoracle import reduced_inputs
    n = 700
    rng = np.random.default_rng(700)
    inp = reduced_inputs(rng, n)
    dt, end, S = 1.3e-3, 0.02, 3
    K = core.step_count(dt, end, S)
    noise = rng.normal(size=K * 3 * n)
    kw = dict(field_shape="constant", happ=0.2, dt=dt, end_time=end, max_samples=S,
              use_implicit=False, renorm=False, interactions=True)
    a = _gpu_reduced(core, inp, kw, noise, precision="mixed")
    b = oracle.full_dynamics_reduced(inp, noise=noise, **kw)
    assert a["status"] == 0
    m_a = np.stack([a["x"][:, -1], a["y"][:, -1], a["z"][:, -1]], 1)
    m_b = np.stack([b["x"][:, -1], b["y"][:, -1], b["z"][:, -1]], 1)
    err = np.linalg.norm(m_a - m_b, axis=1) / np.linalg.norm(m_b, axis=1)
    assert err.max() < 1e-5, err.max()


@pytest.mark.parametrize("n,E,steps", [(64, 8, 200), (512, 4, 40)])
def test_mixed_implicit_strong_error(gpu_lib, n, E, steps):
    from magpy_gb300 import core
    radius, loc, axes = _sphere_cluster(n, n)
    dt = 2e-13
    seeds = np.arange(E) + 11
    args = (E, radius, np.full(n, 2e4), axes, axes.copy(), loc, 4e5, 0.01, 300.0, False, True,
            True, dt, dt * (steps - 0.5), 3, seeds, "sine", 1e4, 3e5, 1e-9)
    a64 = core.simulate_ensemble(*args, precision="fp64")
    amx = core.simulate_ensemble(*args, precision="mixed")
    assert np.all(a64.status == 0) and np.all(amx.status == 0)
    assert np.all(amx.steps == a64.steps)
    m64 = np.stack([a64.mx[-1], a64.my[-1], a64.mz[-1]], 1)
    mmx = np.stack([amx.mx[-1], amx.my[-1], amx.mz[-1]], 1)
    err = np.linalg.norm(mmx - m64, axis=1) / np.linalg.norm(m64, axis=1)
    assert err.max() < 1e-5, err.max()
    assert err.max() > 0.0  # the dipolar sum really ran in FP32


@pytest.mark.parametrize("mpc", [2, 4])
def test_mixed_members_per_cta(gpu_lib, mpc):
    """Several members per CTA (clusters of more than 32 particles sharing one
    cluster): the same results as one member per CTA to FP32 rounding, and
    strong error <= 1e-5 against the FP64 kernel; E not a multiple of the
    members per CTA."""
    from magpy_gb300 import core
    n, E, steps = 100, 7, 300
    radius, loc, axes = _sphere_cluster(n, 3)
    dt = 5e-14
    args = (E, radius, np.full(n, 2e4), axes, axes.copy(), loc, 4e5, 0.1, 300.0, False, True,
            False, dt, dt * steps, 4, np.arange(E) + 21, "sine", 1e4, 3e5)
    ref = core.EnsemblePlan(*args, precision="fp64").run().arrays()
    one = core.EnsemblePlan(*args, precision="mixed").run().arrays()
    multi = core.EnsemblePlan(*args, precision="mixed").set_launch(4, mpc).run().arrays()
    assert np.all(multi.status == 0) and np.array_equal(multi.steps, ref.steps)
    for m in (one, multi):
        f = np.stack([m.mx[-1], m.my[-1], m.mz[-1]], 1)
        r = np.stack([ref.mx[-1], ref.my[-1], ref.mz[-1]], 1)
        err = np.linalg.norm(f - r, axis=1) / np.linalg.norm(r, axis=1)
        assert err.max() < 1e-5, err.max()
    np.testing.assert_allclose(multi.mz, one.mz, rtol=0, atol=1e-5 * 4e5)
    np.testing.assert_array_equal(multi.time, ref.time)
