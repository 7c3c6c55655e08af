"""The oracle against golden fixtures produced by the reference itself
(tests/golden/make_golden.py) and, where the compiled reference is present
(oracle/_ref), against live runs of it."""
import os

import numpy as np
import pytest

from conftest import golden_files, load_reduced_case

FIELDS = ("x", "y", "z", "field", "time")


@pytest.mark.parametrize("path", golden_files("reduced_"), ids=os.path.basename)
def test_oracle_reduced_matches_reference_fixture_bitwise(oracle, path):
    inp, kw, z = load_reduced_case(path)
    out = oracle.full_dynamics_reduced(inp, noise=z["noise"], **kw)
    assert out["status"] == 0
    for k in FIELDS:
        assert np.array_equal(out[k], z[k]), k


@pytest.mark.parametrize("path", golden_files("physical_"), ids=os.path.basename)
def test_oracle_physical_matches_reference_fixture_bitwise(oracle, path):
    z = np.load(path)
    kw = {k[3:]: z[k].item() for k in z.files if k.startswith("kw_")}
    out = oracle.full_dynamics(z["radius"], z["anisotropy"], z["axes"], z["m0"], z["location"],
                               float(z["ms"]), float(z["damping"]), float(z["temperature"]), **kw)
    for k in FIELDS:
        assert np.array_equal(out[k], z[k]), k


def test_oracle_components_match_reference_fixture(oracle):
    z = np.load(golden_files("components")[0])
    for i in range(z["m"].shape[0]):
        assert np.array_equal(oracle.drift(z["m"][i], z["alpha"][i], z["h"][i]), z["drift"][i])
        assert np.array_equal(oracle.diffusion(z["m"][i], z["sr"][i], z["alpha"][i]), z["diffusion"][i])
        assert np.array_equal(oracle.drift_jacobian(z["m"][i], z["alpha"][i], z["h"][i], z["hj"][i]),
                              z["drift_jac"][i])
        assert np.array_equal(oracle.diffusion_jacobian(z["m"][i], z["sr"][i], z["alpha"][i]),
                              z["diff_jac"][i])
    assert np.array_equal(oracle.mt_norm(1001, 1.0, 64), z["mt_norm_1001"])


@pytest.mark.parametrize("n,implicit", [(1, False), (5, True), (16, False), (33, False)])
def test_oracle_matches_live_reference(oracle, reference, n, implicit):
    from oracle.pyoracle import reduced_inputs
    rng = np.random.default_rng(n)
    inp = reduced_inputs(rng, n)
    noise = rng.normal(size=60 * 3 * n)
    kw = dict(field_shape="sine", happ=0.25, fapp=2.0, dt=2e-3, end_time=0.1, max_samples=8,
              use_implicit=implicit, renorm=False, interactions=True, noise=noise)
    a = oracle.full_dynamics_reduced(inp, **kw)
    b = reference.full_dynamics_reduced(inp, **kw)
    for k in FIELDS:
        assert np.array_equal(a[k], b[k]), k


def test_oracle_noise_exhaustion_like_rngarray(oracle, reference):
    # RngArray throws std::out_of_range when the injected array runs out
    # (lib/rng.cpp:84-94); the oracle reports status bit 8.
    from oracle.pyoracle import reduced_inputs
    inp = reduced_inputs(np.random.default_rng(1), 2)
    noise = np.zeros(10 * 6)
    kw = dict(dt=1e-3, end_time=0.05, max_samples=5, noise=noise)
    assert oracle.full_dynamics_reduced(inp, **kw)["status"] == 8
    assert reference.full_dynamics_reduced(inp, **kw)["status"] == 8
