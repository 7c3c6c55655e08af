"""Generates the golden fixtures in this folder from the reference itself.

Runs the reference's own lib/*.cpp (built by ``make -C oracle ref`` from the
reference checkout into oracle/_ref/libmagpy_ref.so, driven through
oracle/ref_harness.cpp) on seeded inputs and stores inputs and outputs:

* ``reduced_*.npz``  -- reduced-unit simulation::full_dynamics
  (lib/simulation.cpp:132) with injected increments through RngArray;
* ``physical_*.npz`` -- physical-unit simulation::full_dynamics
  (lib/simulation.cpp:476) with the reference's own RngMtNorm noise;
* ``components.npz`` -- llg/field component functions on random inputs.

Usage:  python tests/golden/make_golden.py   (needs oracle/_ref built here)
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.pyoracle import Reference, reduced_inputs  # noqa: E402

# (name, n, implicit, field shape, renorm, interactions, dt, end, samples)
REDUCED_CASES = [
    ("reduced_n1_heun_const", 1, False, "constant", False, True, 1.7e-3, 0.5, 21),
    ("reduced_n1_implicit_sine", 1, True, "sine", False, True, 1.7e-3, 0.5, 21),
    ("reduced_n2_heun_sine", 2, False, "sine", False, True, 1.7e-3, 0.3, 11),
    ("reduced_n3_implicit_square", 3, True, "square", True, True, 1.7e-3, 0.3, 11),
    ("reduced_n8_heun_square_renorm", 8, False, "square", True, True, 2.0e-3, 0.2, 9),
    ("reduced_n27_heun_sine", 27, False, "sine", False, True, 1.0e-3, 0.05, 6),
    ("reduced_n27_implicit_const", 27, True, "constant", False, True, 1.0e-3, 0.03, 4),
    ("reduced_n40_heun_const", 40, False, "constant", False, True, 1.0e-3, 0.02, 3),
    ("reduced_n8_heun_noint", 8, False, "constant", False, False, 1.0e-3, 0.05, 6),
    # a sample interval shorter than the step: samples repeat the held state
    ("reduced_n2_heun_oversampled", 2, False, "constant", False, True, 1.0e-2, 0.05, 23),
]

PHYSICAL_CASES = [
    # (name, n, implicit, shape, amp, freq, dt, end, samples, seed)
    ("physical_n1_heun", 1, False, "constant", 0.0, 0.0, 1e-13, 2e-11, 21, 1001),
    ("physical_n1_implicit", 1, True, "constant", 0.0, 0.0, 1e-13, 2e-11, 21, 1001),
    ("physical_n4_heun_sine", 4, False, "sine", 1e4, 3e9, 5e-14, 1e-11, 11, 77),
    ("physical_n5_implicit_sine", 5, True, "sine", 1e4, 3e9, 1e-13, 1e-11, 11, 12345),
]


def main():
    R = Reference()
    rng = np.random.default_rng(20240601)
    for name, n, implicit, shape, renorm, inter, dt, end, S in REDUCED_CASES:
        inp = reduced_inputs(rng, n)
        K = int(end / dt) + 4
        noise = rng.normal(size=K * 3 * n)
        kw = dict(field_shape=shape, happ=0.2, fapp=1.5, k_av=2.0e4, v_av=1.0, alpha=0.1,
                  ms=4.0e5, dt=dt, end_time=end, renorm=renorm, interactions=inter,
                  use_implicit=implicit, eps=1e-9, max_samples=S, noise=noise)
        out = R.full_dynamics_reduced(inp, **kw)
        assert out["status"] == 0, name
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            **{"in_" + k: np.asarray(v) for k, v in inp.items()},
            **{"kw_" + k: np.asarray(v) for k, v in kw.items() if k != "noise"},
            noise=noise, x=out["x"], y=out["y"], z=out["z"], field=out["field"],
            time=out["time"])
        print(name, "ok")
    for name, n, implicit, shape, amp, freq, dt, end, S, seed in PHYSICAL_CASES:
        radius = rng.uniform(6e-9, 9e-9, n)
        K = rng.uniform(1.5e4, 2.5e4, n)
        axes = rng.normal(size=(n, 3))
        axes /= np.linalg.norm(axes, axis=1, keepdims=True)
        m0 = rng.normal(size=(n, 3))
        m0 /= np.linalg.norm(m0, axis=1, keepdims=True)
        loc = np.stack([np.arange(n) * 18e-9, rng.uniform(-2e-9, 2e-9, n),
                        rng.uniform(-2e-9, 2e-9, n)], axis=1)
        kw = dict(renorm=False, interactions=True, use_implicit=implicit, eps=1e-9,
                  time_step=dt, end_time=end, max_samples=S, seed=seed, field_shape=shape,
                  field_amplitude=amp, field_frequency=freq)
        out = R.full_dynamics(radius, K, axes, m0, loc, 4e5, 0.1, 300.0, **kw)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"), radius=radius, anisotropy=K, axes=axes, m0=m0,
            location=loc, ms=4e5, damping=0.1, temperature=300.0,
            **{"kw_" + k: np.asarray(v) for k, v in kw.items()},
            x=out["x"], y=out["y"], z=out["z"], field=out["field"], time=out["time"])
        print(name, "ok")
    # component functions on random inputs
    m = rng.normal(size=(64, 3))
    h = rng.normal(size=(64, 3))
    hj = rng.normal(size=(64, 9))
    alpha = rng.uniform(0.01, 1.0, 64)
    sr = rng.uniform(0.01, 1.0, 64)
    comp = dict(m=m, h=h, hj=hj, alpha=alpha, sr=sr,
                drift=np.array([R.drift(m[i], alpha[i], h[i]) for i in range(64)]),
                diffusion=np.array([R.diffusion(m[i], sr[i], alpha[i]) for i in range(64)]),
                drift_jac=np.array([R.drift_jacobian(m[i], alpha[i], h[i], hj[i])
                                    for i in range(64)]),
                diff_jac=np.array([R.diffusion_jacobian(m[i], sr[i], alpha[i])
                                   for i in range(64)]),
                mt_norm_1001=R.mt_norm(1001, 1.0, 64))
    np.savez_compressed(os.path.join(HERE, "components.npz"), **comp)
    print("components ok")


if __name__ == "__main__":
    main()
