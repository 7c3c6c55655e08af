"""Generates stats_reference.npz: ensemble statistics computed by the
reference's own magpy/results.py on trajectories from the reference itself.

The trajectories are the reference's physical-unit simulation::full_dynamics
(lib/simulation.cpp:476-624, built by ``make -C oracle ref`` into
oracle/_ref/libmagpy_ref.so) for a small interacting ensemble in an AC field,
one call per member with the member's seed and the reference's own
RngMtNorm noise.  They are wrapped into the reference's ``Results`` and
``EnsembleResults`` (magpy/results.py:6-217), loaded from the reference
checkout with the shims the shipped module needs to import and run in this
environment:

* ``scipy.integrate.trapz`` no longer exists in scipy 1.18; the reference's
  ``trapz(y, x)`` was numpy's trapezoid rule, so ``numpy.trapezoid`` stands in;
* ``matplotlib`` (used only by ``plot``) is a stub module;
* ``get_mu0`` is used at magpy/results.py:191 but never imported (a NameError
  as shipped); it is injected as magpy/core.pyx:31-32 defines it (MU0 of
  include/constants.hpp:11).

Outputs: member magnetisation, ensemble magnetisation (x, y, z), energy
dissipated over the whole run and over a window, and over the final field
cycle.

Usage:  python tests/golden/make_stats_golden.py   (needs oracle/_ref and the
reference checkout, MAGPY_REFERENCE or the default location)
"""
from __future__ import annotations

import os
import sys
import types

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from oracle.pyoracle import Reference  # noqa: E402

REF = os.environ.get("MAGPY_REFERENCE", "/root/reference")
MU0 = 1.25663706e-6  # include/constants.hpp:11, returned by magpy/core.pyx:31-32

# ensemble: E members of an N-particle chain, sine field over ~2.5 cycles
E, N = 6, 3
DT, END, S = 5e-14, 1.25e-9, 251
H0, F = 2e4, 2e9


def reference_results_module():
    import scipy.integrate
    if not hasattr(scipy.integrate, "trapz"):
        scipy.integrate.trapz = np.trapezoid
    mpl = types.ModuleType("matplotlib")
    mpl.pyplot = types.ModuleType("matplotlib.pyplot")
    sys.modules.setdefault("matplotlib", mpl)
    sys.modules.setdefault("matplotlib.pyplot", mpl.pyplot)
    path = os.path.join(REF, "magpy", "results.py")
    mod = types.ModuleType("reference_results")
    mod.__file__ = path
    code = compile(open(path).read(), path, "exec")
    exec(code, mod.__dict__)
    mod.get_mu0 = lambda: MU0
    return mod


def main():
    rng = np.random.default_rng(8128)
    radius = rng.uniform(6e-9, 8e-9, N)
    K = rng.uniform(1.8e4, 2.2e4, N)
    axes = rng.normal(size=(N, 3))
    axes /= np.linalg.norm(axes, axis=1, keepdims=True)
    m0 = axes.copy()
    loc = np.stack([np.arange(N) * 20e-9, np.zeros(N), np.zeros(N)], 1)
    seeds = rng.integers(1, 2**31 - 1, size=E)
    kw = dict(renorm=False, interactions=True, use_implicit=False, eps=1e-9, time_step=DT,
              end_time=END, max_samples=S, field_shape="sine", field_amplitude=H0,
              field_frequency=F)
    R = Reference()
    res = reference_results_module()
    x, y, z = (np.empty((E, N, S)) for _ in range(3))
    members = []
    for e in range(E):
        out = R.full_dynamics(radius, K, axes, m0, loc, 4e5, 0.1, 300.0, seed=int(seeds[e]), **kw)
        x[e], y[e], z[e] = out["x"], out["y"], out["z"]
        time, field = out["time"], out["field"]
        members.append(res.Results(time, field, {i: x[e, i] for i in range(N)},
                                   {i: y[e, i] for i in range(N)},
                                   {i: z[e, i] for i in range(N)}, N))
    ens = res.EnsembleResults(members)
    t = ens.time
    win = (t[40], t[180])
    np.savez_compressed(
        os.path.join(HERE, "stats_reference.npz"),
        radius=radius, anisotropy=K, axes=axes, m0=m0, location=loc, seeds=seeds,
        ms=4e5, damping=0.1, temperature=300.0,
        **{"kw_" + k: np.asarray(v) for k, v in kw.items()},
        x=x, y=y, z=z, time=time, field=field,
        member_magnetisation_z=np.array(ens.magnetisation("z")),
        ensemble_magnetisation_x=ens.ensemble_magnetisation("x"),
        ensemble_magnetisation_y=ens.ensemble_magnetisation("y"),
        ensemble_magnetisation_z=ens.ensemble_magnetisation("z"),
        energy_dissipated=ens.energy_dissipated(),
        window=np.array(win),
        energy_dissipated_window=ens.energy_dissipated(*win),
        final_cycle_energy_dissipated=ens.final_cycle_energy_dissipated(F))
    print("stats_reference ok: E_full", ens.energy_dissipated(), "E_last_cycle",
          ens.final_cycle_energy_dissipated(F))


if __name__ == "__main__":
    main()
