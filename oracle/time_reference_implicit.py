"""Timing recipe (test infrastructure): the reference's implicit-midpoint path
at N = 27, 64, 125 against the oracle's block-3x3 restatement.

The reference assembles dense (3N)^3 diffusion Jacobians and solves a dense
3N system per Newton iteration (lib/integrators.cpp:576-651,
lib/optimisation.cpp:81-149), so at N = 512 one member needs a ~29 GB work
array; this recipe measures how its cost grows at the sizes where it runs,
one member, one core, on the cluster geometry of the benchmark (sphere
packing, log-normal radii), alpha = 0.01, dt = 2e-13 s, eps = 1e-9.

Needs the compiled reference (oracle/_ref/libmagpy_ref.so, built by
`make -C oracle ref` where the reference sources exist).  Prints one JSON
line per N.

    python oracle/time_reference_implicit.py [--steps 3]
"""
import argparse
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

from bench import cluster_geometry  # noqa: E402
from oracle.pyoracle import Oracle, Reference, REF_SO  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--sizes", default="27,64,125")
    args = ap.parse_args()
    if not os.path.exists(REF_SO):
        print(json.dumps({"unavailable": f"{REF_SO} not built"}))
        return
    ref, port = Reference(), Oracle()
    dt = 2e-13
    for n in (int(s) for s in args.sizes.split(",")):
        g = cluster_geometry(n, seed=512)
        kw = dict(renorm=False, interactions=True, use_implicit=True, eps=1e-9, time_step=dt,
                  end_time=dt * (args.steps - 0.5), max_samples=2, seed=77,
                  field_shape="sine", field_amplitude=1e4, field_frequency=3e5)
        geo = (g["radius"], g["anisotropy"], g["anisotropy_axis"],
               g["magnetisation_direction"], g["location"], 4e5, 0.01, 300.0)
        t0 = time.perf_counter()
        a = ref.full_dynamics(*geo, **kw)
        t_ref = time.perf_counter() - t0
        t0 = time.perf_counter()
        b = port.full_dynamics(*geo, **kw)
        t_port = time.perf_counter() - t0
        diff = max(float(np.max(np.abs(a[c] - b[c]))) for c in "xyz")
        units = n * args.steps
        print(json.dumps({
            "n": n, "steps": args.steps,
            "reference_particle_steps_per_s": units / t_ref,
            "reference_s_per_step": t_ref / args.steps,
            "port_particle_steps_per_s": units / t_port,
            "max_abs_diff_port_vs_reference": diff,
            "cores": 1}))


if __name__ == "__main__":
    main()
