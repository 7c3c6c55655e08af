"""Results containers: counterpart of magpy/results.py.

``Results`` and ``EnsembleResults`` keep the reference's attributes and
methods (magpy/results.py:6-217).  The reference's ``energy_dissipated``
cannot run as shipped (``get_mu0`` is not imported and
``scipy.integrate.trapz`` no longer exists); here it computes
-mu0 * trapezoid(field, M) as written at magpy/results.py:191, in FP64.
"""
from __future__ import annotations

import numpy as np

from .core import MU0


def _trapezoid(y, x):
    y = np.asarray(y, dtype=np.float64)
    x = np.asarray(x, dtype=np.float64)
    if y.size < 2:
        return 0.0
    return float(np.sum((x[1:] - x[:-1]) * (y[1:] + y[:-1]) / 2.0))


class Results:
    """Time-dependent magnetisation of one cluster (magpy/results.py:6-100)."""

    def __init__(self, time, field, x, y, z, N, status=0):
        self.time = time
        self.field = field
        self.x = x
        self.y = y
        self.z = z
        self.N = N
        self.status = status

    def magnetisation(self, direction="z"):
        """Sum of the particles' components (magpy/results.py:61-75)."""
        return np.sum([vals for vals in getattr(self, direction).values()], axis=0)

    def save(self, prefix):
        """Particle i's trajectory to '<prefix>_<i>.mx' etc. in the binary format
        of simulation::save_results (lib/simulation.cpp:38-63)."""
        from .core import save_results
        for i in sorted(self.x):
            save_results(f"{prefix}_{i}", self.x[i], self.y[i], self.z[i], self.field, self.time)

    def final_state(self):
        return {
            "x": {k: v[-1] for k, v in self.x.items()},
            "y": {k: v[-1] for k, v in self.y.items()},
            "z": {k: v[-1] for k, v in self.z.items()},
        }

    def plot(self):  # pragma: no cover - matplotlib is optional
        import matplotlib.pyplot as plt
        fg, axs = plt.subplots(nrows=self.N)
        if self.N == 1:
            axs = [axs]
        for idx in range(self.N):
            for c in "xyz":
                axs[idx].plot(self.time, getattr(self, c)[idx], label=c)
            axs[idx].legend()
        return fg


class EnsembleResults:
    """Results of an ensemble (magpy/results.py:103-217).

    Built either from a list of ``Results`` (as in the reference) or from the
    dense arrays of one batched GPU run, in which case the per-member
    ``Results`` are created only when asked for and the ensemble statistics
    are computed on the dense arrays directly.
    """

    def __init__(self, results=None, arrays=None):
        self._arrays = arrays
        self._results = results
        if arrays is not None:
            self.time = arrays.time[0]
            self.field = arrays.field[0]
        else:
            self.time = results[0].time
            self.field = results[0].field

    @property
    def results(self):
        if self._results is None:
            a = self._arrays
            self._results = [Results(**a.member(e), status=int(a.status[e]))
                             for e in range(a.n_members)]
        return self._results

    @property
    def status(self):
        if self._arrays is not None:
            return self._arrays.status
        return np.array([r.status for r in self.results])

    def magnetisation(self, direction="z"):
        if self._arrays is not None:
            a = self._arrays
            m = {"x": a.mx, "y": a.my, "z": a.mz}[direction]
            S = m.shape[0]
            return list(m.reshape(S, a.n_members, a.n_particles).sum(axis=2).T)
        return [res.magnetisation(direction) for res in self.results]

    def ensemble_magnetisation(self, direction="z"):
        """Mean over members of the cluster magnetisation (magpy/results.py:134-151)."""
        if self._arrays is not None:
            a = self._arrays
            m = {"x": a.mx, "y": a.my, "z": a.mz}[direction]
            S = m.shape[0]
            return m.reshape(S, a.n_members, a.n_particles).sum(axis=2).sum(axis=1) / a.n_members
        return np.sum(self.magnetisation(direction), axis=0) / len(self.results)

    def final_state(self):
        return [res.final_state() for res in self.results]

    def energy_dissipated(self, start_time=None, end_time=None):
        """-mu0 * integral of H dM over a time window (magpy/results.py:167-191)."""
        before = (self.time >= start_time) if start_time is not None else True
        after = (self.time <= end_time) if end_time is not None else True
        mask = np.ones_like(self.time, dtype=bool) & before & after
        return -MU0 * _trapezoid(self.field[mask], self.ensemble_magnetisation()[mask])

    def final_cycle_energy_dissipated(self, field_frequency):
        """Energy dissipated in the last field period (magpy/results.py:193-217)."""
        T = 1.0 / field_frequency
        return self.energy_dissipated(start_time=self.time[-1] - T)
