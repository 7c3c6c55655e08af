"""Model API: counterpart of magpy/model.py (Model, EnsembleModel).

Same constructor arguments, same ``simulate`` signatures and the same seed
derivation for ensembles (magpy/model.py:202-203).  ``EnsembleModel.simulate``
runs every member in one GPU launch instead of one joblib process per member;
``n_jobs`` is accepted and ignored.
"""
from __future__ import annotations

import numpy as np

from . import core
from .results import EnsembleResults, Results


class Model:
    """A cluster of interacting magnetic nanoparticles (magpy/model.py:16-58)."""

    def __init__(self, radius, anisotropy, anisotropy_axis, magnetisation_direction, location,
                 magnetisation, damping, temperature, field_shape="constant",
                 field_frequency=0.0, field_amplitude=0.0):
        self.radius = np.array(radius)
        self.anisotropy = np.array(anisotropy)
        self.anisotropy_axis = np.array(anisotropy_axis)
        self.magnetisation_direction = np.array(magnetisation_direction)
        self.location = np.array(location)
        self.magnetisation = magnetisation
        self.damping = damping
        self.temperature = temperature
        self.field_shape = field_shape
        self.field_frequency = field_frequency
        self.field_amplitude = field_amplitude

    def simulate(self, end_time, time_step, max_samples, seed=1001, renorm=False,
                 interactions=True, implicit_solve=True, implicit_tol=1e-9, precision="fp64"):
        """magpy/model.py:70-115, on the GPU."""
        res = core.simulate(self.radius, self.anisotropy, self.anisotropy_axis,
                            self.magnetisation_direction, self.location, self.magnetisation,
                            self.damping, self.temperature, renorm, interactions,
                            implicit_solve, time_step, end_time, max_samples, seed,
                            self.field_shape, self.field_amplitude, self.field_frequency,
                            implicit_tol, precision=precision)
        return Results(**res)


_GEOMETRY = ("radius", "anisotropy", "anisotropy_axis", "magnetisation_direction", "location")
_SCALARS = ("magnetisation", "damping", "temperature", "field_amplitude", "field_frequency")


class EnsembleModel:
    """Ensemble of particle clusters (magpy/model.py:118-208)."""

    def __init__(self, N, base_model, **kwargs):
        self.ensemble_size = N
        self.base_model_params = base_model.__dict__
        self.model_params = [
            {**self.base_model_params, **{key: kwargs[key][i] for key in kwargs}}
            for i in range(self.ensemble_size)
        ]
        self.models = [Model(**params) for params in self.model_params]
        self._overrides = set(kwargs)

    def seeds(self, random_state):
        """Per-member seeds exactly as magpy/model.py:202-203 derives them."""
        np.random.seed(random_state)
        return np.random.randint(np.iinfo(np.int32).max, size=self.ensemble_size)

    def simulate(self, end_time, time_step, max_samples, random_state, renorm=False,
                 interactions=True, n_jobs=1, implicit_solve=True, implicit_tol=1e-9,
                 precision="fp64"):
        """magpy/model.py:159-208, all members batched on the GPU."""
        return self.simulate_members(range(self.ensemble_size), self.seeds(random_state),
                                     end_time, time_step, max_samples, renorm=renorm,
                                     interactions=interactions, implicit_solve=implicit_solve,
                                     implicit_tol=implicit_tol, precision=precision)

    def simulate_members(self, members, seeds, end_time, time_step, max_samples, renorm=False,
                         interactions=True, implicit_solve=True, implicit_tol=1e-9,
                         precision="fp64"):
        """Integrate the members ``members`` (indices into ``self.models``) with
        the given per-member seeds; one launch per (field shape, size) group."""
        members = list(members)
        seeds = np.asarray(seeds)
        groups = {}
        for j, e in enumerate(members):
            m = self.models[e]
            key = (m.field_shape, np.asarray(m.radius).size)
            groups.setdefault(key, []).append(j)
        per_geom = bool(self._overrides & set(_GEOMETRY))
        results = [None] * len(members)
        for (shape, n), loc in groups.items():
            ms = [self.models[members[j]] for j in loc]
            if per_geom:
                geo = {k: np.concatenate([np.asarray(getattr(m, k), dtype=np.float64).reshape(
                    n, -1) for m in ms]) for k in _GEOMETRY}
            else:
                geo = {k: np.asarray(getattr(ms[0], k), dtype=np.float64) for k in _GEOMETRY}
            per_member = {k: np.array([getattr(m, k) for m in ms], dtype=np.float64)
                          for k in _SCALARS if k in self._overrides}
            base = ms[0]
            arr = core.simulate_ensemble(
                len(loc), geo["radius"], geo["anisotropy"], geo["anisotropy_axis"],
                geo["magnetisation_direction"], geo["location"], base.magnetisation,
                base.damping, base.temperature, renorm, interactions, implicit_solve, time_step,
                end_time, max_samples, seeds[loc], shape, base.field_amplitude,
                base.field_frequency, implicit_tol, per_member_geometry=per_geom,
                per_member=per_member, precision=precision)
            if len(groups) == 1:
                return EnsembleResults(arrays=arr)
            for i, j in enumerate(loc):
                results[j] = Results(**arr.member(i), status=int(arr.status[i]))
        return EnsembleResults(results)


class DOModel:
    """Two-state (up/down) probabilistic model of one uniaxial particle
    (magpy/model.py:211-295): the master equation with Neel-Brown rates,
    integrated on the GPU."""

    def __init__(self, radius, anisotropy, initial_probabilities, magnetisation, damping,
                 temperature, field_shape="constant", field_frequency=0.0, field_amplitude=0.0,
                 field_n_components=1):
        self.radius = radius
        self.volume = 4. / 3 * np.pi * self.radius ** 3  # magpy/model.py:255
        self.anisotropy = anisotropy
        self.initial_probabilities = np.array(initial_probabilities)
        self.magnetisation = magnetisation
        self.damping = damping
        self.temperature = temperature
        self.field_shape = field_shape
        self.field_frequency = field_frequency
        self.field_amplitude = field_amplitude
        self.field_n_components = field_n_components

    def simulate(self, end_time, time_step, max_samples):
        """magpy/model.py:266-295."""
        res = core.simulate_dom(self.initial_probabilities, self.volume, self.anisotropy,
                                self.temperature, self.magnetisation, self.damping, time_step,
                                end_time, max_samples, self.field_shape, self.field_amplitude,
                                self.field_frequency, self.field_n_components)
        return Results(**res)
