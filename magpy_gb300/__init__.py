"""magpy_gb300 -- GB300-native stochastic LLG ensemble integrator.

Drop-in for magpy's ``Model`` / ``EnsembleModel`` / ``magpy.core.simulate``
path; the work runs in hand-written CUDA (libmagpy_gpu.so, sm_103a) behind a
C-ABI (include/magpy_gpu.h).
"""
from . import core, results
from .core import get_KB, get_gamma, get_mu0, simulate, simulate_dom, simulate_ensemble
from .model import DOModel, EnsembleModel, Model
from .results import EnsembleResults, Results

__all__ = ["Model", "EnsembleModel", "DOModel", "Results", "EnsembleResults", "simulate",
           "simulate_ensemble", "simulate_dom", "get_KB", "get_mu0", "get_gamma", "core", "results"]
