"""magpy_gb300 -- GB300-native stochastic LLG ensemble integrator.

Drop-in for magpy's ``Model`` / ``EnsembleModel`` / ``magpy.core.simulate``
path; the work runs in hand-written CUDA (libmagpy_gpu.so, sm_103a) behind a
C-ABI (include/magpy_gpu.h).
"""
from . import core, results
from .core import get_KB, get_gamma, get_mu0, simulate, simulate_ensemble
from .model import EnsembleModel, Model
from .results import EnsembleResults, Results

__all__ = ["Model", "EnsembleModel", "Results", "EnsembleResults", "simulate",
           "simulate_ensemble", "get_KB", "get_mu0", "get_gamma", "core", "results"]
