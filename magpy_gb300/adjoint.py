"""Gradients of ensemble statistics through the pathwise adjoint.

``EnsembleAdjoint`` wraps the C-ABI adjoint (magpy_adjoint_*): a mixed-precision
Heun run over the in-kernel (fixed, seeded) increments with checkpoints, and the
backward sweep that returns dJ/d(K, alpha, H0) for any objective J of the
ensemble magnetisation samples.  ``sar_and_mz`` is a ``torch.autograd.Function``
giving the energy dissipated (the reference's EnsembleResults.energy_dissipated,
magpy/results.py:167-191) and the final ensemble magnetisation
(magpy/results.py:134-151) as differentiable functions of (K, alpha, H0).
PyTorch is only the autograd wrapper here; all arithmetic runs in the library.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import check, dptr
from .core import MU0, _ensemble_desc, _GroupPlan


class EnsembleAdjoint:
    """Forward run with checkpoints and its adjoint for one parameter set.

    Arguments as ``core.simulate_ensemble`` (members share the geometry; no
    renormalisation; Heun; in-kernel increments).  The anisotropy argument is
    the per-particle K; the gradient is with respect to the mean K with all
    particles scaled together.
    """

    def __init__(self, n_members, radius, anisotropy, anisotropy_axis, magnetisation_direction,
                 location, magnetisation, damping, temperature, time_step, end_time,
                 max_samples, seeds, field_shape="sine", field_amplitude=0.0,
                 field_frequency=0.0, interactions=True, checkpoint_every=256, stream=None):
        d, self._keep, self.n_particles = _ensemble_desc(
            n_members, radius, anisotropy, anisotropy_axis, magnetisation_direction, location,
            magnetisation, damping, temperature, False, interactions, False, time_step,
            end_time, max_samples, seeds, field_shape, field_amplitude, field_frequency, 1e-9,
            False, None, "mixed", None, 1000)
        self.handle = C.c_void_p()
        check(_lib.lib().magpy_adjoint_create(C.byref(d), int(checkpoint_every),
                                              C.byref(self.handle), stream))
        ph = C.c_void_p()
        check(_lib.lib().magpy_adjoint_plan(self.handle, C.byref(ph)))
        self.plan = _GroupPlan(ph, self.n_particles)
        self.field_amplitude = float(field_amplitude)

    def forward(self, stream=None):
        """Integrate; returns (time [S] s, field [S] A/m, M_z [S] A/m)."""
        check(_lib.lib().magpy_adjoint_forward(self.handle, stream))
        arr = self.plan.arrays()
        self.status = arr.status
        return arr.time[0], arr.field[0], self.plan.ensemble_magnetisation("z")

    def backward(self, dJ_dM, stream=None):
        """dJ/d(K, alpha, H0) for dJ/dM_s (the direct field term excluded)."""
        g = np.ascontiguousarray(dJ_dM, dtype=np.float64)
        theta, red = np.zeros(3), np.zeros(5)
        check(_lib.lib().magpy_adjoint_backward(self.handle, dptr(g), dptr(theta), dptr(red),
                                                stream))
        return theta, red

    def close(self):
        if getattr(self, "handle", None):
            _lib.lib().magpy_adjoint_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def sar(field, M):
    """-mu0 * trapezoid(field, M): magpy/results.py:191 over all samples."""
    return float(-MU0 * np.sum((M[1:] - M[:-1]) * (field[1:] + field[:-1]) / 2.0))


def sar_grad_M(field):
    """d sar / d M_s."""
    g = np.zeros_like(field)
    g[1:] += -MU0 * (field[1:] + field[:-1]) / 2.0
    g[:-1] -= -MU0 * (field[1:] + field[:-1]) / 2.0
    return g


def _autograd():
    import torch

    class SarMz(torch.autograd.Function):
        """(K, alpha, H0) -> (energy dissipated, final ensemble magnetisation)."""

        @staticmethod
        def forward(ctx, K, alpha, H0, cfg):
            cfg = dict(cfg)
            n = np.asarray(cfg["radius"]).size
            adj = EnsembleAdjoint(cfg["n_members"], cfg["radius"], np.full(n, float(K)),
                                  cfg["anisotropy_axis"], cfg["magnetisation_direction"],
                                  cfg["location"], cfg["magnetisation"], float(alpha),
                                  cfg["temperature"], cfg["time_step"], cfg["end_time"],
                                  cfg["max_samples"], cfg["seeds"],
                                  cfg.get("field_shape", "sine"), float(H0),
                                  cfg.get("field_frequency", 0.0),
                                  cfg.get("interactions", True),
                                  cfg.get("checkpoint_every", 256))
            t, field, M = adj.forward()
            ctx.adj, ctx.field, ctx.M, ctx.H0 = adj, field, M, float(H0)
            out = torch.tensor([sar(field, M), M[-1]], dtype=torch.float64)
            return out

        @staticmethod
        def backward(ctx, g):
            g = g.detach().cpu().double().numpy()
            dJ_dM = g[0] * sar_grad_M(ctx.field)
            dJ_dM[-1] += g[1]
            theta, _ = ctx.adj.backward(dJ_dM)
            # the energy dissipated is linear in the field samples H0 s(t)
            if ctx.H0 != 0.0:
                theta[2] += g[0] * sar(ctx.field, ctx.M) / ctx.H0
            ctx.adj.close()
            gt = [torch.tensor(x, dtype=torch.float64) for x in theta]
            return gt[0], gt[1], gt[2], None

    return SarMz


def sar_and_mz(K, alpha, H0, cfg):
    """Differentiable (energy dissipated, final ensemble magnetisation)."""
    return _autograd().apply(K, alpha, H0, cfg)
