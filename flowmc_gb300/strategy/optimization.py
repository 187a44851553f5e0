"""AdamOptimization (mirrors strategy/optimization.py:12-164 of the reference).

The reference vmaps, over chains, a scan of n_steps Adam updates on
-logpdf with multiplicative gradient noise and a box projection
(optimization.py:117-152). Here the whole optimisation is one persistent
launch (``fmc_adam_optimize``): each chain's position and Adam moments stay
on-chip and the target's gradient is the fused device target's adjoint.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .. import _lib
from ..random import split
from ..resource.logPDF import as_target
from .base import Strategy


class AdamOptimization(Strategy):
    """Optimize a set of chains using Adam optimization. Note that if the
    posterior can go to infinity, this optimization scheme is likely to
    return NaNs.

    bounds: [n_dim, 2] or [1, 2] (broadcast to every dimension), projected
    onto after each update."""

    n_steps: int = 100
    learning_rate: float = 1e-2
    noise_level: float = 10

    def __repr__(self):
        return "AdamOptimization"

    def __init__(self, logpdf, n_steps: int = 100, learning_rate: float = 1e-2, noise_level: float = 10,
                 bounds=np.array([[-np.inf, np.inf]])):
        self.logpdf = logpdf
        self.n_steps = n_steps
        self.learning_rate = learning_rate
        self.noise_level = noise_level
        b = np.asarray(torch.as_tensor(bounds).cpu().numpy() if isinstance(bounds, torch.Tensor) else bounds,
                       np.float64)
        if b.ndim != 2 or b.shape[1] != 2:
            raise ValueError(f"bounds must have shape (n_dim, 2) or (1, 2), got {b.shape}")
        self.bounds = b

    def __call__(self, rng_key, resources, initial_position, data):
        rng_key, optimized_positions, _ = self.optimize(rng_key, None, initial_position, data)
        return rng_key, resources, optimized_positions

    def optimize(self, rng_key, objective, initial_position, data, noise=None):
        """optimization.py:85-164. ``objective`` must be None (-logpdf of the
        strategy's device target): an arbitrary Python objective cannot run
        inside the fused kernel. ``noise`` [n_chains, n_steps] replaces the
        in-kernel normals. Returns (rng_key, positions, final log-probabilities)."""
        if objective is not None:
            raise NotImplementedError("the fused optimiser minimises -logpdf of a registered device target; "
                                      "pass objective=None")
        target = as_target(self.logpdf)
        x0 = _lib.require_cuda_f32(torch.atleast_2d(torch.as_tensor(initial_position)).to(torch.float32)
                                   .contiguous(), "initial_position")
        C, d = x0.shape
        if not (self.bounds.shape[0] == 1 or self.bounds.shape[0] == d):
            raise ValueError(f"bounds shape {self.bounds.shape} is incompatible with n_dim={d}. "
                             "Provide bounds of shape (1, 2) for broadcasting or (n_dim, 2) for per-dimension "
                             "bounds.")
        if d != target.n_dim:
            raise ValueError(f"positions have {d} coordinates, target has {target.n_dim}")
        lo = np.broadcast_to(self.bounds[:, 0], (d,))
        hi = np.broadcast_to(self.bounds[:, 1], (d,))
        lower = None if np.all(np.isneginf(lo)) else torch.tensor(lo, dtype=torch.float32, device=x0.device)
        upper = None if np.all(np.isposinf(hi)) else torch.tensor(hi, dtype=torch.float32, device=x0.device)
        if noise is not None:
            noise = _lib.require_cuda_f32(noise.contiguous(), "noise", (C, self.n_steps))
        print("Using Adam optimization")
        rng_key, subkey = split(rng_key)                          # optimization.py:154
        x_out = torch.empty_like(x0)
        lp_out = torch.empty(C, device=x0.device)
        tgt = target.c_struct()
        _lib.check(_lib.lib().fmc_adam_optimize(
            ctypes.byref(tgt), x0.data_ptr(), C, int(self.n_steps), float(self.learning_rate),
            float(self.noise_level), _lib.ptr(lower), _lib.ptr(upper), subkey.value, 0, _lib.ptr(noise),
            x_out.data_ptr(), lp_out.data_ptr(), _lib.stream_handle(x0.device)))
        if not bool(torch.isfinite(lp_out).all()):                # optimization.py:161-162
            print("Warning: Optimization accessed infinite or NaN log-probabilities.")
        return rng_key, x_out, lp_out
