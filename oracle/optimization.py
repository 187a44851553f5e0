"""Oracle AdamOptimization (float64) -- TEST INFRASTRUCTURE ONLY.

Restates strategy/optimization.py:117-164 with the per-chain-step gradient
noise passed in, and optax.adam (Kingma & Ba 2015 with optax's defaults
b1 = 0.9, b2 = 0.999, eps = 1e-8, eps_root = 0, bias correction by
1 - b**t) followed by optax.projections.projection_box (a clip).
"""
from __future__ import annotations

import numpy as np

from . import targets as T


def adam_optimize(t, x0, n_steps, lr, noise_level, xi, bounds=None):
    """x0 [C, d]; xi [C, n_steps] standard normals. Returns (x [C, d], log p(x) [C])."""
    x = np.array(x0, np.float64)
    C, d = x.shape
    b = np.array([[-np.inf, np.inf]]) if bounds is None else np.asarray(bounds, np.float64)
    lo, hi = np.broadcast_to(b[:, 0], (d,)), np.broadcast_to(b[:, 1], (d,))
    m = np.zeros_like(x)
    v = np.zeros_like(x)
    b1, b2, eps = 0.9, 0.999, 1e-8
    for s in range(n_steps):
        _, g = T.value_grad(t, x)
        gr = -g * (1.0 + xi[:, s:s + 1] * noise_level)          # optimization.py:122-124
        m = (1 - b1) * gr + b1 * m
        v = (1 - b2) * gr * gr + b2 * v
        tt = s + 1
        upd = (m / (1 - b1 ** tt)) / (np.sqrt(v / (1 - b2 ** tt)) + eps)
        x = np.clip(x - lr * upd, lo, hi)                        # optimization.py:125-129
    return x, T.value(t, x)
