"""Registered device targets.

The reference samples any JAX callable ``logpdf(x, data)`` and gets its
gradient from ``jax.value_and_grad`` (resource/kernel/MALA.py:59). A fused
CUDA kernel cannot call back into Python, so a target here is a descriptor
of a log-density whose value and gradient are written out in the kernels
(``csrc/targets.cuh``). ``LogPDF`` wraps one exactly as the reference's
``LogPDF`` wraps a callable.

Every target is callable like the reference's logpdf: ``t(x, data)`` with x
of shape [d] or [n, d] (a CUDA tensor) returns the log-density;
``t.value_and_grad(x)`` returns both.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from . import _lib


class Target:
    """Base class: owns the device arrays referenced by the C descriptor."""

    kind: int
    n_dim: int

    def __init__(self, n_dim: int, device="cuda"):
        self.n_dim = int(n_dim)
        self.device = torch.device(device)
        self._tensors: dict[str, torch.Tensor] = {}
        self._scalars = [0.0] * 8
        self.n_comp = 0

    def _put(self, name: str, arr) -> torch.Tensor:
        t = torch.as_tensor(np.asarray(arr, dtype=np.float32)).contiguous()
        if self.device.type == "cuda":
            t = t.to(self.device)
        self._tensors[name] = t
        return t

    def to(self, device) -> "Target":
        self.device = torch.device(device)
        for k, v in list(self._tensors.items()):
            self._tensors[k] = v.to(self.device)
        return self

    def c_struct(self) -> _lib.FmcTarget:
        s = _lib.FmcTarget()
        s.kind = self.kind
        s.n_dim = self.n_dim
        s.n_comp = self.n_comp
        for field in ("mean", "inv_var", "log_w", "precision"):
            t = self._tensors.get(field)
            setattr(s, field, _lib.ptr(t) if t is not None else None)
        for i, v in enumerate(self._scalars):
            s.scalars[i] = float(v)
        return s

    # -- the reference's logpdf call signature
    def value_and_grad(self, x: torch.Tensor):
        single = x.dim() == 1
        xx = x.reshape(1, -1) if single else x
        xx = _lib.require_cuda_f32(xx.contiguous(), "x")
        if xx.shape[1] != self.n_dim:
            raise ValueError(f"x has {xx.shape[1]} coordinates, target has {self.n_dim}")
        n = xx.shape[0]
        lp = torch.empty(n, device=xx.device, dtype=torch.float32)
        g = torch.empty_like(xx)
        st = self.c_struct()
        _lib.check(_lib.lib().fmc_target_value_grad(ctypes_byref(st), xx.data_ptr(), n, lp.data_ptr(),
                                                    g.data_ptr(), _lib.stream_handle(xx.device)))
        if single:
            return lp[0], g[0]
        return lp, g

    def __call__(self, x: torch.Tensor, data=None):
        return self.value_and_grad(x)[0]

    def describe(self) -> dict:
        """Plain-dict form (the oracle's target format)."""
        raise NotImplementedError


def ctypes_byref(s):
    import ctypes
    return ctypes.byref(s)


class DiagGaussian(Target):
    """-0.5 * sum_j (x_j - mean_j)^2 * inv_var_j + const (unnormalised by default,
    as the reference's test targets, e.g. test/unit/test_kernels.py:14-15)."""

    kind = _lib.TARGET_DIAG_GAUSSIAN

    def __init__(self, n_dim: int, mean=None, inv_var=None, const: float = 0.0, device="cuda"):
        super().__init__(n_dim, device)
        self.mean = np.zeros(n_dim) if mean is None else np.asarray(mean, np.float64)
        self.inv_var = np.ones(n_dim) if inv_var is None else np.asarray(inv_var, np.float64)
        if mean is not None:
            self._put("mean", self.mean)
        if inv_var is not None:
            self._put("inv_var", self.inv_var)
        self.const = float(const)
        self._scalars[0] = self.const

    def describe(self):
        return {"kind": "diag_gaussian", "mean": self.mean, "inv_var": self.inv_var, "const": self.const}


class DualMoon(Target):
    """-0.5((|x| - r0)/sr)^2 + logsumexp(-0.5((x0 + mu)/s0)^2, -0.5((x0 - mu)/s0)^2)."""

    kind = _lib.TARGET_DUAL_MOON

    def __init__(self, n_dim: int = 5, r0=2.0, sr=0.1, mu=3.0, s0=0.6, device="cuda"):
        super().__init__(n_dim, device)
        self.p = dict(r0=float(r0), sr=float(sr), mu=float(mu), s0=float(s0))
        self._scalars[:4] = [r0, sr, mu, s0]

    def describe(self):
        return {"kind": "dual_moon", "n_dim": self.n_dim, **self.p}


class GaussianMixture(Target):
    """Normalised mixture of K Gaussians with diagonal covariances:
    log sum_k w_k N(x; mean_k, diag(var_k))."""

    kind = _lib.TARGET_GAUSS_MIXTURE

    def __init__(self, means, variances, weights=None, device="cuda"):
        means = np.atleast_2d(np.asarray(means, np.float64))
        K, d = means.shape
        var = np.asarray(variances, np.float64)
        var = np.broadcast_to(var if var.ndim == 2 else np.broadcast_to(var, (d,)), (K, d)).copy()
        w = np.full(K, 1.0 / K) if weights is None else np.asarray(weights, np.float64)
        super().__init__(d, device)
        self.n_comp = K
        self.means, self.var, self.weights = means, var, w
        self.log_w = np.log(w) - 0.5 * np.sum(np.log(2 * np.pi * var), axis=1)
        self._put("mean", means)
        self._put("inv_var", 1.0 / var)
        self._put("log_w", self.log_w)

    def mean_cov(self):
        """Analytic mean and covariance of the mixture."""
        mu = (self.weights[:, None] * self.means).sum(0)
        cov = np.zeros((self.n_dim, self.n_dim))
        for k in range(self.n_comp):
            dm = self.means[k] - mu
            cov += self.weights[k] * (np.diag(self.var[k]) + np.outer(dm, dm))
        return mu, cov

    def describe(self):
        return {"kind": "mixture", "mean": self.means, "inv_var": 1.0 / self.var, "log_w": self.log_w}


class Rosenbrock(Target):
    """-sum_{i<d-1} [(b - x_i)^2 / a + c (x_{i+1} - x_i^2)^2]; defaults a=20, b=1,
    c=5 (the 128-D Rosenbrock-chain workload)."""

    kind = _lib.TARGET_ROSENBROCK

    def __init__(self, n_dim: int = 128, a=20.0, b=1.0, c=5.0, device="cuda"):
        super().__init__(n_dim, device)
        self.p = dict(a=float(a), b=float(b), c=float(c))
        self._scalars[:3] = [a, b, c]

    def describe(self):
        return {"kind": "rosenbrock", "n_dim": self.n_dim, **self.p}


class DenseGaussian(Target):
    """-0.5 (x - mean)^T P (x - mean) + const, P symmetrised."""

    kind = _lib.TARGET_DENSE_GAUSSIAN

    def __init__(self, precision, mean=None, const: float = 0.0, device="cuda"):
        P = np.asarray(precision, np.float64)
        d = P.shape[0]
        super().__init__(d, device)
        self.P = 0.5 * (P + P.T)
        self.mean = np.zeros(d) if mean is None else np.asarray(mean, np.float64)
        self._put("precision", self.P)
        if mean is not None:
            self._put("mean", self.mean)
        self.const = float(const)
        self._scalars[0] = self.const

    def describe(self):
        return {"kind": "dense_gaussian", "mean": self.mean, "precision": self.P, "const": self.const}


def normal_logpdf_const(d: int, var: float = 1.0) -> float:
    return -0.5 * d * math.log(2 * math.pi * var)
