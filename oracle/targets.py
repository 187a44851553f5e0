"""Oracle target log-densities with analytic gradients (float64, NumPy).

TEST INFRASTRUCTURE ONLY. These are the synthetic targets the sampler is run
on. In the reference a target is a user JAX callable wrapped by ``LogPDF``
(resource/logPDF.py:20-81) and differentiated by ``jax.value_and_grad``
(resource/kernel/MALA.py:59); here each registered target has its value and
gradient written out, and tests check the gradients against central finite
differences.

A target is a plain dict:
  {"kind": "diag_gaussian", "mean": [d], "inv_var": [d], "const": c}
  {"kind": "dual_moon", "n_dim": d, "r0": 2, "sr": 0.1, "mu": 3, "s0": 0.6}
  {"kind": "mixture", "mean": [K, d], "inv_var": [K, d], "log_w": [K]}
  {"kind": "rosenbrock", "n_dim": d, "a": 20, "b": 1, "c": 5}
  {"kind": "dense_gaussian", "mean": [d], "precision": [d, d], "const": c}
"""
from __future__ import annotations

import numpy as np


def value_grad(t: dict, x: np.ndarray) -> tuple[np.ndarray, np.ndarray]:
    """x [n, d] -> (logp [n], grad [n, d]) in float64."""
    x = np.asarray(x, dtype=np.float64)
    k = t["kind"]
    if k == "tempered":
        # TemperedPDF.tempered_log_pdf (resource/logPDF.py:106-108): per-row
        # beta = 1 / T times the base log-density, plus an optional diagonal
        # Gaussian log prior
        lp, g = value_grad(t["base"], x)
        beta = np.asarray(t["beta"], np.float64)
        lp, g = beta * lp, beta[:, None] * g
        pr = t.get("prior")
        if pr is not None:
            dx = x - np.asarray(pr["mean"], np.float64)
            iv = np.asarray(pr["inv_var"], np.float64)
            lp = lp - 0.5 * np.sum(dx * dx * iv, axis=-1) + pr.get("const", 0.0)
            g = g - dx * iv
        return lp, g
    if k == "diag_gaussian":
        m = np.asarray(t["mean"], np.float64)
        iv = np.asarray(t["inv_var"], np.float64)
        dx = x - m
        lp = -0.5 * np.sum(dx * dx * iv, axis=-1) + t.get("const", 0.0)
        return lp, -dx * iv
    if k == "dual_moon":
        r0, sr, mu, s0 = t["r0"], t["sr"], t["mu"], t["s0"]
        r = np.linalg.norm(x, axis=-1)
        tt = (r - r0) / sr
        za = (x[:, 0] + mu) / s0
        zb = (x[:, 0] - mu) / s0
        a, b = -0.5 * za * za, -0.5 * zb * zb
        lse = np.logaddexp(a, b)
        lp = -0.5 * tt * tt + lse
        g = (-(tt / sr) / r)[:, None] * x
        wa, wb = np.exp(a - lse), np.exp(b - lse)
        g[:, 0] += wa * (-za / s0) + wb * (-zb / s0)
        return lp, g
    if k == "mixture":
        m = np.asarray(t["mean"], np.float64)        # [K, d]
        iv = np.asarray(t["inv_var"], np.float64)    # [K, d]
        lw = np.asarray(t["log_w"], np.float64)      # [K]
        dx = x[:, None, :] - m[None]                 # [n, K, d]
        e = lw[None] - 0.5 * np.sum(dx * dx * iv[None], axis=-1)
        emax = e.max(axis=1, keepdims=True)
        lse = (emax + np.log(np.exp(e - emax).sum(axis=1, keepdims=True)))[:, 0]
        w = np.exp(e - lse[:, None])
        g = -np.sum(w[:, :, None] * dx * iv[None], axis=1)
        return lse, g
    if k == "rosenbrock":
        a, b, c = t["a"], t["b"], t["c"]
        x0, x1 = x[:, :-1], x[:, 1:]
        u = b - x0
        v = x1 - x0 * x0
        lp = -np.sum(u * u / a + c * v * v, axis=-1)
        g = np.zeros_like(x)
        g[:, :-1] += 2.0 * u / a + 4.0 * c * x0 * v
        g[:, 1:] -= 2.0 * c * v
        return lp, g
    if k == "dense_gaussian":
        m = np.asarray(t["mean"], np.float64)
        P = np.asarray(t["precision"], np.float64)
        P = 0.5 * (P + P.T)
        dx = x - m
        Pd = dx @ P
        lp = -0.5 * np.sum(dx * Pd, axis=-1) + t.get("const", 0.0)
        return lp, -Pd
    raise ValueError(f"unknown target kind {k}")


def value(t: dict, x: np.ndarray) -> np.ndarray:
    return value_grad(t, x)[0]


def n_dim(t: dict) -> int:
    if t["kind"] == "tempered":
        return n_dim(t["base"])
    if "n_dim" in t:
        return int(t["n_dim"])
    m = np.asarray(t["mean"])
    return int(m.shape[-1])
