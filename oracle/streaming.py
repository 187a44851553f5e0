"""Oracle of the streaming diagnostics (fmc_welford_ess_*) -- TEST
INFRASTRUCTURE ONLY, float64 NumPy.

The reference has no streaming diagnostics (its tutorials run arviz after
sampling), so these follow the published estimators the library implements:
Welford's running mean and sum of squared deviations (Technometrics 4, 1962)
per chain and coordinate, Welford over each chain's completed batch means,
the chains merged with the pairwise formulas of Chan, Golub & LeVeque (1979),
R-hat of Gelman & Rubin (1992) and the multi-chain batch-means ESS
N var / (b var_bm) (Flegal & Jones, Ann. Stat. 2010). The recurrences are
applied in the same order as the device kernel, draw by draw.
"""
from __future__ import annotations

import numpy as np


class StreamingOracle:
    def __init__(self, n_chains: int, n_dim: int, batch: int):
        self.n = 0
        self.batch = batch
        shp = (n_chains, n_dim)
        self.mean, self.m2 = np.zeros(shp), np.zeros(shp)
        self.bsum, self.bmean, self.bm2 = np.zeros(shp), np.zeros(shp), np.zeros(shp)

    def update(self, rows: np.ndarray):
        """rows [n_chains, n_steps, n_dim] (float32 values, taken as float64)."""
        rows = np.asarray(rows, np.float64)
        for s in range(rows.shape[1]):
            x = rows[:, s]
            n = self.n + 1
            delta = x - self.mean
            self.mean = self.mean + delta / n
            self.m2 = self.m2 + delta * (x - self.mean)
            self.bsum = self.bsum + x
            if n % self.batch == 0:
                bm = self.bsum / self.batch
                k = n // self.batch
                bd = bm - self.bmean
                self.bmean = self.bmean + bd / k
                self.bm2 = self.bm2 + bd * (bm - self.bmean)
                self.bsum = np.zeros_like(self.bsum)
            self.n = n

    def finalize(self):
        """(mean, var, ess, rhat) per coordinate."""
        C = self.mean.shape[0]
        n, b = self.n, self.batch
        k = n // b
        mu = self.mean.mean(0)
        dev = ((self.mean - mu) ** 2).sum(0)
        N = C * n
        var = (self.m2.sum(0) + n * dev) / (N - 1)
        W = self.m2.sum(0) / (C * (n - 1)) if n > 1 else np.zeros_like(mu)
        B_n = dev / (C - 1) if C > 1 else np.zeros_like(mu)
        with np.errstate(invalid="ignore", divide="ignore"):
            rhat = np.sqrt(((n - 1) / n * W + B_n) / W)
        Kb = C * k
        if Kb > 1:
            mub = self.bmean.mean(0)
            var_bm = (self.bm2.sum(0) + k * ((self.bmean - mub) ** 2).sum(0)) / (Kb - 1)
            tau = b * var_bm / var
            ess = np.minimum(np.where(tau > 0, N / np.where(tau > 0, tau, 1.0), N), N)
        else:
            ess = np.full_like(mu, np.nan)
        return mu, var, ess, rhat
