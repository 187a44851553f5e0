"""HMC kernel (mirrors resource/kernel/HMC.py:11-163 of the reference).

The leapfrog table has rows [0, .5], [1, 1] x n_leapfrog, [1, .5]
(HMC.py:47-50): n_leapfrog + 1 drifts with half kicks at both ends. The
momentum is xi @ cholesky(inv(M)).T and the kinetic energy 0.5 * sum(p^2 * M)
with numpy broadcasting (for a matrix M: the column sums of M weight p^2),
H uses the incoming log_prob (HMC.py:118-151). The fused kernel takes the
column sums as a vector and the momentum transform either as the diagonal of
cholesky(inv(M)) (diagonal M) or as the full lower-triangular factor (dense
M: one triangular matvec per step, the chain's normals shared through shared
memory).
"""
from __future__ import annotations

import numpy as np
import torch

from ... import _lib
from .base import LocalKernel


class HMC(LocalKernel):
    """Hamiltonian Monte Carlo sampler class."""

    kernel_kind = _lib.KERNEL_HMC

    @property
    def n_leapfrog(self) -> int:
        return self.leapfrog_coefs.shape[0] - 2

    def __repr__(self):
        return ("HMC with step size " + str(self.step_size) + " and " + str(self.n_leapfrog)
                + " leapfrog steps")

    def __init__(self, condition_matrix=1, step_size=0.1, n_leapfrog: int = 10):
        self.condition_matrix = condition_matrix
        self.step_size = step_size
        coefs = np.ones((n_leapfrog + 2, 2))
        coefs[0] = [0, 0.5]
        coefs[-1] = [1, 0.5]
        self.leapfrog_coefs = coefs
        self._cache = {}

    def metric_vectors(self, n_dim: int):
        """(momentum_scale, column_sums, cholesky factor) as float64 arrays:
        (None, None, None) for M = I, (diag(L), colsum, None) for a diagonal M,
        (None, colsum, L) for a dense M, with L = cholesky(inv(M))."""
        M = self.condition_matrix
        if isinstance(M, torch.Tensor):
            M = M.detach().cpu().numpy()
        M = np.asarray(M, np.float64)
        if M.ndim == 0:
            M = float(M) * np.eye(n_dim)
        elif M.ndim == 1:
            M = np.diag(M)
        if M.shape != (n_dim, n_dim):
            raise ValueError(f"condition_matrix has shape {M.shape}, expected ({n_dim}, {n_dim})")
        if np.array_equal(M, np.eye(n_dim)):
            return None, None, None
        L = np.linalg.cholesky(np.linalg.inv(M))
        if np.count_nonzero(M - np.diag(np.diag(M))):
            return None, M.sum(axis=0), L
        return np.diag(L).copy(), M.sum(axis=0), None

    def local_params(self, n_dim, device):
        key = (n_dim, str(device))
        if key not in self._cache:
            ms, mc, L = self.metric_vectors(n_dim)
            tms = None if ms is None else torch.tensor(ms, dtype=torch.float32, device=device)
            tmc = None if mc is None else torch.tensor(mc, dtype=torch.float32, device=device)
            tl = None if L is None else torch.tensor(L, dtype=torch.float32, device=device).contiguous()
            self._cache[key] = (tms, tmc, tl)
        tms, tmc, tl = self._cache[key]
        p = _lib.FmcLocalParams()
        p.kind = self.kernel_kind
        p.n_leapfrog = int(self.n_leapfrog)
        p.step_size = float(self.step_size)
        p.lanes_per_chain = int(self.lanes_per_chain)
        p.philox_rounds = int(self.philox_rounds)
        p.momentum_scale = _lib.ptr(tms) if tms is not None else None
        p.metric_colsum = _lib.ptr(tmc) if tmc is not None else None
        p.momentum_chol = _lib.ptr(tl) if tl is not None else None
        return p, [tms, tmc, tl]

    def print_parameters(self):
        print("HMC parameters:")
        print(f"step_size: {self.step_size}")
        print(f"n_leapfrog: {self.n_leapfrog}")
        print(f"condition_matrix: {self.condition_matrix}")

    def save_resource(self, path):
        raise NotImplementedError

    def load_resource(self, path):
        raise NotImplementedError
