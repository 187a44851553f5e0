"""Gaussian random walk kernel (mirrors resource/kernel/Gaussian_random_walk.py:10-71).

Proposal x + sigma xi, accept iff log(u) < logpdf(prop) - log_prob
(Gaussian_random_walk.py:48-61); the step runs in the fused local-step kernel.
"""
from __future__ import annotations

from ... import _lib
from .base import LocalKernel


class GaussianRandomWalk(LocalKernel):
    """Gaussian random walk sampler class."""

    kernel_kind = _lib.KERNEL_GRW

    def __repr__(self):
        return "Gaussian Random Walk with step size " + str(self.step_size)

    def __init__(self, step_size):
        super().__init__()
        self.step_size = step_size

    def local_params(self, n_dim, device):
        p = _lib.FmcLocalParams()
        p.kind = self.kernel_kind
        p.step_size = float(self.step_size)
        p.lanes_per_chain = int(self.lanes_per_chain)
        p.philox_rounds = int(self.philox_rounds)
        return p, []

    def print_parameters(self):
        print("Gaussian Random Walk parameters:")
        print(f"step_size: {self.step_size}")

    def save_resource(self, path):
        raise NotImplementedError

    def load_resource(self, path):
        raise NotImplementedError
