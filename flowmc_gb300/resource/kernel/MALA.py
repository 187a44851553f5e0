"""MALA kernel (mirrors resource/kernel/MALA.py:11-99 of the reference).

The step itself runs in the fused local-step kernel (csrc/local_steps.cuh):
proposal x + dt^2 grad/2 + dt xi, the two isotropic Gaussian proposal
densities in the log-ratio, accept iff log(u) < ratio (MALA.py:26-89).
"""
from __future__ import annotations

from ... import _lib
from .base import LocalKernel


class MALA(LocalKernel):
    """Metropolis-adjusted Langevin algorithm sampler class."""

    kernel_kind = _lib.KERNEL_MALA

    def __repr__(self):
        return "MALA with step size " + str(self.step_size)

    def __init__(self, step_size):
        super().__init__()
        self.step_size = step_size

    def local_params(self, n_dim, device):
        p = _lib.FmcLocalParams()
        p.kind = self.kernel_kind
        p.n_leapfrog = 0
        p.step_size = float(self.step_size)
        p.lanes_per_chain = int(self.lanes_per_chain)
        p.philox_rounds = int(self.philox_rounds)
        return p, []

    def print_parameters(self):
        print("MALA parameters:")
        print(f"step_size: {self.step_size}")

    def save_resource(self, path):
        raise NotImplementedError

    def load_resource(self, path):
        raise NotImplementedError
