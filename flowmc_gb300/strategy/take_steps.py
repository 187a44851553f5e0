"""TakeSteps / TakeSerialSteps / TakeGroupSteps (mirrors
strategy/take_steps.py:14-206 of the reference).

The reference vmaps a per-chain scan over all chains in one XLA program
(take_steps.py:126-132). Here one strategy call is one fused launch over all
chains: the local kernels run the whole scan in a persistent kernel
(``run_local_steps``) and NFProposal runs its fused global step, both writing
their thinned rows straight into the resource buffers at the stepper's
cursor. ``chain_batch_size`` is accepted for API compatibility; it never
changes results in the reference (chunks reuse the per-chain keys,
take_steps.py:106-125) and the fused launch needs no chunking.
"""
from __future__ import annotations

from abc import abstractmethod

import torch

from ..profiling import region
from ..random import split
from ..resource.buffers import Buffer
from ..resource.logPDF import as_target
from ..resource.states import State
from .base import Strategy


class TakeSteps(Strategy):
    logpdf_name: str
    kernel_name: str
    state_name: str
    buffer_names: list
    n_steps: int
    current_position: int
    thinning: int
    chain_batch_size: int
    verbose: bool

    def __init__(self, logpdf_name: str, kernel_name: str, state_name: str, buffer_names: list,
                 n_steps: int, thinning: int = 1, chain_batch_size: int = 0, verbose: bool = False,
                 autotune: bool = False):
        self.logpdf_name = logpdf_name
        self.kernel_name = kernel_name
        self.state_name = state_name
        self.buffer_names = buffer_names
        self.n_steps = n_steps
        self.current_position = 0
        self.thinning = thinning
        self.chain_batch_size = chain_batch_size
        self.verbose = verbose
        # measure the local kernel's chain-block shape on the first call
        self.autotune = autotune

    def set_current_position(self, current_position: int):
        self.current_position = current_position

    def _buffers(self, resources):
        state = resources[self.state_name]
        assert isinstance(state, State), "State resource must be a State"
        # the reference's checks and messages (take_steps.py:74-97)
        kinds = ("Position", "Log probability", "Acceptance")
        names = [state.data[b] for b in self.buffer_names[:3]]
        for k, n in zip(kinds, names):
            assert isinstance(n, str), f"{k} buffer resource name must be a string"
        bufs = [resources[n] for n in names]
        for k, b in zip(kinds, bufs):
            assert isinstance(b, Buffer), f"{k} buffer resource must be a Buffer"
            assert b.cursor_dim == 1, "chain buffers are written along axis 1"
        return bufs

    @abstractmethod
    def sample(self, kernel, seed: int, initial_position: torch.Tensor, target, bufs, cursor: int,
               data: dict, noise=None, uniform=None) -> torch.Tensor:
        raise NotImplementedError

    def __call__(self, rng_key, resources, initial_position, data, noise=None, uniform=None):
        rng_key, subkey = split(rng_key)                       # take_steps.py:71
        bufs = self._buffers(resources)
        kernel = resources[self.kernel_name]
        target = as_target(resources[self.logpdf_name])
        x0 = torch.atleast_2d(initial_position).to(torch.float32).contiguous()
        last = self.sample(kernel, subkey.value, x0, target, bufs, self.current_position, data,
                           noise=noise, uniform=uniform)
        self.current_position += self.n_steps // self.thinning   # take_steps.py:143
        return rng_key, resources, last


class TakeSerialSteps(TakeSteps):
    """n_steps of a local kernel, one after the other (take_steps.py:147-180),
    as one persistent fused launch."""

    def sample(self, kernel, seed, initial_position, target, bufs, cursor, data, noise=None, uniform=None):
        from ..resource.kernel.base import LocalKernel, run_local_steps
        if not isinstance(kernel, LocalKernel):
            raise TypeError(f"{type(kernel).__name__} is not a local kernel")
        pos, lp, acc = bufs
        if getattr(self, "autotune", False) and not getattr(kernel, "_tuned", False):
            from ..autotune import tune_local_kernel
            tune_local_kernel(kernel, target, initial_position.shape[0])
            kernel._tuned = True
        with region("local_steps", units=initial_position.shape[0] * self.n_steps):
            x_last, _ = run_local_steps(kernel, target, initial_position, self.n_steps, self.thinning, seed, 0,
                                        pos.data, lp.data, acc.data, cursor, noise=noise, uniform=uniform)
        return x_last

    def prepare(self, resources, n_chains: int):
        """One-time work that must not run inside a CUDA graph capture: the
        autotuner's timed probes (they synchronise)."""
        from ..resource.kernel.base import LocalKernel
        kernel = resources[self.kernel_name]
        if self.autotune and isinstance(kernel, LocalKernel) and not getattr(kernel, "_tuned", False):
            from ..autotune import tune_local_kernel
            tune_local_kernel(kernel, as_target(resources[self.logpdf_name]), n_chains)
            kernel._tuned = True


class TakeGroupSteps(TakeSteps):
    """n_steps proposals drawn at once (take_steps.py:183-206): the NFProposal
    global step. With ``autotune`` the flow's GEMM tile width is measured on
    the first call (autotune.tune_flow_gemm)."""

    def _tune(self, kernel, n_chains):
        model = getattr(kernel, "model", None)
        if self.autotune and model is not None and not getattr(model, "_gemm_tuned", False):
            from ..autotune import tune_flow_gemm
            tune_flow_gemm(model, min(65536, max(128, n_chains * self.n_steps)))
            model._gemm_tuned = True

    def prepare(self, resources, n_chains: int):
        """The GEMM tile probe, which synchronises, outside any graph capture."""
        self._tune(resources[self.kernel_name], n_chains)

    def sample(self, kernel, seed, initial_position, target, bufs, cursor, data, noise=None, uniform=None):
        self._tune(kernel, initial_position.shape[0])
        pos, lp, acc = bufs
        with region("nf_global", units=initial_position.shape[0] * self.n_steps):
            return kernel.group_steps(seed, initial_position, target, self.n_steps, self.thinning,
                                      pos.data, lp.data, acc.data, cursor, noise=noise, uniform=uniform)
