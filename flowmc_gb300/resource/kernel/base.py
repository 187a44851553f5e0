"""ProposalBase (mirrors resource/kernel/base.py:9-27 of the reference) and
the launcher shared by the local kernels.

``ProposalBase.kernel(rng_key, position, log_prob, logpdf, data)`` keeps the
reference's signature; it accepts one chain ([n_dim]) or a batch
([n_chains, n_dim]) and runs one step through the C ABI. Strategies do not
call it per step: they hand whole phases to ``run_local_steps``, one
persistent launch per call.
"""
from __future__ import annotations

import ctypes
from abc import abstractmethod

import torch

from ... import _lib
from ...random import PRNGKey
from ..base import Resource
from ..logPDF import as_target


class ProposalBase(Resource):
    @abstractmethod
    def __init__(self):
        """Initialise the kernel."""

    @abstractmethod
    def kernel(self, rng_key, position, log_prob, logpdf, data):
        """One step of the proposal cycle."""


class LocalKernel(ProposalBase):
    """A kernel the fused local-step launch can run (MALA, HMC, GRW)."""

    kernel_kind: int
    lanes_per_chain: int = 0   # 0 = library default; set by the autotuner
    philox_rounds: int = 10    # in-kernel noise generator: Philox-4x32-10, or 7 (opt-in, another stream)

    def local_params(self, n_dim: int, device) -> tuple[_lib.FmcLocalParams, list]:
        raise NotImplementedError

    def kernel(self, rng_key: PRNGKey, position, log_prob, logpdf, data=None, noise=None, uniform=None):
        single = position.dim() == 1
        x0 = position.reshape(1, -1) if single else position
        x0 = _lib.require_cuda_f32(x0.contiguous(), "position")
        C, d = x0.shape
        lp0 = None
        if log_prob is not None:
            lp0 = torch.as_tensor(log_prob, dtype=torch.float32, device=x0.device).reshape(-1)
            lp0 = lp0.expand(C).contiguous() if lp0.numel() == 1 else lp0.contiguous()
        pos = torch.empty(C, 1, d, device=x0.device)
        lp = torch.empty(C, 1, device=x0.device)
        acc = torch.empty(C, 1, device=x0.device)
        if noise is not None:
            noise = noise.reshape(C, 1, d).contiguous()
        if uniform is not None:
            uniform = torch.as_tensor(uniform, dtype=torch.float32, device=x0.device).reshape(C, 1).contiguous()
        run_local_steps(self, as_target(logpdf), x0, 1, 1, rng_key.value, 0, pos, lp, acc, 0,
                        lp0=lp0, noise=noise, uniform=uniform)
        out = (pos[:, 0], lp[:, 0], acc[:, 0] > 0.5)
        if single:
            return out[0][0], out[1][0], out[2][0]
        return out


def run_local_steps(kernel: LocalKernel, target, x0: torch.Tensor, n_steps: int, thinning: int,
                    seed: int, counter: int, out_pos: torch.Tensor, out_logp: torch.Tensor,
                    out_acc: torch.Tensor, cursor: int, lp0=None, noise=None, uniform=None,
                    x_last=None, lp_last=None):
    """One fmc_local_steps launch; returns (x_last [C, d], lp_last [C])."""
    x0 = _lib.require_cuda_f32(x0, "initial_position")
    C, d = x0.shape
    if d != target.n_dim:
        raise ValueError(f"positions have {d} coordinates, target has {target.n_dim}")
    buf_len = out_pos.shape[1]
    _lib.require_cuda_f32(out_pos, "position buffer", (C, buf_len, d))
    _lib.require_cuda_f32(out_logp, "log_prob buffer", (C, buf_len))
    _lib.require_cuda_f32(out_acc, "acceptance buffer", (C, buf_len))
    if noise is not None:
        _lib.require_cuda_f32(noise, "noise", (C, n_steps, d))
    if uniform is not None:
        _lib.require_cuda_f32(uniform, "uniform", (C, n_steps))
    if lp0 is not None:
        _lib.require_cuda_f32(lp0, "log_prob", (C,))
    if x_last is None:
        x_last = torch.empty_like(x0)
    if lp_last is None:
        lp_last = torch.empty(C, device=x0.device)
    tgt = target.c_struct()
    prm, keep = kernel.local_params(d, x0.device)
    _lib.check(_lib.lib().fmc_local_steps(
        ctypes.byref(tgt), ctypes.byref(prm), x0.data_ptr(), _lib.ptr(lp0), C, int(n_steps), int(thinning),
        int(seed) & ((1 << 64) - 1), int(counter), _lib.ptr(noise), _lib.ptr(uniform), out_pos.data_ptr(),
        out_logp.data_ptr(), out_acc.data_ptr(), buf_len, int(cursor), x_last.data_ptr(), lp_last.data_ptr(),
        _lib.stream_handle(x0.device)))
    del keep
    return x_last, lp_last
