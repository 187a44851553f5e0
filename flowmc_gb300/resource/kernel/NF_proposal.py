"""NFProposal (mirrors resource/kernel/NF_proposal.py:15-184 of the reference).

``group_steps`` runs the whole global step for every chain through
``fmc_nf_global_steps`` (MaskedCouplingRQSpline; other flows such as
RealNVP make their proposals with their own sample / log_prob launches and
share the fused accept scan, ``fmc_nf_accept``): n_steps flow proposals per chain, their flow
log-density (recomputed by the forward pass, NF_proposal.py:165-166) and
target log-density, and the sequential independent-MH scan
(NF_proposal.py:91-126), writing straight into the buffers.
``n_NFproposal_batch_size`` only chunks the reference's JAX evaluation
(NF_proposal.py:50-89, 135-163) and so only changes its key stream; the
fused step needs no chunking and keeps the attribute for API compatibility.
"""
from __future__ import annotations

import ctypes

import torch

from ... import _lib
from ...random import PRNGKey
from ..logPDF import as_target
from .base import ProposalBase


class NFProposal(ProposalBase):
    def __repr__(self):
        return "NF proposal with " + self.model.__repr__()

    def __init__(self, model, n_NFproposal_batch_size: int = 100):
        super().__init__()
        self.model = model
        self.n_batch_size = n_NFproposal_batch_size
        self._ws = _lib.Workspace()

    def group_steps(self, seed: int, x0: torch.Tensor, target, n_steps: int, thinning: int, out_pos, out_logp,
                    out_acc, cursor: int, noise=None, uniform=None, x_last=None, lp_last=None, counter: int = 0):
        x0 = _lib.require_cuda_f32(x0, "initial_position")
        C, d = x0.shape
        buf_len = out_pos.shape[1]
        _lib.require_cuda_f32(out_pos, "position buffer", (C, buf_len, d))
        _lib.require_cuda_f32(out_logp, "log_prob buffer", (C, buf_len))
        _lib.require_cuda_f32(out_acc, "acceptance buffer", (C, buf_len))
        if noise is not None:
            _lib.require_cuda_f32(noise, "noise", (C, n_steps, d))
        if uniform is not None:
            _lib.require_cuda_f32(uniform, "uniform", (C, n_steps))
        if x_last is None:
            x_last = torch.empty_like(x0)
        if lp_last is None:
            lp_last = torch.empty(C, device=x0.device)
        if not hasattr(self.model, "num_bins"):
            return self._group_steps_generic(seed, x0, target, n_steps, thinning, out_pos, out_logp, out_acc,
                                             cursor, noise, uniform, x_last, lp_last, counter)
        fs = self.model.c_struct()
        nb = ctypes.c_size_t()
        L = _lib.lib()
        _lib.check(L.fmc_nf_workspace_size(ctypes.byref(fs), C, int(n_steps), ctypes.byref(nb)))
        ptr, size = self._ws.get(nb.value, x0.device)
        tgt = target.c_struct()
        _lib.check(L.fmc_nf_global_steps(
            ctypes.byref(fs), ctypes.byref(tgt), x0.data_ptr(), C, int(n_steps), int(thinning),
            int(seed) & ((1 << 64) - 1), int(counter), _lib.ptr(noise), _lib.ptr(uniform), out_pos.data_ptr(),
            out_logp.data_ptr(), out_acc.data_ptr(), buf_len, int(cursor), x_last.data_ptr(), lp_last.data_ptr(),
            ptr, size, _lib.stream_handle(x0.device)))
        return x_last

    def _group_steps_generic(self, seed, x0, target, n_steps, thinning, out_pos, out_logp, out_acc, cursor, noise,
                             uniform, x_last, lp_last, counter):
        """Flows without a fused global step (RealNVP): the model's own sample
        and log_prob launches make the proposals and their densities
        (NF_proposal.py:130-172), then the fused accept scan."""
        C, d = x0.shape
        rows = C * int(n_steps)
        z = None if noise is None else noise.reshape(rows, d)
        props = self.model.sample(PRNGKey._raw(int(seed) ^ int(counter)), rows, z=z)
        lnf = self.model.log_prob(torch.cat([props, x0], 0))
        tgt = target.c_struct()
        _lib.check(_lib.lib().fmc_nf_accept(
            ctypes.byref(tgt), x0.data_ptr(), C, int(n_steps), int(thinning), int(seed) & ((1 << 64) - 1),
            int(counter), props.data_ptr(), lnf.data_ptr(), _lib.ptr(uniform), out_pos.data_ptr(),
            out_logp.data_ptr(), out_acc.data_ptr(), out_pos.shape[1], int(cursor), x_last.data_ptr(),
            lp_last.data_ptr(), _lib.stream_handle(x0.device)))
        return x_last

    def kernel(self, rng_key: PRNGKey, position, log_prob, logpdf, data):
        """NFProposal.kernel for one chain ([d]) or a batch ([C, d]):
        data["n_steps"] proposals; returns (positions, log_probs, accepts)
        with a leading step axis per chain."""
        n_steps = int(data["n_steps"])
        single = position.dim() == 1
        x0 = (position.reshape(1, -1) if single else position).to(torch.float32).contiguous()
        C, d = x0.shape
        pos = torch.empty(C, n_steps, d, device=x0.device)
        lp = torch.empty(C, n_steps, device=x0.device)
        acc = torch.empty(C, n_steps, device=x0.device)
        self.group_steps(rng_key.value, x0, as_target(logpdf), n_steps, 1, pos, lp, acc, 0,
                         noise=data.get("noise"), uniform=data.get("uniform"))
        out = (pos, lp, acc > 0.5)
        return tuple(o[0] for o in out) if single else out

    def sample_flow(self, rng_key: PRNGKey, n_steps: int):
        """(proposals [n_steps, d], their flow log_prob) (NF_proposal.py:130-172)."""
        props = self.model.sample(rng_key, n_steps)
        return props, self.model.log_prob(props)

    def print_parameters(self):
        raise NotImplementedError

    def save_resource(self, path):
        raise NotImplementedError

    def load_resource(self, path):
        raise NotImplementedError
