"""Optimizer resource (mirrors resource/optimizer.py:8-35 of the reference):
optax.chain(clip_by_global_norm(1.0), optax.adamw(learning_rate, b1=momentum))
run by fmc_adamw_step. b2, eps and weight_decay are optax's adamw defaults
(0.999, 1e-8, 1e-4)."""
from __future__ import annotations

import ctypes

import torch

from .. import _lib
from .base import Resource


class AdamWState:
    """optax state of the chain: first/second moments and the step count."""

    def __init__(self, n: int, device):
        self.m = torch.zeros(n, device=device)
        self.v = torch.zeros(n, device=device)
        self.count = torch.zeros((), dtype=torch.int32, device=device)

    def tensors(self):
        return [self.m, self.v, self.count]


class Optimizer(Resource):
    def __repr__(self):
        return "Optimizer"

    def __init__(self, model, learning_rate: float = 1e-3, momentum: float = 0.9, b2: float = 0.999,
                 eps: float = 1e-8, weight_decay: float = 1e-4, max_norm: float = 1.0):
        self.params = _lib.FmcAdamParams(lr=learning_rate, b1=momentum, b2=b2, eps=eps, weight_decay=weight_decay,
                                         max_norm=max_norm)
        self.optim = self
        self.optim_state = AdamWState(model.n_params, model.device)
        self._ws = _lib.Workspace()

    def apply(self, model, grad: torch.Tensor, state: AdamWState):
        nb = ctypes.c_size_t()
        L = _lib.lib()
        _lib.check(L.fmc_adamw_workspace_size(ctypes.byref(nb)))
        ptr, size = self._ws.get(nb.value, model.device)
        _lib.check(L.fmc_adamw_step(model.theta.data_ptr(), None, grad.data_ptr(), state.m.data_ptr(),
                                    state.v.data_ptr(), model.n_params, model.aux.data_ptr(), model.aux.numel(),
                                    state.count.data_ptr(), ctypes.byref(self.params), ptr, size,
                                    _lib.stream_handle(model.device)))
        if model.precision in ("bf16", "bfloat16"):
            model.sync_bf16()   # re-pack the padded bf16 weights the tensor-core GEMMs read

    def __call__(self, params, grads):
        raise NotImplementedError

    def print_parameters(self):
        raise NotImplementedError

    def save_resource(self, path: str):
        raise NotImplementedError

    def load_resource(self, path: str):
        raise NotImplementedError
