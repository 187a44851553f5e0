"""NFModel base (mirrors resource/model/nf_model/base.py:14-245 of the reference).

Training runs on the device with no host synchronisation: the batch
shuffle, the loss and hand-written gradient (fmc_flow_loss_grad), the
clipped AdamW update (fmc_adamw_step) and the best-epoch selection
(fmc_flag_less + fmc_copy_if) are all stream-ordered launches, so a whole
``train`` call can be captured in a CUDA graph.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from .... import _lib
from ....random import split
from ...base import Resource


class NFModel(Resource):
    """Base class for the flow models: subclasses provide theta, aux,
    theta_bf16, c_struct() and the forward/inverse/log_prob/sample passes."""

    def __call__(self, x):
        return self.forward(x)

    # ---------------------------------------------------------------- loss
    def loss_and_grad(self, x: torch.Tensor, loss: torch.Tensor | None = None, grad: torch.Tensor | None = None):
        """loss = -mean(log_prob(x)) and its gradient w.r.t. theta
        (nf_model/base.py:98-100), both on the device."""
        x = _lib.require_cuda_f32(torch.as_tensor(x).contiguous(), "x")
        n = x.shape[0]
        s = self.c_struct()
        nb = ctypes.c_size_t()
        _lib.check(_lib.lib().fmc_flow_workspace_size(ctypes.byref(s), n, 1, ctypes.byref(nb)))
        if not hasattr(self, "_ws_train"):
            self._ws_train = _lib.Workspace()
        ptr, size = self._ws_train.get(nb.value, self.device)
        if loss is None:
            loss = torch.empty((), device=self.device)
        if grad is None:
            grad = torch.empty(self.n_params, device=self.device)
        _lib.check(_lib.lib().fmc_flow_loss_grad(ctypes.byref(s), x.data_ptr(), n, loss.data_ptr(), grad.data_ptr(),
                                                 ptr, size, _lib.stream_handle(self.device)))
        return loss, grad

    # ---------------------------------------------------------------- train
    def train_step(self, x, optim, state):
        """One optimiser step (nf_model/base.py:102-125); returns the loss tensor."""
        loss, grad = self.loss_and_grad(x)
        optim.apply(self, grad, state)
        return loss

    def train(self, rng, data, optim, state, num_epochs: int, batch_size: int, verbose: bool = True):
        """NFModel.train (nf_model/base.py:153-210). ``optim`` is the
        Optimizer resource and ``state`` its state (Optimizer.optim_state).
        Returns (rng, best_model, best_state, loss_values); the model and the
        state are updated in place and the best epoch's values restored."""
        data = _lib.require_cuda_f32(torch.as_tensor(data).contiguous(), "data")
        N, d = data.shape
        dev = self.device
        stream = _lib.stream_handle(dev)
        L = _lib.lib()
        loss_values = torch.zeros(num_epochs, device=dev)
        best_loss = torch.full((), 1e9, device=dev)
        flag = torch.zeros((), dtype=torch.int32, device=dev)
        snap = [(self.theta, self.theta.clone()), (self.aux, self.aux.clone())] + \
               [(t, t.clone()) for t in state.tensors()]
        # nf_model/base.py:187-188: data_mean / data_cov from the training data
        if N >= 2:
            if getattr(self, "_colstat_ws", None) is None:
                self._colstat_ws = _lib.Workspace()
            _lib.column_stats(data, self.aux[:d], self.aux[d:2 * d], self._colstat_ws)
        steps = N // batch_size
        batch = torch.empty(batch_size if steps > 0 else N, d, device=dev)
        grad = torch.empty(self.n_params, device=dev)
        loss = torch.empty((), device=dev)
        for epoch in range(num_epochs):
            rng, input_rng = split(rng)
            if steps > 0:
                for b in range(steps):
                    _lib.check(L.fmc_permute_rows(data.data_ptr(), N, d, input_rng.value, 0, b * batch_size,
                                                  batch_size, batch.data_ptr(), stream))
                    self.loss_and_grad(batch, loss, grad)
                    optim.apply(self, grad, state)
            else:
                self.loss_and_grad(data, loss, grad)
                optim.apply(self, grad, state)
            loss_values[epoch].copy_(loss)
            _lib.check(L.fmc_flag_less(loss.data_ptr(), best_loss.data_ptr(), flag.data_ptr(), stream))
            for cur, best in snap:
                _lib.check(L.fmc_copy_if(flag.data_ptr(), cur.data_ptr(), best.data_ptr(),
                                         cur.numel() * cur.element_size(), stream))
        for cur, best in snap:
            cur.copy_(best)
        self.sync_bf16()
        if verbose:
            print(f"Training NF, final losses: {loss_values.detach().cpu().numpy()}")
        return rng, self, state, loss_values

    # ---------------------------------------------------------------- persistence
    def save_model(self, path: str):
        """The reference's checkpoint (nf_model/base.py:92-93): an equinox
        tree_serialise_leaves file at path + ".eqx"."""
        from .eqx_format import save_eqx
        save_eqx(self, path + ".eqx")

    def load_model(self, path: str):
        """Load a reference checkpoint (nf_model/base.py:95-96) into this model
        (same architecture); returns the model."""
        from .eqx_format import load_eqx
        return load_eqx(self, path if path.endswith(".eqx") else path + ".eqx")

    def save_npz(self, path: str):
        """Exact device state (flat parameters and the aux block) as .npz."""
        full = self.to_full()
        arrs = {"aux": self.aux.detach().cpu().numpy()}
        for l, Lr in enumerate(full):
            arrs[f"l{l}_scale"] = np.asarray(Lr["scale"])
            arrs[f"l{l}_shift"] = np.asarray(Lr["shift"])
            for i, (W, b) in enumerate(zip(Lr["W"], Lr["b"])):
                arrs[f"l{l}_W{i}"] = W
                arrs[f"l{l}_b{i}"] = b
        np.savez(path + ".npz", **arrs)

    def load_npz(self, path: str):
        z = np.load(path if path.endswith(".npz") else path + ".npz")
        layers = []
        for l in range(self.n_layers):
            nl = len(self.hidden_size) + 1
            layers.append({"W": [z[f"l{l}_W{i}"] for i in range(nl)], "b": [z[f"l{l}_b{i}"] for i in range(nl)],
                           "scale": float(z[f"l{l}_scale"]), "shift": float(z[f"l{l}_shift"])})
        self.load_full(layers)
        self.aux.copy_(torch.as_tensor(z["aux"]))
        return self

    save_resource = save_model
    load_resource = load_model
