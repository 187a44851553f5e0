"""TrainModel strategy (mirrors strategy/train_model.py:12-112 of the reference).

The training-data selection (finite rows, per-chain history window,
with-replacement resampling, train_model.py:66-80) runs on the device
(fmc_select_training_data) instead of boolean-mask indexing, so no host sync
is needed; the epoch losses land in the loss buffer with a device copy.
"""
from __future__ import annotations

import ctypes

import torch

from .. import _lib
from ..profiling import region
from ..random import split
from ..resource.buffers import Buffer
from ..resource.model.nf_model.base import NFModel
from ..resource.optimizer import Optimizer
from .base import Strategy


class TrainModel(Strategy):
    def __repr__(self):
        return "Train " + self.model_resource

    def __init__(self, model_resource: str, data_resource: str, optimizer_resource: str, loss_buffer_name: str = "",
                 n_epochs: int = 100, batch_size: int = 64, n_max_examples: int = 10000, history_window: int = 100,
                 verbose: bool = False, autotune: bool = False):
        self.model_resource = model_resource
        self.data_resource = data_resource
        self.optimizer_resource = optimizer_resource
        self.loss_buffer_name = loss_buffer_name
        self.n_epochs = n_epochs
        self.batch_size = batch_size
        self.n_max_examples = n_max_examples
        self.verbose = verbose
        self.history_window = history_window
        self.autotune = autotune   # time the BF16 weight-gradient split (autotune.tune_flow_train) once
        self._ws = _lib.Workspace()
        self._err = None
        self._err_host = None     # pinned copy of the device error word
        self._err_event = None    # recorded after the copy (eager runs and graph replays)

    def select(self, seed: int, buf: torch.Tensor, idx: torch.Tensor | None = None) -> torch.Tensor:
        C, S, d = buf.shape
        dev = buf.device
        nb = ctypes.c_size_t()
        L = _lib.lib()
        _lib.check(L.fmc_select_workspace_size(C, S, ctypes.byref(nb)))
        ptr, size = self._ws.get(nb.value, dev)
        self._error_words(dev)
        out = torch.empty(self.n_max_examples, d, device=dev)
        _lib.check(L.fmc_select_training_data(buf.data_ptr(), C, S, d, self.history_window, self.n_max_examples,
                                              int(seed) & ((1 << 64) - 1), 0, _lib.ptr(idx), out.data_ptr(),
                                              self._err.data_ptr(), ptr, size, _lib.stream_handle(dev)))
        # the error word goes to pinned host memory behind the selection (a
        # copy node when captured), so that a later poll needs no stream sync
        self._err_host.copy_(self._err, non_blocking=True)
        if not torch.cuda.is_current_stream_capturing():
            self.mark_error_copy()
        return out

    _MSG = "finite training rows do not split evenly over the chains"

    def _error_words(self, dev):
        """The device error word and its pinned host copy (allocated outside
        any CUDA-graph capture: Sampler.capture calls prepare first)."""
        if self._err is None or self._err.device != dev:
            self._err = torch.zeros((), dtype=torch.int32, device=dev)
        if self._err_host is None:
            self._err_host = torch.zeros((), dtype=torch.int32, pin_memory=True)

    def prepare(self, resources, n_chains):
        """Before a CUDA-graph capture: allocate what select() needs, and with
        ``autotune`` time the BF16 weight-gradient split (it synchronises)."""
        self._error_words(resources[self.data_resource].data.device)
        self._tune(resources[self.model_resource])

    def _tune(self, model):
        if getattr(self, "autotune", False) and not getattr(model, "_train_tuned", False):
            from ..autotune import tune_flow_train
            tune_flow_train(model, min(self.batch_size, self.n_max_examples))
            model._train_tuned = True

    def mark_error_copy(self, event=None):
        """Record (or take) the event after which the pinned error word is valid."""
        if event is None:
            event = torch.cuda.Event()
            event.record()
        self._err_event = event

    def poll_errors(self):
        """Raise ValueError if a finished selection found finite rows that do
        not split evenly over the chains (the reference's reshape would raise
        there; the selection then fills the training data with NaN). Waits
        only for the event recorded after that selection's copy, not for the
        stream."""
        ev = self._err_event
        if ev is None or self._err_host is None:
            return
        ev.synchronize()
        self._err_event = None
        if int(self._err_host.item()) != 0:
            self._err_host.zero_()
            self._err.zero_()
            raise ValueError(self._MSG)

    def check_errors(self):
        """Raise if a selection found finite rows that do not split evenly over
        the chains (the reference's reshape would raise). Synchronises."""
        if self._err is not None and int(self._err.item()) != 0:
            self._err.zero_()
            if self._err_host is not None:
                self._err_host.zero_()
            self._err_event = None
            raise ValueError(self._MSG)

    def __call__(self, rng_key, resources, initial_position, data):
        model = resources[self.model_resource]
        assert isinstance(model, NFModel), "Target resource must be a NFModel"
        data_resource = resources[self.data_resource]
        assert isinstance(data_resource, Buffer), "Data resource must be a buffer"
        optimizer = resources[self.optimizer_resource]
        assert isinstance(optimizer, Optimizer), "Optimizer resource must be an optimizer"
        if not torch.cuda.is_current_stream_capturing():
            self.poll_errors()      # the previous call's selection, long finished
            self._tune(model)
        rng_key, subkey = split(rng_key)                              # train_model.py:72
        training_data = self.select(subkey.value, data_resource.data)
        rng_key, subkey = split(rng_key)                              # train_model.py:81
        if self.verbose:
            print("Training model")
            print(f"Training data shape: {tuple(training_data.shape)}")
            print(f"n_epochs: {self.n_epochs}")
            print(f"batch_size: {self.batch_size}")
        # the key returned by NFModel.train replaces rng_key (train_model.py:81-97)
        with region("train", units=self.n_epochs * max(1, self.n_max_examples // self.batch_size)):
            rng_key, model, state, loss_values = model.train(subkey, training_data, optimizer,
                                                             optimizer.optim_state, self.n_epochs, self.batch_size,
                                                             verbose=self.verbose)
        if self.loss_buffer_name != "":
            loss_buffer = resources[self.loss_buffer_name]
            assert isinstance(loss_buffer, Buffer), "Loss buffer resource must be a buffer"
            loss_buffer.update_buffer(loss_values, start=loss_buffer.cursor)
            loss_buffer.cursor += len(loss_values)
        optimizer.optim_state = state
        resources[self.model_resource] = model
        resources[self.optimizer_resource] = optimizer
        return rng_key, resources, initial_position
