"""ParallelTempering (mirrors strategy/parallel_tempering.py:13-436 of the
reference).

The reference vmaps, per chain, a vmap over temperatures of a scan of local
kernel steps on the tempered density, then a per-chain scan of adjacent
swaps, then adapts the temperatures (parallel_tempering.py:47-133). Here one
call is three launches over the whole [n_chains, n_temps] ensemble:

  pt_local_steps   the fused local-step kernel over the n_chains * n_temps
                   (chain, temperature) rows, row c at inverse temperature
                   1 / temps[c % n_temps], keeping only each row's end state
  pt_exchange      per chain: log L at every temperature, the sequential swap
                   sweep, the rows written out in their new order (the T = 1
                   row as the chain position, the rest into the
                   tempered-positions buffer while training)
  pt_adapt_temperatures
                   the damping update from exact per-pair swap counts,
                   written back into the temperature buffer on the device

Nothing is read back to the host unless ``verbose`` asks for the acceptance
printouts.
"""
from __future__ import annotations

import ctypes

import torch

from .. import _lib
from ..profiling import region
from ..random import split
from ..resource.buffers import Buffer
from ..resource.logPDF import TemperedPDF
from ..resource.states import State
from .base import Strategy


def pt_local_steps(kernel, tempered_logpdf: TemperedPDF, x: torch.Tensor, temperatures: torch.Tensor,
                   n_steps: int, seed: int, counter: int = 0, noise=None, uniform=None, x_last=None, lp_last=None,
                   acc_count=None):
    """_ensemble_step for every chain (parallel_tempering.py:250-289).

    x [C, T, d]; temperatures [T] (device); noise [C, T, n_steps, d] and
    uniform [C, T, n_steps] or None (in-kernel Philox). Returns the last
    positions [C, T, d], their tempered log-densities [C, T] and, when
    ``acc_count`` is given, the accepted steps per row [C, T].
    """
    from ..resource.kernel.base import LocalKernel
    if not isinstance(kernel, LocalKernel):
        raise TypeError(f"{type(kernel).__name__} is not a local kernel")
    x = _lib.require_cuda_f32(x, "positions")
    if x.dim() != 3:
        raise ValueError("positions must be [n_chains, n_temps, n_dim]")
    C, T, d = x.shape
    target = tempered_logpdf.target
    if d != target.n_dim:
        raise ValueError(f"positions have {d} coordinates, target has {target.n_dim}")
    _lib.require_cuda_f32(temperatures, "temperatures", (T,))
    if noise is not None:
        _lib.require_cuda_f32(noise, "noise", (C, T, n_steps, d))
    if uniform is not None:
        _lib.require_cuda_f32(uniform, "uniform", (C, T, n_steps))
    if x_last is None:
        x_last = torch.empty_like(x)
    if lp_last is None:
        lp_last = torch.empty(C, T, device=x.device)
    prior = tempered_logpdf.prior_arrays(x.device)
    pm, piv, pc = (prior if prior is not None else (None, None, 0.0))
    tgt = target.c_struct()
    prm, keep = kernel.local_params(d, x.device)
    _lib.check(_lib.lib().fmc_pt_local_steps(
        ctypes.byref(tgt), ctypes.byref(prm), x.data_ptr(), C, T, temperatures.data_ptr(), _lib.ptr(pm),
        _lib.ptr(piv), float(pc), int(n_steps), int(seed) & ((1 << 64) - 1), int(counter), _lib.ptr(noise),
        _lib.ptr(uniform), x_last.data_ptr(), lp_last.data_ptr(), _lib.ptr(acc_count),
        _lib.stream_handle(x.device)))
    del keep, prior
    return x_last, lp_last, acc_count


def pt_exchange(target, x: torch.Tensor, temperatures: torch.Tensor, seed: int, counter: int = 0, uniform=None,
                out_first=None, out_rest=None, out_logp=None, out_acc=None, acc_pairs=None):
    """_exchange for every chain (parallel_tempering.py:291-398).

    x [C, T, d] (not modified); uniform [C, T-1] or None (Philox). Writes the
    swept positions to out_first [C, d] and, if given, out_rest [C, T-1, d];
    returns (out_first, out_logp, out_acc, acc_pairs) with acc_pairs [T-1]
    int32 swap counts.
    """
    x = _lib.require_cuda_f32(x, "positions")
    C, T, d = x.shape
    if out_first is None:
        out_first = torch.empty(C, d, device=x.device)
    if acc_pairs is None:
        acc_pairs = torch.empty(max(T - 1, 1), dtype=torch.int32, device=x.device)
    _lib.require_cuda_f32(out_first, "chain positions", (C, d))
    if out_rest is not None:
        _lib.require_cuda_f32(out_rest, "tempered positions", (C, T - 1, d))
    if out_logp is not None:
        _lib.require_cuda_f32(out_logp, "log_probs", (C, T))
    if out_acc is not None:
        _lib.require_cuda_f32(out_acc, "swap flags", (C, T - 1))
    if uniform is not None:
        _lib.require_cuda_f32(uniform, "uniform", (C, T - 1))
    tgt = target.c_struct()
    _lib.check(_lib.lib().fmc_pt_exchange(
        ctypes.byref(tgt), x.data_ptr(), C, T, temperatures.data_ptr(), int(seed) & ((1 << 64) - 1), int(counter),
        _lib.ptr(uniform), out_first.data_ptr(), _lib.ptr(out_rest), _lib.ptr(out_logp), _lib.ptr(out_acc),
        acc_pairs.data_ptr(), _lib.stream_handle(x.device)))
    return out_first, out_logp, out_acc, acc_pairs


def pt_adapt_temperatures(temperatures: torch.Tensor, acc_pairs: torch.Tensor, n_chains: int, out=None):
    """_adapt_temperature (parallel_tempering.py:400-436) on the device;
    ``out`` may be ``temperatures`` itself."""
    T = temperatures.shape[0]
    if out is None:
        out = torch.empty_like(temperatures)
    _lib.check(_lib.lib().fmc_pt_adapt_temperatures(
        temperatures.data_ptr(), acc_pairs.data_ptr(), int(n_chains), T, out.data_ptr(),
        _lib.stream_handle(temperatures.device)))
    return out


class ParallelTempering(Strategy):
    """Sample a tempered PDF with one exchange step (parallel_tempering.py:13-133).

    Tempered positions and temperatures are updated only while the sampler
    state's ``training`` flag is set, as in the reference."""

    n_steps: int
    tempered_logpdf_name: str
    kernel_name: str
    tempered_buffer_names: list
    verbose: bool = False

    def __init__(self, n_steps: int, tempered_logpdf_name: str, kernel_name: str, tempered_buffer_names: list,
                 state_name: str, verbose: bool = False):
        self.n_steps = n_steps
        self.tempered_logpdf_name = tempered_logpdf_name
        self.kernel_name = kernel_name
        self.tempered_buffer_names = tempered_buffer_names
        self.verbose = verbose
        self.state_name = state_name
        self._ws = None

    def _workspace(self, C, T, d, device):
        key = (C, T, d, str(device))
        if self._ws is None or self._ws[0] != key:
            self._ws = (key, {
                "x": torch.empty(C, T, d, device=device),
                "x_last": torch.empty(C, T, d, device=device),
                "lp_last": torch.empty(C, T, device=device),
                "acc_count": torch.empty(C, T, device=device),
                "acc_pairs": torch.empty(max(T - 1, 1), dtype=torch.int32, device=device),
            })
        return self._ws[1]

    def __call__(self, rng_key, resources, initial_position, data):
        rng_key, subkey = split(rng_key)                       # parallel_tempering.py:71
        kernel = resources[self.kernel_name]
        tempered_logpdf = resources[self.tempered_logpdf_name]
        assert isinstance(tempered_logpdf, TemperedPDF), "tempered logpdf resource must be a TemperedPDF"
        tempered_positions = resources[self.tempered_buffer_names[0]]
        temperatures = resources[self.tempered_buffer_names[1]]
        assert isinstance(tempered_positions, Buffer) and isinstance(temperatures, Buffer)
        state = resources[self.state_name]
        assert isinstance(state, State)

        x0 = torch.atleast_2d(initial_position).to(torch.float32)
        C, d = x0.shape
        T = temperatures.data.shape[0]
        if tuple(tempered_positions.data.shape) != (C, T - 1, d):
            raise ValueError(f"tempered positions buffer is {tuple(tempered_positions.data.shape)}, "
                             f"expected {(C, T - 1, d)}")
        ws = self._workspace(C, T, d, x0.device)
        # [C, T, d]: the chain position first, then the tempered ones (parallel_tempering.py:87-90)
        ws["x"][:, 0].copy_(x0)
        ws["x"][:, 1:].copy_(tempered_positions.data)

        rng_key, subkey = split(rng_key)
        with region("pt_local_steps", units=C * T * self.n_steps):
            pt_local_steps(kernel, tempered_logpdf, ws["x"], temperatures.data, self.n_steps, subkey.value,
                           x_last=ws["x_last"], lp_last=ws["lp_last"],
                           acc_count=ws["acc_count"] if self.verbose else None)
        if self.verbose:
            mean_accs = float(ws["acc_count"].sum()) / (C * T * self.n_steps)
            print("Mean acceptance of individual steps in PT: " + str(mean_accs))

        rng_key, subkey = split(rng_key)
        training = bool(state.data["training"])
        first = torch.empty(C, d, device=x0.device)
        with region("pt_exchange", units=C * T):
            # tempered buffer and temperatures change only while training (parallel_tempering.py:123-132)
            pt_exchange(tempered_logpdf.target, ws["x_last"], temperatures.data, subkey.value, out_first=first,
                        out_rest=tempered_positions.data if training else None, acc_pairs=ws["acc_pairs"])
            if training and T > 1:
                pt_adapt_temperatures(temperatures.data, ws["acc_pairs"], C, out=temperatures.data)
        if self.verbose and T > 1:
            mean_accs = float(ws["acc_pairs"][: T - 1].sum()) / (C * (T - 1))
            print("Mean acceptance of exchange steps in PT: " + str(mean_accs))
        return rng_key, resources, first
