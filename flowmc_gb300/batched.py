"""Many independent dense-Gaussian targets sampled in one persistent launch.

``BatchedDenseLocalSteps`` runs MALA or HMC (identity mass) for the chains of
every target at once through ``fmc_batched_dense_local_steps``: work items
are 32-chain tiles of one target, pulled by the CTAs from a shared counter,
so targets of uneven dimension (1..256) and chain count share the GPU
without per-target launches. Step semantics are TakeSerialSteps with
MALA.kernel / HMC.kernel (strategy/take_steps.py:156-180,
resource/kernel/MALA.py:26-89, HMC.py:98-151).
"""
from __future__ import annotations

import ctypes

import torch

from . import _lib
from .targets import DenseGaussian

_lib.register_extra("fmc_batched_workspace_size", ctypes.c_int,
                    [ctypes.c_int32, ctypes.c_int64, ctypes.POINTER(ctypes.c_size_t)])
_lib.register_extra("fmc_batched_dense_local_steps", ctypes.c_int, [
    ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.POINTER(_lib.FmcLocalParams), ctypes.c_void_p,
    ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p,
    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
    ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p])

D_MAX = 256


class BatchedDenseLocalSteps:
    def __init__(self, targets: list, n_chains: list, step_sizes: list, kind: str = "mala", n_leapfrog: int = 10):
        if kind not in ("mala", "hmc"):
            raise ValueError("kind must be 'mala' or 'hmc'")
        for t in targets:
            if not isinstance(t, DenseGaussian):
                raise TypeError("batched local steps take DenseGaussian targets")
            if t.n_dim > D_MAX:
                raise ValueError(f"n_dim {t.n_dim} > {D_MAX}")
        self.targets = list(targets)
        self.n_chains = [int(c) for c in n_chains]
        self.step_sizes = [float(s) for s in step_sizes]
        self.kind = kind
        self.n_leapfrog = int(n_leapfrog)
        self.offsets = [0]
        for c in self.n_chains:
            self.offsets.append(self.offsets[-1] + c)
        self._ws = _lib.Workspace()

    def pack(self, xs: list) -> torch.Tensor:
        """Per-target positions [C_t, d_t] -> the padded [sum C, 256] layout."""
        dev = xs[0].device
        out = torch.zeros(self.offsets[-1], D_MAX, device=dev)
        for t, x in enumerate(xs):
            out[self.offsets[t]:self.offsets[t + 1], :x.shape[1]] = x
        return out

    def unpack(self, packed: torch.Tensor) -> list:
        return [packed[self.offsets[t]:self.offsets[t + 1], :tg.n_dim] for t, tg in enumerate(self.targets)]

    def run(self, xs: list, n_steps: int, thinning: int = 1, seed: int = 0, counter: int = 0, noise=None,
            uniform=None, buf_len: int | None = None, cursor: int = 0, outputs=None):
        n = len(self.targets)
        dev = xs[0].device
        R = -(-n_steps // thinning)
        buf_len = buf_len or R
        if outputs is None:
            outputs = [(torch.full((c, buf_len, t.n_dim), -float("inf"), device=dev),
                        torch.full((c, buf_len), -float("inf"), device=dev),
                        torch.full((c, buf_len), -float("inf"), device=dev))
                       for t, c in zip(self.targets, self.n_chains)]
        x0 = self.pack(xs)
        x_last = torch.zeros_like(x0)
        lp_last = torch.empty(self.offsets[-1], device=dev)
        tg = (_lib.FmcTarget * n)(*[t.c_struct() for t in self.targets])
        nc = (ctypes.c_int32 * n)(*self.n_chains)
        ss = (ctypes.c_float * n)(*self.step_sizes)
        prm = _lib.FmcLocalParams()
        prm.kind = _lib.KERNEL_MALA if self.kind == "mala" else _lib.KERNEL_HMC
        prm.n_leapfrog = self.n_leapfrog
        ptrs = lambda ts: (ctypes.c_void_p * n)(*[_lib.ptr(t) for t in ts])
        nz = ptrs([z.contiguous() for z in noise]) if noise is not None else None
        un = ptrs([u.contiguous() for u in uniform]) if uniform is not None else None
        keep = [noise, uniform]
        nb = ctypes.c_size_t()
        L = _lib.lib()
        _lib.check(L.fmc_batched_workspace_size(n, self.offsets[-1], ctypes.byref(nb)))
        wptr, wsize = self._ws.get(nb.value, dev)
        _lib.check(L.fmc_batched_dense_local_steps(
            ctypes.cast(tg, ctypes.c_void_p), n, ctypes.cast(nc, ctypes.c_void_p), ctypes.byref(prm),
            ctypes.cast(ss, ctypes.c_void_p), x0.data_ptr(), int(n_steps), int(thinning),
            int(seed) & ((1 << 64) - 1), int(counter), ctypes.cast(nz, ctypes.c_void_p) if nz else None,
            ctypes.cast(un, ctypes.c_void_p) if un else None,
            ctypes.cast(ptrs([o[0] for o in outputs]), ctypes.c_void_p),
            ctypes.cast(ptrs([o[1] for o in outputs]), ctypes.c_void_p),
            ctypes.cast(ptrs([o[2] for o in outputs]), ctypes.c_void_p), buf_len, int(cursor), x_last.data_ptr(),
            lp_last.data_ptr(), wptr, wsize, _lib.stream_handle(dev)))
        del keep
        return outputs, self.unpack(x_last), [lp_last[self.offsets[t]:self.offsets[t + 1]] for t in range(n)]
