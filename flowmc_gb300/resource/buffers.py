"""Buffer resource (mirrors resource/buffers.py:11-64 of the reference).

``data`` is a float32 torch tensor (on the GPU by default) initialised to
-inf, in the reference's layout (e.g. positions [n_chains, n_steps, n_dim]).
The local and global step kernels write into it directly; ``update_buffer``
is the general path and keeps ``jax.lax.dynamic_update_slice_in_dim``'s
clamping of the start index.
"""
from __future__ import annotations

import numpy as np
import torch

from .base import Resource


def default_device() -> torch.device:
    return torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu")


def clamp_start(start: int, n: int, size: int) -> int:
    """Start index of jax.lax.dynamic_update_slice: clamped so [start, start+n) fits."""
    if n > size:
        raise ValueError(f"update of length {n} does not fit a buffer axis of length {size}")
    return min(max(int(start), 0), size - n)


class Buffer(Resource):
    name: str
    data: torch.Tensor
    cursor: int = 0
    cursor_dim: int = 0

    def __repr__(self):
        return "Buffer " + self.name + " with shape " + str(tuple(self.data.shape))

    @property
    def shape(self):
        return tuple(self.data.shape)

    def __init__(self, name: str, shape: tuple[int, ...], cursor_dim: int = 0, device=None,
                 dtype=torch.float32):
        self.cursor_dim = cursor_dim
        self.name = name
        self.cursor = 0
        dev = default_device() if device is None else torch.device(device)
        self.data = torch.full(tuple(shape), -float("inf"), dtype=dtype, device=dev)

    def __call__(self):
        return self.data

    def update_buffer(self, updates, start: int = 0):
        """Write `updates` at `start` along cursor_dim (buffers.py:32-41)."""
        u = torch.as_tensor(updates, dtype=self.data.dtype, device=self.data.device)
        ax = self.cursor_dim
        if u.dim() != self.data.dim():
            raise ValueError(f"update rank {u.dim()} != buffer rank {self.data.dim()}")
        s = clamp_start(start, u.shape[ax], self.data.shape[ax])
        self.data.narrow(ax, s, u.shape[ax]).copy_(u)

    def print_parameters(self):
        print(
            f"Buffer: {self.name} with shape {tuple(self.data.shape)} and cursor"
            f" {self.cursor} at dimension {self.cursor_dim}"
        )

    def get_distribution(self, n_bins: int = 100):
        return np.histogram(self.data.detach().cpu().numpy().flatten(), bins=n_bins)

    def save_resource(self, path: str):
        np.savez(path + self.name, name=self.name, data=self.data.detach().cpu().numpy())

    def load_resource(self, path: str) -> "Buffer":
        d = np.load(path)
        arr = d["data"]
        result = Buffer(str(d["name"]), arr.shape, device=self.data.device)
        result.data.copy_(torch.as_tensor(arr))
        return result
