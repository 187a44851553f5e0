"""jax.numpy stand-in on float64 torch tensors (only what the golden script's reference code calls)."""
import builtins
import math

import torch

from . import linalg  # noqa: F401

float32 = torch.float32
float64 = torch.float64
dtype = torch.dtype
ndarray = torch.Tensor
_DT = torch.float64
pi = math.pi
inf = math.inf


def _is_key(v):
    return type(v).__name__ == "Key"


def _t(x, dtype=None):
    if isinstance(x, torch.Tensor):
        return x if dtype is None else x.to(dtype)
    return torch.as_tensor(x, dtype=dtype or _DT)


def array(x, dtype=None):
    if isinstance(x, (list, tuple)) and x and builtins.all(_is_key(v) for v in x):
        return list(x)
    if isinstance(x, (list, tuple)) and builtins.any(isinstance(v, torch.Tensor) for v in x):
        return torch.stack([_t(v, dtype) for v in x])
    return _t(x, dtype)


asarray = array


def where(c, a, b):
    c = c if isinstance(c, torch.Tensor) else torch.as_tensor(c)
    a, b = _t(a), _t(b)
    return torch.where(c.bool(), a, b)


def log(x):
    return torch.log(_t(x))


def exp(x):
    return torch.exp(_t(x))


def tanh(x):
    return torch.tanh(_t(x))


def isfinite(x):
    return torch.isfinite(_t(x))


def isinf(x):
    return torch.isinf(_t(x))


def isnan(x):
    return torch.isnan(_t(x))


def sqrt(x):
    return torch.sqrt(_t(x))


def square(x):
    x = _t(x)
    return x * x


def abs(x):  # noqa: A001
    return torch.abs(_t(x))


def sum(x, axis=None):  # noqa: A001
    x = _t(x)
    return x.sum() if axis is None else x.sum(dim=axis)


def mean(x, axis=None):
    x = _t(x)
    return x.mean() if axis is None else x.mean(dim=axis)


def zeros(shape, dtype=None):
    return torch.zeros(shape, dtype=dtype or _DT)


def ones(shape, dtype=None):
    return torch.ones(shape, dtype=dtype or _DT)


def full(shape, value, dtype=None):
    return torch.full(tuple(shape), float(value), dtype=dtype or _DT)


def dot(a, b):
    a, b = _t(a), _t(b)
    if a.dim() == 0 or b.dim() == 0:
        return a * b
    return torch.matmul(a, b)


def concatenate(xs, axis=0):
    return torch.cat([_t(v) for v in xs], dim=axis)


def flip(x, axis=None):
    x = _t(x)
    return torch.flip(x, dims=tuple(range(x.dim())) if axis is None else (axis,))


def stack(xs, axis=0):
    return torch.stack([_t(v) for v in xs], dim=axis)


def clip(x, a_min=None, a_max=None):
    x = _t(x)
    if a_min is not None:
        x = torch.maximum(x, _t(a_min))
    if a_max is not None:
        x = torch.minimum(x, _t(a_max))
    return x


def arange(*args):
    return torch.arange(*args)


def logical_and(a, b):
    return torch.logical_and(torch.as_tensor(a), torch.as_tensor(b))


def any(x, axis=None):  # noqa: A001
    x = torch.as_tensor(x)
    return x.any() if axis is None else x.any(dim=axis)


def eye(n, dtype=None):
    return torch.eye(n, dtype=dtype or _DT)


def atleast_2d(x):
    return torch.atleast_2d(_t(x))


def diag(x):
    return torch.diag(_t(x))


def cumsum(x, axis=None):
    x = _t(x)
    return torch.cumsum(x.reshape(-1) if axis is None else x, dim=0 if axis is None else axis)


class finfo:
    def __init__(self, dtype):
        fi = torch.finfo(dtype if isinstance(dtype, torch.dtype) else _DT)
        self.tiny = fi.tiny
        self.eps = fi.eps
        self.max = fi.max
        self.min = fi.min


# functional index update: x.at[i].set(v)
class _AtIdx:
    def __init__(self, t, idx):
        self.t, self.idx = t, idx

    def set(self, v):
        out = self.t.clone()
        out[self.idx] = _t(v, out.dtype)
        return out


class _At:
    def __init__(self, t):
        self.t = t

    def __getitem__(self, idx):
        return _AtIdx(self.t, idx)


torch.Tensor.at = property(lambda self: _At(self))


def _astype(self, dt):
    if dt is bool:
        return self.to(torch.bool)
    if dt is float:
        return self.to(_DT)
    if dt is int:
        return self.to(torch.int64)
    return self.to(dt)


torch.Tensor.astype = _astype
