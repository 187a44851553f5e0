"""jax stand-in for the golden-fixture script (torch float64, autograd, Python loops)."""
import torch

from . import lax, nn, numpy, random, scipy, tree_util  # noqa: F401


def _prep(x):
    return torch.as_tensor(x, dtype=torch.float64).detach().clone().requires_grad_(True)


def value_and_grad(f):
    def vg(x, *args):
        x = _prep(x)
        with torch.enable_grad():
            v = f(x, *args)
            (g,) = torch.autograd.grad(v, x)
        return v.detach(), g.detach()
    return vg


def grad(f):
    def gf(x, *args):
        return value_and_grad(f)(x, *args)[1]
    return gf


def vmap(f, in_axes=0):
    def vf(*args):
        axes = in_axes if isinstance(in_axes, (tuple, list)) else (in_axes,) * len(args)

        def size(a, ax):
            return len(a) if isinstance(a, list) else torch.as_tensor(a).shape[ax]

        def pick(a, ax, i):
            if ax is None:
                return a
            return a[i] if isinstance(a, list) else torch.as_tensor(a).select(ax, i)

        n = next(size(a, ax) for a, ax in zip(args, axes) if ax is not None)
        outs = []
        for i in range(n):
            outs.append(f(*[pick(a, ax, i) for a, ax in zip(args, axes)]))
        if isinstance(outs[0], tuple):
            return tuple(torch.stack([o[k] for o in outs]) for k in range(len(outs[0])))
        return torch.stack(outs)
    return vf


def jit(f, **kw):
    return f
