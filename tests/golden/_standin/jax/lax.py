import torch


def _stack(ys):
    y0 = ys[0]
    if y0 is None:
        return None
    if isinstance(y0, tuple):
        return tuple(_stack([y[k] for y in ys]) for k in range(len(y0)))
    return torch.stack([torch.as_tensor(y, dtype=torch.float64) for y in ys])


def scan(f, init, xs=None, length=None, reverse=False):
    carry = init
    ys = []
    if xs is None:
        it = list(range(length))
    elif isinstance(xs, tuple):
        it = list(zip(*xs))     # a tuple of arrays scans over their leading axis together
    else:
        it = list(xs)           # an array, or the golden script's list of per-layer modules
    for x in (reversed(it) if reverse else it):
        carry, y = f(carry, x)
        ys.append(y)
    if reverse:
        ys.reverse()
    return carry, _stack(ys) if ys else None


def stop_gradient(x):
    return x.detach() if isinstance(x, torch.Tensor) else x


def cond(pred, true_fun, false_fun, *operands):
    return true_fun(*operands) if bool(pred) else false_fun(*operands)


def dynamic_slice_in_dim(x, start, size, axis=0):
    return x.narrow(axis, int(start), size)


def dynamic_update_slice_in_dim(x, update, start, axis=0):
    out = x.clone()
    n = update.shape[axis]
    s = min(max(int(start), 0), x.shape[axis] - n)
    out.narrow(axis, s, n).copy_(update)
    return out
