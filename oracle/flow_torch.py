"""Float64 autograd restatement of the flow loss -- TEST INFRASTRUCTURE ONLY.

The same MaskedCouplingRQSpline log_prob as ``oracle.flow`` (rqSpline.py:
20-128, 310-504; common.py:68-168, 211-293), written with torch CPU float64
tensors so that reverse-mode autodiff gives the gradient oracle that
``jax.value_and_grad`` gives the reference (nf_model/base.py:98-100, 122).
Central finite differences in ``tests/`` pin this gradient in turn.
"""
from __future__ import annotations

import numpy as np
import torch

from . import flow as F


def _params(flow: F.Flow):
    leaves = []
    for k, L in F.param_list(flow):
        leaves.append(torch.tensor(np.asarray(F.get_leaf(k, L), np.float64), dtype=torch.float64,
                                   requires_grad=True))
    return leaves


def _spline_fwd(x, raw, K):
    R = F.RANGE_MAX - F.RANGE_MIN
    w = torch.softmax(raw[..., :K], -1) * (R - K * F.MIN_BIN) + F.MIN_BIN
    h = torch.softmax(raw[..., K:2 * K], -1) * (R - K * F.MIN_BIN) + F.MIN_BIN
    shp = raw.shape[:-1] + (1,)
    lo = torch.full(shp, F.RANGE_MIN, dtype=raw.dtype)
    hi = torch.full(shp, F.RANGE_MAX, dtype=raw.dtype)
    xp = torch.cat([lo, F.RANGE_MIN + torch.cumsum(w[..., :-1], -1), hi], -1)
    yp = torch.cat([lo, F.RANGE_MIN + torch.cumsum(h[..., :-1], -1), hi], -1)
    off = float(np.log(np.exp(1.0 - F.MIN_SLOPE) - 1.0))
    sl = torch.nn.functional.softplus(raw[..., 2 * K:] + off) + F.MIN_SLOPE
    below = x <= xp[..., 0]
    above = x >= xp[..., -1]
    inb = (x[..., None] >= xp[..., :-1]) & (x[..., None] < xp[..., 1:])
    k = torch.where(inb.any(-1), torch.argmax(inb.to(torch.int8), -1), torch.zeros_like(x, dtype=torch.long))

    def take(a, kk):
        return torch.gather(a, -1, kk[..., None])[..., 0]

    x0, x1 = take(xp, k), take(xp, k + 1)
    y0, y1 = take(yp, k), take(yp, k + 1)
    d0, d1 = take(sl, k), take(sl, k + 1)
    bw = x1 - x0
    bh = y1 - y0
    s = bh / bw
    z = torch.clamp((x - x0) / bw, 0.0, 1.0)
    sq = z * z
    q = z - sq
    sq1 = (1.0 - z) ** 2
    num = bh * (s * sq + d0 * q)
    den = s + (d1 + d0 - 2.0 * s) * q
    y = y0 + num / den
    ld = 2.0 * torch.log(s) + torch.log(d1 * sq + 2.0 * s * q + d0 * sq1) - 2.0 * torch.log(den)
    y = torch.where(below, (x - xp[..., 0]) * sl[..., 0] + yp[..., 0], y)
    y = torch.where(above, (x - xp[..., -1]) * sl[..., -1] + yp[..., -1], y)
    ld = torch.where(below, torch.log(sl[..., 0]), ld)
    ld = torch.where(above, torch.log(sl[..., -1]), ld)
    return y, ld


def log_prob(flow: F.Flow, leaves, x: np.ndarray):
    xt = torch.tensor(np.asarray(x, np.float64))
    mean = torch.tensor(flow.data_mean)
    std = torch.tensor(flow.std())
    h = (xt - mean) / std
    n, d = h.shape
    K = flow.n_bins
    P = 3 * K + 1
    ld = torch.zeros(n, dtype=torch.float64)
    it = iter(leaves)
    for L in flow.layers:
        s = next(it)
        t = next(it)
        Ws, bs = [], []
        for _ in range(len(L["W"])):
            Ws.append(next(it))
            bs.append(next(it))
        h = (h + t) * torch.exp(s)
        ld = ld + d * s
        m = torch.tensor(L["mask"].astype(np.float64))
        a = h * m
        for i, (W, b) in enumerate(zip(Ws, bs)):
            a = a @ W.T + b
            if i < len(Ws) - 1:
                a = torch.tanh(a)
        y, l2 = _spline_fwd(h, a.reshape(n, d, P), K)
        h = (1 - m) * y + m * h
        ld = ld + ((1 - m) * l2).sum(-1)
    c = flow.base_cov_scale
    return ld - 0.5 * (h * h).sum(-1) / c - 0.5 * d * np.log(2.0 * np.pi * c)


def loss_and_grad(flow: F.Flow, x: np.ndarray):
    """(loss, flat gradient in oracle.flow.param_list order), float64."""
    leaves = _params(flow)
    lp = log_prob(flow, leaves, x)
    loss = -lp.mean()
    grads = torch.autograd.grad(loss, leaves)
    flat = np.concatenate([g.detach().numpy().ravel() for g in grads])
    return float(loss.detach()), flat
