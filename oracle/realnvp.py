"""Oracle RealNVP (float64) -- TEST INFRASTRUCTURE ONLY.

Restates resource/model/nf_model/realNVP.py:120-222 with the layer math of
resource/model/common.py (MLP :68-112 with relu, MaskedCouplingLayer
:127-168, MLPAffine :171-208):
  c = x * m,  s = tanh(MLP_s(c)) * dt,  t = MLP_t(c) * dt
  forward  y = (1 - m) * ((x + t) * exp(s)) + m * x,  log-det += sum (1 - m) s
  inverse  y = (1 - m) * (x * exp(-s) - t) + m * x,   log-det -= sum (1 - m) s
  log_prob = forward((x - mean) / sqrt(var)) log-det + log N(y; 0, I)
  sample   = inverse(sqrt(c) z) * sqrt(var) + mean
Masks are general floats (the reference's masks are float leaves that
weight decay moves). ``loss_and_grad`` differentiates -mean(log_prob) with
torch autograd in float64.
"""
from __future__ import annotations

import math

import numpy as np

KEYS = ("W1s", "b1s", "W2s", "b2s", "W1t", "b1t", "W2t", "b2t")


class RealNVP:
    """params: dict of KEYS -> arrays with a leading layer axis (W1 [L, H, d],
    b1 [L, H], W2 [L, d, H], b2 [L, d]); masks [L, d]."""

    def __init__(self, params, masks, mean, var, base_scale=1.0, dt=1.0):
        self.p = {k: np.asarray(params[k], np.float64) for k in KEYS}
        self.masks = np.asarray(masks, np.float64)
        self.mean, self.var = np.asarray(mean, np.float64), np.asarray(var, np.float64)
        self.base_scale, self.dt = float(base_scale), float(dt)
        self.L, self.d = self.masks.shape

    def _mlps(self, l, c):
        p = self.p
        hs = np.maximum(c @ p["W1s"][l].T + p["b1s"][l], 0.0)
        ht = np.maximum(c @ p["W1t"][l].T + p["b1t"][l], 0.0)
        return hs @ p["W2s"][l].T + p["b2s"][l], ht @ p["W2t"][l].T + p["b2t"][l]

    def _layer(self, l, x, inverse):
        m = self.masks[l]
        sr, tr = self._mlps(l, x * m)
        s, t = np.tanh(sr) * self.dt, tr * self.dt
        ya = x * np.exp(-s) - t if inverse else (x + t) * np.exp(s)
        ld = ((1 - m) * s).sum(-1)
        return (1 - m) * ya + m * x, (-ld if inverse else ld)

    def forward(self, x):
        x = np.atleast_2d(np.asarray(x, np.float64))
        ld = np.zeros(x.shape[0])
        for l in range(self.L):
            x, dl = self._layer(l, x, False)
            ld = ld + dl
        return x, ld

    def inverse(self, y):
        y = np.atleast_2d(np.asarray(y, np.float64))
        ld = np.zeros(y.shape[0])
        for l in reversed(range(self.L)):
            y, dl = self._layer(l, y, True)
            ld = ld + dl
        return y, ld

    def log_prob(self, x):
        xt = (np.atleast_2d(np.asarray(x, np.float64)) - self.mean) / np.sqrt(self.var)
        y, ld = self.forward(xt)
        return ld - 0.5 * (y * y).sum(-1) - 0.5 * self.d * math.log(2 * math.pi)

    def sample(self, z):
        x, _ = self.inverse(np.asarray(z, np.float64) * math.sqrt(self.base_scale))
        return x * np.sqrt(self.var) + self.mean


def loss_and_grad(model: RealNVP, x):
    """loss = -mean(log_prob(x)) and d loss / d params (dict of KEYS), float64."""
    import torch
    P = {k: torch.tensor(v, dtype=torch.float64, requires_grad=True) for k, v in model.p.items()}
    masks = torch.tensor(model.masks)
    xt = (torch.tensor(np.asarray(x, np.float64)) - torch.tensor(model.mean)) / torch.sqrt(torch.tensor(model.var))
    ld = torch.zeros(xt.shape[0], dtype=torch.float64)
    for l in range(model.L):
        m = masks[l]
        c = xt * m
        hs = torch.relu(c @ P["W1s"][l].T + P["b1s"][l])
        ht = torch.relu(c @ P["W1t"][l].T + P["b1t"][l])
        s = torch.tanh(hs @ P["W2s"][l].T + P["b2s"][l]) * model.dt
        t = (ht @ P["W2t"][l].T + P["b2t"][l]) * model.dt
        xt = (1 - m) * ((xt + t) * torch.exp(s)) + m * xt
        ld = ld + ((1 - m) * s).sum(-1)
    lp = ld - 0.5 * (xt * xt).sum(-1) - 0.5 * model.d * math.log(2 * math.pi)
    loss = -lp.mean()
    loss.backward()
    return float(loss.detach()), {k: P[k].grad.numpy() for k in KEYS}


def pack(params, L):
    """Flat vector in the library's per-layer order: [W1s; W1t], [b1s; b1t],
    W2s, b2s, W2t, b2t."""
    out = []
    for l in range(L):
        out += [params["W1s"][l].ravel(), params["W1t"][l].ravel(), params["b1s"][l], params["b1t"][l],
                params["W2s"][l].ravel(), params["b2s"][l], params["W2t"][l].ravel(), params["b2t"][l]]
    return np.concatenate(out)
