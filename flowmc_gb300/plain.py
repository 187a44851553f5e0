"""The plain FP32 GPU form of the sampling path: the comparison baseline.

A PyTorch-eager float32 restatement that follows flowMC's algorithm one
reference op at a time, on the GPU, with no hand-written kernels, no fusion
and no graph capture:
  * MALA evaluates value and gradient twice per step (MALA.py:57-81); HMC
    runs the full leapfrog table, n_leapfrog + 2 gradient rows (HMC.py:71-96);
  * the flow is MaskedCouplingRQSpline with full-width conditioners (the
    masked input and all d * (3K+1) outputs, rqSpline.py:427-440), the
    spline vectorised with the reference's one-hot bin selection
    (rqSpline.py:42-239), trained with autograd and optax's
    clip_by_global_norm + adamw semantics (optimizer.py:19-22);
  * NFProposal draws all proposals, then scans the independent-MH accept
    over the steps (NF_proposal.py:27-128).
It exists so the fused path can be measured against it at equal moment
error; the product path never calls it.
"""
from __future__ import annotations

import math
import time

import torch

RMIN, RMAX, MIN_BIN, MIN_SLOPE = -10.0, 10.0, 1e-4, 1e-4


# ------------------------------------------------------------------ targets
def rosenbrock_value_grad(x, a=20.0, b=1.0, c=5.0):
    x0, x1 = x[:, :-1], x[:, 1:]
    u = b - x0
    v = x1 - x0 * x0
    lp = -(u * u / a + c * v * v).sum(-1)
    g = torch.zeros_like(x)
    g[:, :-1] += 2.0 * u / a + 4.0 * c * x0 * v
    g[:, 1:] -= 2.0 * c * v
    return lp, g


def dual_moon_value_grad(x, r0=2.0, sr=0.1, mu=3.0, s0=0.6):
    r = torch.linalg.vector_norm(x, dim=-1)
    a = (x[:, 0] + mu) / s0
    b = (x[:, 0] - mu) / s0
    ea, eb = -0.5 * a * a, -0.5 * b * b
    lse = torch.logaddexp(ea, eb)
    lp = -0.5 * ((r - r0) / sr) ** 2 + lse
    g = (-(r - r0) / (sr * sr) / r)[:, None] * x
    g[:, 0] -= (torch.exp(ea - lse) * a + torch.exp(eb - lse) * b) / s0
    return lp, g


def mixture_value_grad(x, means, inv_var, log_w):
    dx = x[:, None, :] - means[None]
    e = log_w[None] - 0.5 * (dx * dx * inv_var[None]).sum(-1)
    lse = torch.logsumexp(e, 1)
    w = torch.exp(e - lse[:, None])
    g = -(w[:, :, None] * dx * inv_var[None]).sum(1)
    return lse, g


# ------------------------------------------------------------------ local kernels
def hmc_step(vg, x, lp, eps, n_leapfrog, gen):
    p = torch.randn(x.shape, device=x.device, generator=gen)
    H = -lp + 0.5 * (p * p).sum(-1)
    xq, pq = x, p
    coefs = [(0.0, 0.5)] + [(1.0, 1.0)] * n_leapfrog + [(1.0, 0.5)]
    for c0, c1 in coefs:
        xq = xq + eps * c0 * pq
        _, g = vg(xq)
        pq = pq - eps * c1 * (-g)
    lpq, _ = vg(xq)
    Hq = -lpq + 0.5 * (pq * pq).sum(-1)
    u = torch.rand(lp.shape, device=x.device, generator=gen)
    acc = torch.log(u) < H - Hq
    return torch.where(acc[:, None], xq, x), torch.where(acc, lpq, lp), acc


def mala_step(vg, x, lp, dt, gen):
    dt2 = dt * dt
    lp0, g0 = vg(x)
    xi = torch.randn(x.shape, device=x.device, generator=gen)
    prop = x + dt2 * g0 / 2 + dt * xi
    lp1, g1 = vg(prop)
    d = x.shape[1]

    def lnq(a, m):
        r = a - m
        return -0.5 * (r * r).sum(-1) / dt2 - 0.5 * d * math.log(2 * math.pi * dt2)
    ratio = lp1 - lp0 - lnq(prop, x + dt2 * g0 / 2) + lnq(x, prop + dt2 * g1 / 2)
    u = torch.rand(lp.shape, device=x.device, generator=gen)
    acc = torch.log(u) < ratio
    return torch.where(acc[:, None], prop, x), torch.where(acc, lp1, lp0), acc


# ------------------------------------------------------------------ flow
class PlainFlow:
    """MaskedCouplingRQSpline in float32 torch eager, reference layout."""

    def __init__(self, d, n_layers, hidden, K, gen, device):
        self.d, self.L, self.K, self.P = d, n_layers, K, 3 * K + 1
        self.params = []
        shape = [d] + list(hidden) + [d * self.P]
        for i in range(n_layers):
            Ws, bs = [], []
            for j, (a, b) in enumerate(zip(shape[:-1], shape[1:])):
                lim = 1.0 / math.sqrt(a)
                if j < len(shape) - 2:
                    W = torch.randn(b, a, device=device, generator=gen) * math.sqrt(1e-2 / a)
                else:
                    W = (torch.rand(b, a, device=device, generator=gen) * 2 - 1) * lim
                bias = (torch.rand(b, device=device, generator=gen) * 2 - 1) * lim
                Ws.append(W.requires_grad_())
                bs.append(bias.requires_grad_())
            s = torch.zeros((), device=device, requires_grad=True)
            t = torch.zeros((), device=device, requires_grad=True)
            mask = ((torch.arange(d, device=device) + i) % 2).float()
            self.params.append({"W": Ws, "b": bs, "scale": s, "shift": t, "mask": mask})
        self.mean = torch.zeros(d, device=device)
        self.var = torch.ones(d, device=device)
        self.base_c = torch.ones((), device=device)
        self.off = math.log(math.expm1(1.0 - MIN_SLOPE))

    def leaves(self):
        out = []
        for p in self.params:
            out += [p["scale"], p["shift"]]
            for W, b in zip(p["W"], p["b"]):
                out += [W, b]
        return out

    def _knots(self, raw):
        K = self.K
        R = RMAX - RMIN
        w = torch.softmax(raw[..., :K], -1) * (R - K * MIN_BIN) + MIN_BIN
        h = torch.softmax(raw[..., K:2 * K], -1) * (R - K * MIN_BIN) + MIN_BIN
        shp = raw.shape[:-1] + (1,)
        lo = torch.full(shp, RMIN, device=raw.device)
        hi = torch.full(shp, RMAX, device=raw.device)
        xp = torch.cat([lo, RMIN + torch.cumsum(w[..., :-1], -1), hi], -1)
        yp = torch.cat([lo, RMIN + torch.cumsum(h[..., :-1], -1), hi], -1)
        sl = torch.nn.functional.softplus(raw[..., 2 * K:] + self.off) + MIN_SLOPE
        return xp, yp, sl

    @staticmethod
    def _bin(v, pos):
        inb = (v[..., None] >= pos[..., :-1]) & (v[..., None] < pos[..., 1:])
        first = torch.zeros_like(inb)
        first[..., 0] = True
        inb = torch.where(inb.any(-1, keepdim=True), inb, first).float()
        return inb

    def _spline(self, x, raw, inverse):
        xp, yp, sl = self._knots(raw)
        pos = yp if inverse else xp
        oh = self._bin(x, pos)
        sel = lambda a, o: (oh * a[..., o:a.shape[-1] - 1 + o]).sum(-1)
        x0, x1, y0, y1, d0, d1 = sel(xp, 0), sel(xp, 1), sel(yp, 0), sel(yp, 1), sel(sl, 0), sel(sl, 1)
        w, h = x1 - x0, y1 - y0
        s = h / w
        st = d1 + d0 - 2.0 * s
        if not inverse:
            z = torch.clamp((x - x0) / w, 0.0, 1.0)
            q = z - z * z
            y = y0 + h * (s * z * z + d0 * q) / (s + st * q)
            ld = 2 * torch.log(s) + torch.log(d1 * z * z + 2 * s * q + d0 * (1 - z) ** 2) - 2 * torch.log(s + st * q)
            below, above = x <= xp[..., 0], x >= xp[..., -1]
            y = torch.where(below, (x - xp[..., 0]) * sl[..., 0] + yp[..., 0], y)
            y = torch.where(above, (x - xp[..., -1]) * sl[..., -1] + yp[..., -1], y)
            ld = torch.where(below, torch.log(sl[..., 0]), ld)
            ld = torch.where(above, torch.log(sl[..., -1]), ld)
            return y, ld
        ww = torch.clamp((x - y0) / h, 0.0, 1.0)
        c = -s * ww
        bb = d0 - st * ww
        a = s - bb
        disc = bb * bb - 4 * a * c
        sq = torch.where(disc > 0, torch.sqrt(torch.clamp(disc, min=1.1754944e-38)), torch.zeros_like(disc))
        z = torch.where(bb >= 0, 2 * c / (-bb - sq), (-bb + sq) / (2 * a))
        z = torch.clamp(z, 0.0, 1.0)
        out = w * z + x0
        below, above = x <= yp[..., 0], x >= yp[..., -1]
        out = torch.where(below, (x - yp[..., 0]) / sl[..., 0] + xp[..., 0], out)
        out = torch.where(above, (x - yp[..., -1]) / sl[..., -1] + xp[..., -1], out)
        return out, None

    def _mlp(self, p, a):
        n = len(p["W"])
        for j, (W, b) in enumerate(zip(p["W"], p["b"])):
            a = a @ W.T + b
            if j < n - 1:
                a = torch.tanh(a)
        return a

    def forward(self, x):
        ld = torch.zeros(x.shape[0], device=x.device)
        for p in self.params:
            x = (x + p["shift"]) * torch.exp(p["scale"])
            ld = ld + self.d * p["scale"]
            m = p["mask"]
            raw = self._mlp(p, x * m).reshape(x.shape[0], self.d, self.P)
            y, l = self._spline(x, raw, False)
            x = (1 - m) * y + m * x
            ld = ld + ((1 - m) * l).sum(-1)
        return x, ld

    def inverse(self, z):
        x = z
        for p in reversed(self.params):
            x = x * torch.exp(-p["scale"]) - p["shift"]
            m = p["mask"]
            raw = self._mlp(p, x * m).reshape(x.shape[0], self.d, self.P)
            y, _ = self._spline(x, raw, True)
            x = (1 - m) * y + m * x
        return x

    def log_prob(self, x):
        xs = (x - self.mean) / torch.sqrt(self.var)
        y, ld = self.forward(xs)
        c = self.base_c
        return ld - 0.5 * (y * y).sum(-1) / c - 0.5 * self.d * torch.log(2 * math.pi * c)

    @torch.no_grad()
    def log_prob_chunked(self, x, chunk):
        return torch.cat([self.log_prob(x[i:i + chunk]) for i in range(0, x.shape[0], chunk)])

    @torch.no_grad()
    def sample(self, n, gen, chunk):
        out = []
        for i in range(0, n, chunk):
            m = min(chunk, n - i)
            z = torch.randn(m, self.d, device=self.mean.device, generator=gen) * torch.sqrt(self.base_c)
            out.append(self.inverse(z) * torch.sqrt(self.var) + self.mean)
        return torch.cat(out)


class PlainAdamW:
    """optax.chain(clip_by_global_norm(1.0), adamw(lr, b1=0.9)) on the leaves."""

    def __init__(self, leaves, lr, b1=0.9, b2=0.999, eps=1e-8, wd=1e-4):
        self.lr, self.b1, self.b2, self.eps, self.wd = lr, b1, b2, eps, wd
        self.m = [torch.zeros_like(p) for p in leaves]
        self.v = [torch.zeros_like(p) for p in leaves]
        self.count = 0

    @torch.no_grad()
    def step(self, leaves, grads, flow):
        gn = torch.sqrt(sum((g * g).sum() for g in grads))
        scale = torch.where(gn < 1.0, torch.ones_like(gn), 1.0 / gn)
        self.count += 1
        bc1, bc2 = 1 - self.b1 ** self.count, 1 - self.b2 ** self.count
        for p, g, m, v in zip(leaves, grads, self.m, self.v):
            g = g * scale
            m.mul_(self.b1).add_((1 - self.b1) * g)
            v.mul_(self.b2).add_((1 - self.b2) * g * g)
            p.add_(-self.lr * ((m / bc1) / (torch.sqrt(v / bc2) + self.eps) + self.wd * p))
        decay = 1 - self.lr * self.wd
        flow.mean.mul_(decay)
        flow.var.mul_(decay)
        flow.base_c.mul_(decay)


def train_flow(flow, opt, data, n_epochs, batch, gen, micro):
    """NFModel.train: per-epoch permutation, last-step loss, best epoch kept."""
    flow.mean = data.mean(0)
    flow.var = data.var(0, unbiased=True)
    leaves = flow.leaves()
    N = data.shape[0]
    best = None
    best_loss = 1e9
    for _ in range(n_epochs):
        steps = N // batch
        perm = torch.randperm(N, device=data.device, generator=gen)
        batches = [data[perm[i * batch:(i + 1) * batch]] for i in range(steps)] if steps > 0 else [data]
        for xb in batches:
            grads = [torch.zeros_like(p) for p in leaves]
            tot = 0.0
            for i in range(0, xb.shape[0], micro):
                part = xb[i:i + micro]
                loss = -flow.log_prob(part).sum() / xb.shape[0]
                gs = torch.autograd.grad(loss, leaves)
                for acc, g in zip(grads, gs):
                    acc.add_(g)
                tot += float(loss.detach())
            opt.step(leaves, grads, flow)
            value = tot
        if value < best_loss:
            best_loss = value
            best = ([p.detach().clone() for p in leaves], flow.mean.clone(), flow.var.clone(), flow.base_c.clone())
    if best is not None:
        with torch.no_grad():
            for p, b in zip(leaves, best[0]):
                p.copy_(b)
        flow.mean, flow.var, flow.base_c = best[1], best[2], best[3]


def run_plain(w, target_vg, n_train, n_prod, x0, gen, timed_from=0, chunk=32768, micro=4096):
    """The bundle's schedule in plain FP32 torch. Returns (production positions
    [C, S, d], seconds of the loops from `timed_from` on, accept rates)."""
    dev = x0.device
    C, d = x0.shape
    S1, S2 = w["n_local"], w["n_global"]
    blk = S1 + S2
    flow = PlainFlow(d, w["n_layers"], w["hidden"], w["n_bins"], gen, dev)
    opt = PlainAdamW(flow.leaves(), w["lr"])
    train_buf = torch.full((C, blk * n_train, d), -float("inf"), device=dev)
    prod_buf = torch.full((C, blk * n_prod, d), -float("inf"), device=dev)
    x = x0.clone()
    t0 = None
    accs = {"local": [], "global": []}
    for loop in range(n_train + n_prod):
        if loop == timed_from:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
        training = loop < n_train
        buf = train_buf if training else prod_buf
        base = (loop if training else loop - n_train) * blk
        lp, _ = target_vg(x)
        for s in range(S1):
            if w["local"] == "hmc":
                x, lp, acc = hmc_step(target_vg, x, lp, w["step"], w["n_leapfrog"], gen)
            else:
                x, lp, acc = mala_step(target_vg, x, lp, w["step"], gen)
            buf[:, base + s] = x
            accs["local"].append(acc.float().mean())
        if training:
            n_fin = (base + S1) if loop == 0 else base + S1
            flat = buf[:, :n_fin].reshape(C, -1, d)[:, -100:].reshape(-1, d)
            idx = torch.randint(0, flat.shape[0], (w["n_max"],), device=dev, generator=gen)
            train_flow(flow, opt, flat[idx], w["n_epochs"], w["batch"], gen, micro)
        with torch.no_grad():
            lp, _ = target_vg(x)
            lnf = flow.log_prob_chunked(x, chunk)
            props = flow.sample(C * S2, gen, chunk)
            lnf_p = flow.log_prob_chunked(props, chunk).reshape(C, S2)
            lp_p = torch.cat([target_vg(props[i:i + chunk])[0] for i in range(0, C * S2, chunk)]).reshape(C, S2)
            props = props.reshape(C, S2, d)
            u = torch.rand(C, S2, device=dev, generator=gen)
            for s in range(S2):
                ratio = (lp_p[:, s] - lp) - (lnf_p[:, s] - lnf)
                acc = torch.log(u[:, s]) < ratio
                x = torch.where(acc[:, None], props[:, s], x)
                lp = torch.where(acc, lp_p[:, s], lp)
                lnf = torch.where(acc, lnf_p[:, s], lnf)
                buf[:, base + S1 + s] = x
                accs["global"].append(acc.float().mean())
    torch.cuda.synchronize()
    secs = time.perf_counter() - t0
    rates = {k: float(torch.stack(v[-S1 * max(1, n_prod):]).mean()) for k, v in accs.items() if v}
    return prod_buf, secs, rates
