"""Oracle MaskedCouplingRQSpline flow, its training step and TrainModel
selection (float64, NumPy).

TEST INFRASTRUCTURE ONLY. Restates:
  * _normalize_bin_sizes / _normalize_knot_slopes   model/nf_model/rqSpline.py:20-39
  * _rational_quadratic_spline_fwd                  rqSpline.py:42-128
  * _safe_quadratic_root / _rational_quadratic_spline_inv  rqSpline.py:131-239
  * RQSpline.get_params                             rqSpline.py:310-338
  * MaskedCouplingRQSpline forward/inverse/sample/log_prob  rqSpline.py:364-504
  * MLP (tanh hidden layers, linear last)           model/common.py:68-124
  * MaskedCouplingLayer / ScalarAffine / Gaussian   common.py:127-168, 211-293
  * NFModel.train_epoch / train                     model/nf_model/base.py:127-210
  * optax.chain(clip_by_global_norm(1), adamw(lr, b1=.9))  resource/optimizer.py:19-22
  * TrainModel data selection                       strategy/train_model.py:66-80

Parameters are plain arrays (float64 unless the caller passes float32):
  layers[l] = {"W": [W_0 .. W_n], "b": [b_0 .. b_n], "scale": s, "shift": t,
               "mask": bool[d]}
with W_i of shape [out, in] (Equinox's Linear convention).
"""
from __future__ import annotations

import dataclasses

import numpy as np

RANGE_MIN, RANGE_MAX = -10.0, 10.0
MIN_BIN = 1e-4
MIN_SLOPE = 1e-4


def _softmax(a):
    e = np.exp(a - a.max(axis=-1, keepdims=True))
    return e / e.sum(axis=-1, keepdims=True)


def _softplus(a):
    return np.logaddexp(a, 0.0)


def slope_offset(dtype=np.float64):
    """rqSpline.py:37-38, computed in the parameter dtype."""
    ms = np.asarray(MIN_SLOPE, dtype)
    return np.log(np.exp(np.asarray(1.0, dtype) - ms) - np.asarray(1.0, dtype))


def spline_params(raw, K, rmin=RANGE_MIN, rmax=RANGE_MAX, mb=MIN_BIN, ms=MIN_SLOPE):
    """RQSpline.get_params (rqSpline.py:310-338) on raw [..., 3K+1] ->
    x_pos, y_pos, slopes each [..., K+1]."""
    R = rmax - rmin
    w = _softmax(raw[..., :K]) * (R - K * mb) + mb          # rqSpline.py:26-27
    h = _softmax(raw[..., K:2 * K]) * (R - K * mb) + mb
    shp = raw.shape[:-1] + (1,)
    xp = np.concatenate([np.full(shp, rmin), rmin + np.cumsum(w[..., :-1], -1), np.full(shp, rmax)], -1)
    yp = np.concatenate([np.full(shp, rmin), rmin + np.cumsum(h[..., :-1], -1), np.full(shp, rmax)], -1)
    off = np.log(np.exp(1.0 - ms) - 1.0)
    sl = _softplus(raw[..., 2 * K:] + off) + ms              # rqSpline.py:38-39
    return xp, yp, sl


def _select_bin(v, pos):
    """Bin k with pos[k] <= v < pos[k+1]; bin 0 when none (rqSpline.py:63-72)."""
    inb = (v[..., None] >= pos[..., :-1]) & (v[..., None] < pos[..., 1:])
    anyb = inb.any(-1)
    k = np.argmax(inb, axis=-1)
    return np.where(anyb, k, 0)


def _take(a, k):
    return np.take_along_axis(a, k[..., None], -1)[..., 0]


def rqs_forward(x, xp, yp, sl):
    """_rational_quadratic_spline_fwd (rqSpline.py:42-128), elementwise."""
    below = x <= xp[..., 0]
    above = x >= xp[..., -1]
    k = _select_bin(x, xp)
    x0, x1 = _take(xp, k), _take(xp, k + 1)
    y0, y1 = _take(yp, k), _take(yp, k + 1)
    d0, d1 = _take(sl, k), _take(sl, k + 1)
    w = x1 - x0
    h = y1 - y0
    s = h / w
    z = np.clip((x - x0) / w, 0.0, 1.0)
    sq = z * z
    q = z - sq
    sq1 = (1.0 - z) ** 2
    num = h * (s * sq + d0 * q)
    den = s + (d1 + d0 - 2.0 * s) * q
    y = y0 + num / den
    ld = 2.0 * np.log(s) + np.log(d1 * sq + 2.0 * s * q + d0 * sq1) - 2.0 * np.log(den)
    y = np.where(below, (x - xp[..., 0]) * sl[..., 0] + yp[..., 0], y)
    y = np.where(above, (x - xp[..., -1]) * sl[..., -1] + yp[..., -1], y)
    ld = np.where(below, np.log(sl[..., 0]), ld)
    ld = np.where(above, np.log(sl[..., -1]), ld)
    return y, ld


def _safe_quadratic_root(a, b, c):
    """rqSpline.py:131-155."""
    disc = b * b - 4.0 * a * c
    tiny = np.finfo(np.asarray(disc).dtype).tiny
    sq = np.sqrt(np.clip(disc, tiny, None))
    sq = np.where(disc > 0.0, sq, 0.0)
    num = np.where(b >= 0, 2.0 * c, -b + sq)
    den = np.where(b >= 0, -b - sq, 2.0 * a)
    return num / den


def rqs_inverse(y, xp, yp, sl):
    """_rational_quadratic_spline_inv (rqSpline.py:158-239), elementwise."""
    below = y <= yp[..., 0]
    above = y >= yp[..., -1]
    k = _select_bin(y, yp)
    x0, x1 = _take(xp, k), _take(xp, k + 1)
    y0, y1 = _take(yp, k), _take(yp, k + 1)
    d0, d1 = _take(sl, k), _take(sl, k + 1)
    w = x1 - x0
    h = y1 - y0
    s = h / w
    ww = np.clip((y - y0) / h, 0.0, 1.0)
    st = d1 + d0 - 2.0 * s
    c = -s * ww
    b = d0 - st * ww
    a = s - b
    z = np.clip(_safe_quadratic_root(a, b, c), 0.0, 1.0)
    x = w * z + x0
    sq = z * z
    q = z - sq
    sq1 = (1.0 - z) ** 2
    den = s + st * q
    ld = -2.0 * np.log(s) - np.log(d1 * sq + 2.0 * s * q + d0 * sq1) + 2.0 * np.log(den)
    x = np.where(below, (y - yp[..., 0]) / sl[..., 0] + xp[..., 0], x)
    x = np.where(above, (y - yp[..., -1]) / sl[..., -1] + xp[..., -1], x)
    ld = np.where(below, -np.log(sl[..., 0]), ld)
    ld = np.where(above, -np.log(sl[..., -1]), ld)
    return x, ld


def mlp(Ws, bs, x, bf16=False):
    """MLP.__call__ (common.py:109-112): tanh after every layer but the last.

    bf16=True models the BF16-conditioner arithmetic (not the reference's):
    the input, every weight matrix and every hidden activation are rounded to
    bfloat16, the products and biases stay in float64. It measures the error
    that BF16 operands alone cause, the scale a BF16 kernel is held to."""
    h = round_bf16(x) if bf16 else x
    for i, (W, b) in enumerate(zip(Ws, bs)):
        h = h @ (round_bf16(W) if bf16 else W).T + b
        if i < len(Ws) - 1:
            h = np.tanh(h)
            if bf16:
                h = round_bf16(h)
    return h


def round_bf16(a):
    """Round to the nearest bfloat16 (ties to even), returned as float64: the
    float32 value's top 16 bits after adding 0x7fff plus the kept lsb."""
    u = np.ascontiguousarray(np.asarray(a, np.float32)).view(np.uint32)
    u = (u + (((u >> 16) & 1) + 0x7FFF)).astype(np.uint32) & np.uint32(0xFFFF0000)
    return u.view(np.float32).astype(np.float64)


@dataclasses.dataclass
class Flow:
    """MaskedCouplingRQSpline state (rqSpline.py:364-443)."""

    layers: list
    n_bins: int
    data_mean: np.ndarray
    data_cov: np.ndarray          # [d, d] (only the diagonal is read)
    base_cov_scale: float = 1.0   # base Gaussian covariance = scale * I
    bf16: bool = False            # conditioners with bfloat16 operands (see mlp)

    @property
    def d(self):
        return self.data_mean.shape[0]

    def coupling(self, layer, x, inverse: bool):
        """MaskedCouplingLayer(RQSpline) (common.py:150-168, rqSpline.py:347-361)."""
        m = layer["mask"].astype(np.float64)
        raw = mlp(layer["W"], layer["b"], x * m, self.bf16)
        n, d = x.shape
        P = 3 * self.n_bins + 1
        xp, yp, sl = spline_params(raw.reshape(n, d, P), self.n_bins)
        y, ld = (rqs_inverse if inverse else rqs_forward)(x, xp, yp, sl)
        y = (1 - m) * y + m * x
        return y, ((1 - m) * ld).sum(-1)

    def forward(self, x):
        """rqSpline.py:450-468: per layer ScalarAffine then the spline coupling."""
        ld = np.zeros(x.shape[0])
        for L in self.layers:
            x = (x + L["shift"]) * np.exp(L["scale"])          # common.py:229
            ld = ld + x.shape[1] * L["scale"]                    # mask_all = 0: sum over d
            x, l2 = self.coupling(L, x, inverse=False)
            ld = ld + l2
        return x, ld

    def inverse(self, z):
        """rqSpline.py:470-488: layers reversed; inside a layer the ScalarAffine
        inverse runs first, then the spline inverse (the reference's order)."""
        ld = np.zeros(z.shape[0])
        x = z
        for L in reversed(self.layers):
            x = x * np.exp(-L["scale"]) - L["shift"]             # common.py:238
            ld = ld - x.shape[1] * L["scale"]
            x, l2 = self.coupling(L, x, inverse=True)
            ld = ld + l2
        return x, ld

    def std(self):
        return np.sqrt(np.diag(self.data_cov))

    def log_prob(self, x):
        """rqSpline.py:498-504 (no Jacobian of the standardisation)."""
        xs = (x - self.data_mean) / self.std()
        y, ld = self.forward(xs)
        c = self.base_cov_scale
        d = y.shape[1]
        return ld - 0.5 * np.sum(y * y, -1) / c - 0.5 * d * np.log(2.0 * np.pi * c)

    def sample(self, z):
        """rqSpline.py:490-496 with the base normals z given: base sample =
        mean + z @ cholesky(cov).T (jax.random.multivariate_normal)."""
        zz = z * np.sqrt(self.base_cov_scale)
        x, _ = self.inverse(zz)
        return x * self.std() + self.data_mean


# ---------------------------------------------------------------- parameters
def param_list(flow: Flow):
    """Trainable leaves in a fixed order: per layer scale, shift, W_i, b_i."""
    out = []
    for L in flow.layers:
        out.append(("scale", L))
        out.append(("shift", L))
        for i in range(len(L["W"])):
            out.append((("W", i), L))
            out.append((("b", i), L))
    return out


def get_leaf(key, L):
    if key in ("scale", "shift"):
        return np.asarray(L[key], np.float64)
    name, i = key
    return L[name][i]


def set_leaf(key, L, val):
    if key in ("scale", "shift"):
        L[key] = float(val)
    else:
        name, i = key
        L[name][i] = val


def flatten(flow: Flow) -> np.ndarray:
    return np.concatenate([np.ravel(get_leaf(k, L)) for k, L in param_list(flow)])


def unflatten(flow: Flow, vec: np.ndarray) -> None:
    o = 0
    for k, L in param_list(flow):
        cur = np.asarray(get_leaf(k, L))
        n = cur.size
        set_leaf(k, L, vec[o:o + n].reshape(cur.shape))
        o += n


def clone(flow: Flow) -> Flow:
    layers = []
    for L in flow.layers:
        layers.append({"W": [w.copy() for w in L["W"]], "b": [b.copy() for b in L["b"]],
                       "scale": float(L["scale"]), "shift": float(L["shift"]), "mask": L["mask"].copy()})
    return Flow(layers, flow.n_bins, flow.data_mean.copy(), flow.data_cov.copy(), flow.base_cov_scale)


def loss(flow: Flow, x: np.ndarray) -> float:
    """NFModel.loss_fn (nf_model/base.py:98-100)."""
    return float(-np.mean(flow.log_prob(x)))


# ---------------------------------------------------------------- optimiser
@dataclasses.dataclass
class AdamWState:
    """optax.chain(clip_by_global_norm(1.0), adamw(lr, b1=0.9)) state.

    optax 0.2.4 defaults (its public API docs): b2=0.999, eps=1e-8,
    eps_root=0, weight_decay=1e-4. ``aux`` holds the moments of the
    non-trainable float leaves that Equinox still hands to the optimiser
    (data_mean, data_cov, the base Gaussian mean/cov; their gradients are 0).
    """

    m: np.ndarray
    v: np.ndarray
    count: int = 0


def adamw_update(params, grads, st: AdamWState, lr, b1=0.9, b2=0.999, eps=1e-8, wd=1e-4,
                 max_norm=1.0, extra_sq_norm=0.0):
    """One optax update + apply_updates (nf_model/base.py:123-124) on a flat
    parameter vector. Returns (new_params, decay_factor) where decay_factor
    = 1 - lr*wd is what the zero-gradient float leaves are multiplied by."""
    gnorm = np.sqrt(np.sum(grads * grads) + extra_sq_norm)
    if not gnorm < max_norm:
        grads = grads / gnorm * max_norm
    st.count += 1
    st.m = b1 * st.m + (1 - b1) * grads
    st.v = b2 * st.v + (1 - b2) * grads * grads
    mhat = st.m / (1 - b1 ** st.count)
    vhat = st.v / (1 - b2 ** st.count)
    upd = mhat / (np.sqrt(vhat) + eps) + wd * params
    return params - lr * upd, 1.0 - lr * wd


def train(flow: Flow, data: np.ndarray, grad_fn, st: AdamWState, n_epochs: int, batch_size: int,
          lr: float, perms=None):
    """NFModel.train (nf_model/base.py:153-210) with explicit permutations.

    grad_fn(flow, batch) -> (loss, flat_grad). perms[e] is the epoch's
    permutation of range(len(data)) (jax.random.permutation in the reference).
    Returns (best_flow, best_state, loss_values).
    """
    flow = clone(flow)
    flow.data_mean = data.mean(0)                                   # base.py:187
    flow.data_cov = np.cov(data.T).reshape(data.shape[1], data.shape[1])   # base.py:188
    best, best_st, best_loss = clone(flow), AdamWState(st.m.copy(), st.v.copy(), st.count), 1e9
    losses = np.zeros(n_epochs)
    N = data.shape[0]
    for e in range(n_epochs):
        steps = N // batch_size
        if steps > 0:
            perm = perms[e][: steps * batch_size].reshape(steps, batch_size)
            batches = [data[p] for p in perm]
        else:
            batches = [data]
        value = 1e9
        for batch in batches:
            value, g = grad_fn(flow, batch)
            p = flatten(flow)
            p, decay = adamw_update(p, g, st, lr)
            unflatten(flow, p)
            flow.data_mean = flow.data_mean * decay
            flow.data_cov = flow.data_cov * decay
            flow.base_cov_scale = flow.base_cov_scale * decay
        losses[e] = value
        if losses[e] < best_loss:
            best, best_st, best_loss = clone(flow), AdamWState(st.m.copy(), st.v.copy(), st.count), losses[e]
    return best, best_st, losses


def select_training_data(buf: np.ndarray, history_window: int, choice_idx: np.ndarray) -> np.ndarray:
    """TrainModel.__call__ data selection (train_model.py:66-80): rows with
    all-finite coordinates, reshaped per chain, the last `history_window`
    per chain, then rows `choice_idx` (jax.random.choice with replacement)."""
    C, S, d = buf.shape
    fin = np.isfinite(buf).all(-1)
    td = buf[fin].reshape(C, -1, d)
    td = td[:, -history_window:].reshape(-1, d)
    return td[choice_idx]
