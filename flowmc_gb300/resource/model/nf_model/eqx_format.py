"""Reader and writer for the reference's flow checkpoints (``NFModel.save_model``
/ ``load_model``, resource/model/nf_model/base.py:92-96), which are
``equinox.tree_serialise_leaves`` files, for MaskedCouplingRQSpline and
RealNVP.

Format (equinox's published serialisation, restated -- equinox itself is not
a dependency): the model's pytree leaves in flattening order, each array-like
leaf written as one NumPy ``.npy`` record (``np.save``) back to back; leaves
that are not array-like (functions such as the MLP's ``jax.nn.tanh``) are
skipped. Python scalars (ints, floats, bools) are array-like and take a 0-d
record. An Equinox module flattens its dataclass fields in declaration
order, base-class fields first.

For ``MaskedCouplingRQSpline(n_features=d, n_layers=L, hidden_size=H,
num_bins=K)`` (rqSpline.py:380-443, common.py:68-293) the leaves are:

  NFModel        _n_features (int), _data_mean [d], _data_cov [d, d]
  base_dist      Gaussian: _mean [d], _cov [d, d], learnable (bool)
  layers         one eqx.nn.Sequential built by eqx.filter_vmap over the L
                 layers, so every array leaf has a leading axis L:
    [0] MaskedCouplingLayer: _mask [L, d] bool,
        ScalarAffine: scale [L], shift [L]
    [1] MaskedCouplingLayer: _mask [L, d] bool,
        RQSpline: _range_min, _range_max (float), _num_bins (int),
                  _min_bin_size, _min_knot_slope (float),
                  conditioner MLP: per eqx.nn.Linear weight [L, out, in],
                  bias [L, out] (in/out features and use_bias are static
                  fields; the activations are skipped)

The reader walks this list; a scalar leaf whose record is absent is
tolerated (its value is implied by the model's constructor arguments), every
array record must have the expected shape.
"""
from __future__ import annotations

import numpy as np


def _leaves(model) -> list:
    """[(name, value)] in the reference's flattening order; value is an
    ndarray (float32 / bool) or a Python scalar."""
    d, L = model.n_features, model.n_layers
    full = model.to_full()
    aux = model.aux.detach().cpu().numpy().astype(np.float32)
    mean, var, base_scale = aux[:d], aux[d:2 * d], float(aux[2 * d])
    out = [("_n_features", int(d)),
           ("_data_mean", mean.copy()),
           ("_data_cov", np.diag(var).astype(np.float32)),
           ("base_dist._mean", np.zeros(d, np.float32)),
           ("base_dist._cov", (np.eye(d) * base_scale).astype(np.float32)),
           ("base_dist.learnable", False),
           ("layers[0]._mask", np.zeros((L, d), bool)),
           ("layers[0].bijector.scale", np.array([f["scale"] for f in full], np.float32)),
           ("layers[0].bijector.shift", np.array([f["shift"] for f in full], np.float32)),
           ("layers[1]._mask", np.stack([f["mask"] for f in full]).astype(bool)),
           ("layers[1].bijector._range_min", float(model.spline_range[0])),
           ("layers[1].bijector._range_max", float(model.spline_range[1])),
           ("layers[1].bijector._num_bins", int(model.num_bins)),
           ("layers[1].bijector._min_bin_size", float(model.min_bin_size)),
           ("layers[1].bijector._min_knot_slope", float(model.min_knot_slope))]
    for i in range(len(model.hidden_size) + 1):
        out.append((f"conditioner.layers[{2 * i}].weight", np.stack([f["W"][i] for f in full]).astype(np.float32)))
        out.append((f"conditioner.layers[{2 * i}].bias", np.stack([f["b"][i] for f in full]).astype(np.float32)))
    return out


def save_eqx(model, path: str) -> None:
    """Write `model` as the reference's ``save_model`` would (path as given)."""
    with open(path, "wb") as f:
        for _, v in _leaves(model):
            np.save(f, np.asarray(v), allow_pickle=False)


def _records(path: str) -> list:
    recs = []
    with open(path, "rb") as f:
        end = f.seek(0, 2)
        f.seek(0)
        while f.tell() < end:
            recs.append(np.load(f, allow_pickle=False))
    return recs


def _read_leaves(path: str, expect: list) -> dict:
    """The checkpoint's records matched to `expect` ([(name, value)]): array
    leaves must have the expected shapes, scalar leaves may be absent."""
    recs = _records(path)
    got, r = {}, 0
    for name, v in expect:
        scalar = not isinstance(v, np.ndarray)
        rec = recs[r] if r < len(recs) else None
        if scalar:
            if rec is not None and rec.ndim == 0:
                got[name] = rec.item()
                r += 1
            continue
        if rec is None:
            raise ValueError(f"checkpoint ends before leaf {name}")
        if rec.shape != v.shape:
            raise ValueError(f"leaf {name}: checkpoint shape {rec.shape}, model expects {v.shape}")
        got[name] = rec
        r += 1
    if r != len(recs):
        raise ValueError(f"checkpoint has {len(recs) - r} records beyond the model's leaves")
    return got


def _set_stats(model, got, d):
    aux = model.aux.detach().cpu().numpy().copy()
    aux[:d] = got["_data_mean"]
    aux[d:2 * d] = np.diag(np.atleast_2d(got["_data_cov"]))
    base_cov = got["base_dist._cov"]
    if not np.allclose(base_cov, np.eye(d) * base_cov[0, 0]) or got["base_dist._mean"].any():
        raise ValueError("only a zero-mean isotropic Gaussian base distribution is supported")
    aux[2 * d] = base_cov[0, 0]
    return aux


def load_eqx(model, path: str):
    """Load a reference checkpoint into `model` (same n_features, n_layers,
    hidden_size, num_bins); returns the model."""
    got = _read_leaves(path, _leaves(model))
    for name, want in (("_n_features", model.n_features), ("layers[1].bijector._num_bins", model.num_bins)):
        if name in got and int(got[name]) != int(want):
            raise ValueError(f"{name} = {got[name]} in the checkpoint, {want} in the model")
    d, L = model.n_features, model.n_layers
    masks = got["layers[1]._mask"].astype(bool)
    for l in range(L):
        if not np.array_equal(masks[l], ((np.arange(d) + l) % 2).astype(bool)):
            raise ValueError(f"layer {l}: coupling mask differs from ((arange(d) + l) % 2)")
    if got["layers[0]._mask"].any():
        raise ValueError("the affine layers' masks must be all False")
    for key, attr in (("_range_min", 0), ("_range_max", 1)):
        k = "layers[1].bijector." + key
        if k in got and float(got[k]) != model.spline_range[attr]:
            raise ValueError(f"{key} = {got[k]} in the checkpoint, {model.spline_range[attr]} in the model")
    nl = len(model.hidden_size) + 1
    layers = []
    for l in range(L):
        layers.append({"W": [got[f"conditioner.layers[{2 * i}].weight"][l] for i in range(nl)],
                       "b": [got[f"conditioner.layers[{2 * i}].bias"][l] for i in range(nl)],
                       "scale": float(got["layers[0].bijector.scale"][l]),
                       "shift": float(got["layers[0].bijector.shift"][l])})
    model.load_full(layers)
    aux = _set_stats(model, got, d)
    model.aux.copy_(model.aux.new_tensor(aux))
    return model


# ---------------------------------------------------------------- RealNVP
# RealNVP(n_features=d, n_layers=L, n_hidden=H) (realNVP.py:120-176): the
# NFModel fields, then base_dist, then affine_coupling -- one
# MaskedCouplingLayer built by eqx.filter_vmap over the layers, so its
# arrays carry a leading axis L: _mask [L, d] (float), MLPAffine's scale_MLP
# (Linear weight [L, H, d], bias [L, H], relu skipped, Linear weight
# [L, d, H], bias [L, d]), shift_MLP (the same) and dt (a Python number).
# RealNVP re-declares the NFModel fields, which keeps their position.

def _leaves_realnvp(model) -> list:
    d, L = model.n_features, model.n_layers
    aux = model.aux.detach().cpu().numpy().astype(np.float32)
    lay = model.layers_numpy()
    out = [("_n_features", int(d)),
           ("_data_mean", aux[:d].copy()),
           ("_data_cov", np.diag(aux[d:2 * d]).astype(np.float32)),
           ("base_dist._mean", np.zeros(d, np.float32)),
           ("base_dist._cov", (np.eye(d) * aux[2 * d]).astype(np.float32)),
           ("base_dist.learnable", False),
           ("affine_coupling._mask", aux[2 * d + 2:].reshape(L, d).copy())]
    for mlp in ("scale", "shift"):
        for i in range(2):
            out.append((f"{mlp}_MLP.layers[{2 * i}].weight", np.stack([x[mlp]["W"][i] for x in lay])))
            out.append((f"{mlp}_MLP.layers[{2 * i}].bias", np.stack([x[mlp]["b"][i] for x in lay])))
    out.append(("dt", int(model.dt) if float(model.dt).is_integer() else float(model.dt)))
    return out


def save_eqx_realnvp(model, path: str) -> None:
    with open(path, "wb") as f:
        for _, v in _leaves_realnvp(model):
            np.save(f, np.asarray(v), allow_pickle=False)


def load_eqx_realnvp(model, path: str):
    got = _read_leaves(path, _leaves_realnvp(model))
    d, L = model.n_features, model.n_layers
    if "_n_features" in got and int(got["_n_features"]) != d:
        raise ValueError(f"_n_features = {got['_n_features']} in the checkpoint, {d} in the model")
    if "dt" in got and float(got["dt"]) != float(model.dt):
        raise ValueError(f"dt = {got['dt']} in the checkpoint, {model.dt} in the model")
    layers = []
    for l in range(L):
        layers.append({mlp: {"W": [got[f"{mlp}_MLP.layers[{2 * i}].weight"][l] for i in range(2)],
                             "b": [got[f"{mlp}_MLP.layers[{2 * i}].bias"][l] for i in range(2)]}
                       for mlp in ("scale", "shift")})
    model.load_layers(layers)
    aux = _set_stats(model, got, d)
    aux[2 * d + 2:] = np.asarray(got["affine_coupling._mask"], np.float32).ravel()
    model.aux.copy_(model.aux.new_tensor(aux))
    return model
