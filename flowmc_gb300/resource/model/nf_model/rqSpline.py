"""MaskedCouplingRQSpline (mirrors resource/model/nf_model/rqSpline.py:364-507
of the reference) on the fused flow kernels of libflowmc.

Parameters live in one flat float32 device vector ``theta`` (plus a bf16
shadow for the BF16 conditioner path) in the packing of ``fmc_flow_layout``:
per layer scale, shift, then the conditioner Linear layers with the first
layer restricted to the conditioning coordinates and the last to the
transformed coordinates' outputs. The reference's remaining entries (first
layer columns that multiply masked-out zeros, last layer rows whose outputs
are masked away, common.py:155-157) never affect a result; they are kept on
the host for export, with the weight decay they accumulate tracked in
``aux[2d+1]``.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from .... import _lib
from ....random import PRNGKey, split
from .base import NFModel


def _layer_indices(d: int, l: int):
    """(conditioning, transformed) coordinates of layer l: mask (j + l) % 2
    (rqSpline.py:434) is 1 on the conditioning coordinates."""
    j = np.arange(d)
    mask = ((j + l) % 2).astype(bool)
    return np.nonzero(mask)[0], np.nonzero(~mask)[0]


class MaskedCouplingRQSpline(NFModel):
    def __repr__(self):
        return "MaskedCouplingRQSpline with n_features=" + str(self._n_features) + ", n_layers=" + str(self.n_layers)

    def __init__(self, n_features: int, n_layers: int, hidden_size: list, num_bins: int, key: PRNGKey,
                 spline_range: tuple = (-10.0, 10.0), precision: str = "float32", device=None, **kwargs):
        self._n_features = int(n_features)
        if not 2 <= self._n_features <= 4096:
            # at one feature every other layer has nothing to transform and the
            # rest condition on nothing: the packed conditioner GEMMs have no
            # zero-width form
            raise ValueError(f"MaskedCouplingRQSpline supports 2 to 4096 features, got {self._n_features}")
        self.n_layers = int(n_layers)
        self.hidden_size = [int(h) for h in hidden_size]
        if not 1 <= len(self.hidden_size) <= _lib.FMC_MAX_HIDDEN:
            raise ValueError(f"1 to {_lib.FMC_MAX_HIDDEN} hidden layers are supported")
        self.num_bins = int(num_bins)
        self.spline_range = (float(spline_range[0]), float(spline_range[1]))
        self.min_bin_size = 1e-4
        self.min_knot_slope = 1e-4
        self.device = torch.device(device) if device is not None else (
            torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu"))
        self.precision = precision
        self.gemm_bn = 0   # BF16 hidden-layer GEMM tile width; 0 = library choice (autotune.tune_flow_gemm)
        self.tile_rows = 0   # BF16 tensor-core tile rows (128 one CTA, 256 a CTA pair); 0 = library choice (128)
        self.gemm_stages = 0   # BF16 hidden GEMMs with K >= 256: 0/4 = 4-stage ring, 3 = 3 stages (autotune)
        self.wgrad_splits = 0  # BF16 training weight-gradient K slices; 0 = library choice (autotune.tune_flow_train)
        d = self._n_features
        P = 3 * self.num_bins + 1
        self._P = P
        self._layout()
        # the reference's initialisation (rqSpline.py:427-443, common.py:84-107):
        # hidden Linear weights ~ N(0, scale/in) with scale 1e-2; biases and the
        # last Linear keep Equinox's default U(-1/sqrt(in), 1/sqrt(in)).
        full = []
        gen = np.random.default_rng(key.value if isinstance(key, PRNGKey) else int(key))
        shape = [d] + self.hidden_size + [d * P]
        for _l in range(self.n_layers):
            Ws, bs = [], []
            for i, (a, b) in enumerate(zip(shape[:-1], shape[1:])):
                lim = 1.0 / math.sqrt(a)
                if i < len(shape) - 2:
                    W = gen.normal(size=(b, a)) * math.sqrt(1e-2 / a)
                else:
                    W = gen.uniform(-lim, lim, size=(b, a))
                bias = gen.uniform(-lim, lim, size=b)
                Ws.append(W.astype(np.float32))
                bs.append(bias.astype(np.float32))
            full.append({"W": Ws, "b": bs, "scale": 0.0, "shift": 0.0})
        self._full_init = full
        mean = kwargs.get("data_mean")
        cov = kwargs.get("data_cov")
        aux = np.zeros(2 * d + 2, np.float32)
        aux[:d] = 0.0 if mean is None else np.asarray(torch.as_tensor(mean).cpu(), np.float32)
        aux[d:2 * d] = 1.0 if cov is None else np.diag(np.atleast_2d(np.asarray(torch.as_tensor(cov).cpu())))
        aux[2 * d] = 1.0       # base Gaussian covariance scale
        aux[2 * d + 1] = 1.0   # decay of the packed-out entries
        self.theta = torch.zeros(self.n_params, dtype=torch.float32, device=self.device)
        self.aux = torch.tensor(aux, device=self.device)
        n16 = ctypes.c_int64(0)
        if _lib.LIB_PATH.exists():
            hs = self._host_struct()
            _lib.check(_lib.lib().fmc_flow_bf16_size(ctypes.byref(hs), ctypes.byref(n16)))
        self.theta_bf16 = torch.zeros(max(int(n16.value), 1), dtype=torch.bfloat16, device=self.device)
        self._ws = _lib.Workspace()
        self.load_full(full, sync=True)

    # ------------------------------------------------------------ layout
    def _layout(self):
        d, P = self._n_features, self._P
        self._slices = []   # per layer: list of (name, (offset, shape))
        off = 0
        self.layer_offsets = []
        for l in range(self.n_layers):
            self.layer_offsets.append(off)
            cidx, tidx = _layer_indices(d, l)
            ent = [("scale", off, ()), ("shift", off + 1, ())]
            off += 2
            ins = [len(cidx)] + self.hidden_size
            outs = self.hidden_size + [len(tidx) * P]
            for i, (a, b) in enumerate(zip(ins, outs)):
                ent.append((("W", i), off, (b, a)))
                off += a * b
                ent.append((("b", i), off, (b,)))
                off += b
            self._slices.append((cidx, tidx, ent))
        self.layer_offsets.append(off)
        self.n_params = off

    @property
    def n_features(self):
        return self._n_features

    @property
    def data_mean(self):
        return self.aux[: self._n_features]

    @property
    def data_cov(self):
        return torch.diag(self.aux[self._n_features: 2 * self._n_features])

    def c_struct(self) -> _lib.FmcFlow:
        s = _lib.FmcFlow()
        s.n_dim = self._n_features
        s.n_layers = self.n_layers
        s.n_hidden = len(self.hidden_size)
        s.n_bins = self.num_bins
        for i, h in enumerate(self.hidden_size):
            s.hidden[i] = h
        s.range_min, s.range_max = self.spline_range
        s.min_bin_size = self.min_bin_size
        s.min_knot_slope = self.min_knot_slope
        s.precision = _lib.PREC_BF16 if self.precision in ("bf16", "bfloat16") else _lib.PREC_FP32
        s.gemm_bn = int(getattr(self, "gemm_bn", 0))
        s.tile_rows = int(getattr(self, "tile_rows", 0))
        s.gemm_stages = int(getattr(self, "gemm_stages", 0))
        s.wgrad_splits = int(getattr(self, "wgrad_splits", 0))
        s.theta = _lib.ptr(self.theta)
        s.theta_bf16 = _lib.ptr(self.theta_bf16)
        s.aux = _lib.ptr(self.aux)
        return s

    def check_layout(self):
        """The library's packing agrees with this class's (raises otherwise)."""
        s = self.c_struct() if self.device.type == "cuda" else self._host_struct()
        n = ctypes.c_int64()
        offs = (ctypes.c_int64 * (self.n_layers + 1))()
        _lib.check(_lib.lib().fmc_flow_layout(ctypes.byref(s), ctypes.byref(n), offs))
        if n.value != self.n_params or list(offs) != self.layer_offsets:
            raise RuntimeError("parameter layout mismatch between host and libflowmc")

    def _host_struct(self):
        s = _lib.FmcFlow()
        s.n_dim, s.n_layers, s.n_hidden, s.n_bins = self._n_features, self.n_layers, len(self.hidden_size), self.num_bins
        for i, h in enumerate(self.hidden_size):
            s.hidden[i] = h
        s.range_min, s.range_max = self.spline_range
        s.min_bin_size, s.min_knot_slope = self.min_bin_size, self.min_knot_slope
        return s

    # ------------------------------------------------------------ import / export
    def load_full(self, layers: list, sync: bool = True):
        """Load reference-layout parameters: layers[l] = {"W": [...], "b": [...],
        "scale": s, "shift": t} with W_i [out, in] (Equinox's Linear)."""
        vec = np.zeros(self.n_params, np.float32)
        self._full_init = []
        for l, L in enumerate(layers):
            cidx, tidx, ent = self._slices[l]
            P = self._P
            rows = (tidx[:, None] * P + np.arange(P)[None]).ravel()
            Ws = [np.asarray(w, np.float32) for w in L["W"]]
            bs = [np.asarray(b, np.float32) for b in L["b"]]
            self._full_init.append({"W": [w.copy() for w in Ws], "b": [b.copy() for b in bs],
                                    "scale": float(L["scale"]), "shift": float(L["shift"])})
            nl = len(Ws) - 1
            for name, off, shp in ent:
                if name == "scale":
                    vec[off] = L["scale"]
                elif name == "shift":
                    vec[off] = L["shift"]
                else:
                    kind, i = name
                    if kind == "W":
                        W = Ws[i]
                        if i == 0:
                            W = W[:, cidx]
                        if i == nl:
                            W = W[rows]
                        vec[off:off + W.size] = W.ravel()
                    else:
                        b = bs[i]
                        if i == nl:
                            b = b[rows]
                        vec[off:off + b.size] = b
        self.theta.copy_(torch.from_numpy(vec))
        if self.device.type == "cuda":
            self.aux[2 * self._n_features + 1] = 1.0
        if sync:
            self.sync_bf16()

    def to_full(self) -> list:
        """Reference-layout parameters (numpy), packed-out entries included."""
        vec = self.theta.detach().cpu().numpy()
        decay = float(self.aux[2 * self._n_features + 1].item())
        out = []
        for l in range(self.n_layers):
            cidx, tidx, ent = self._slices[l]
            P = self._P
            rows = (tidx[:, None] * P + np.arange(P)[None]).ravel()
            init = self._full_init[l]
            Ws = [w * decay for w in init["W"]]
            bs = [b * decay for b in init["b"]]
            nl = len(Ws) - 1
            L = {"W": Ws, "b": bs, "scale": 0.0, "shift": 0.0,
                 "mask": ((np.arange(self._n_features) + l) % 2).astype(bool)}
            for name, off, shp in ent:
                n = int(np.prod(shp)) if shp else 1
                blk = vec[off:off + n].reshape(shp) if shp else float(vec[off])
                if name in ("scale", "shift"):
                    L[name] = blk
                else:
                    kind, i = name
                    tgt = Ws if kind == "W" else bs
                    if kind == "W":
                        if i == 0 and i == nl:
                            tgt[i][np.ix_(rows, cidx)] = blk
                        elif i == 0:
                            tgt[i][:, cidx] = blk
                        elif i == nl:
                            tgt[i][rows] = blk
                        else:
                            tgt[i] = blk.copy()
                    else:
                        if i == nl:
                            tgt[i][rows] = blk
                        else:
                            tgt[i] = blk.copy()
            out.append(L)
        return out

    def sync_bf16(self):
        if self.device.type != "cuda":
            return
        s = self.c_struct()
        _lib.check(_lib.lib().fmc_flow_sync_bf16(ctypes.byref(s), _lib.stream_handle(self.device)))

    # ------------------------------------------------------------ compute
    def _ws_infer(self, n: int):
        s = self.c_struct()
        nb = ctypes.c_size_t()
        _lib.check(_lib.lib().fmc_flow_workspace_size(ctypes.byref(s), int(n), 0, ctypes.byref(nb)))
        ptr, size = self._ws.get(nb.value, self.device)
        return s, ptr, size

    def _as_rows(self, x):
        x = torch.as_tensor(x, dtype=torch.float32, device=self.device)
        single = x.dim() == 1
        x = (x.reshape(1, -1) if single else x).contiguous()
        if x.shape[1] != self._n_features:
            raise ValueError(f"inputs have {x.shape[1]} features, model has {self._n_features}")
        return x, single

    def forward(self, x, key=None, condition=None):
        """rqSpline.py:450-468: x -> (y, log_det) (no standardisation)."""
        x, single = self._as_rows(x)
        n = x.shape[0]
        y = torch.empty_like(x)
        ld = torch.empty(n, device=self.device)
        s, ptr, size = self._ws_infer(n)
        _lib.check(_lib.lib().fmc_flow_forward(ctypes.byref(s), x.data_ptr(), n, y.data_ptr(), ld.data_ptr(), ptr,
                                               size, _lib.stream_handle(self.device)))
        return (y[0], ld[0]) if single else (y, ld)

    def inverse(self, x, condition=None):
        """rqSpline.py:470-488 (latent -> data), the reference's in-layer order."""
        x, single = self._as_rows(x)
        n = x.shape[0]
        y = torch.empty_like(x)
        ld = torch.empty(n, device=self.device)
        s, ptr, size = self._ws_infer(n)
        _lib.check(_lib.lib().fmc_flow_inverse(ctypes.byref(s), x.data_ptr(), n, y.data_ptr(), ld.data_ptr(), ptr,
                                               size, _lib.stream_handle(self.device)))
        return (y[0], ld[0]) if single else (y, ld)

    def log_prob(self, x):
        """rqSpline.py:498-504 (data space); x [d] or [n, d]."""
        x, single = self._as_rows(x)
        n = x.shape[0]
        lp = torch.empty(n, device=self.device)
        s, ptr, size = self._ws_infer(n)
        _lib.check(_lib.lib().fmc_flow_log_prob(ctypes.byref(s), x.data_ptr(), n, lp.data_ptr(), ptr, size,
                                                _lib.stream_handle(self.device)))
        return lp[0] if single else lp

    def sample(self, rng_key: PRNGKey, n_samples: int, z=None):
        """rqSpline.py:490-496; z [n, d] optionally gives the base normals."""
        n = int(n_samples)
        out = torch.empty(n, self._n_features, device=self.device)
        s, ptr, size = self._ws_infer(n)
        zp = None
        if z is not None:
            z = _lib.require_cuda_f32(torch.as_tensor(z, dtype=torch.float32, device=self.device).contiguous(), "z",
                                      (n, self._n_features))
            zp = z.data_ptr()
        _lib.check(_lib.lib().fmc_flow_sample(ctypes.byref(s), rng_key.value, 0, zp, n, out.data_ptr(), ptr, size,
                                              _lib.stream_handle(self.device)))
        return out

    def print_parameters(self):
        print("RQSpline parameters:")
        print(f"n_features: {self._n_features}, n_layers: {self.n_layers}, hidden: {self.hidden_size}, "
              f"num_bins: {self.num_bins}, precision: {self.precision}")
