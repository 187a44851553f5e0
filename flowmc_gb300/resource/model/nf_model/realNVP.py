"""RealNVP (mirrors resource/model/nf_model/realNVP.py:18-228 of the reference)
on the fused kernels of libflowmc (csrc/realnvp.cu).

``RealNVP(n_features, n_layers, n_hidden, key)``: n_layers affine coupling
layers, each MaskedCouplingLayer(MLPAffine(scale_MLP, shift_MLP)) with MLPs
[d, H, d] and relu (the MLP class's default activation, common.py:84-90),
masks with the first floor(d/2) coordinates as the conditioning block on
even layers and the rest on odd layers (realNVP.py:163-169).

Parameters are one flat float32 vector ``theta`` (layout in
``include/flowmc.h``, ``FmcRealNVP``). ``aux`` holds data_mean,
diag(data_cov), the base Gaussian's covariance scale, a spare slot and the
coupling masks: all float leaves of the reference model that the optimiser's
weight decay moves (the masks included). Training uses the shared
``NFModel.train`` loop with ``fmc_rnvp_loss_grad``.
"""
from __future__ import annotations

import ctypes
import math

import numpy as np
import torch

from .... import _lib
from ....random import PRNGKey
from .base import NFModel


class FmcRealNVP(ctypes.Structure):
    _fields_ = [("n_dim", ctypes.c_int32), ("n_layers", ctypes.c_int32), ("n_hidden", ctypes.c_int32),
                ("dt", ctypes.c_float), ("theta", ctypes.c_void_p), ("aux", ctypes.c_void_p)]


_SIGS = {
    "fmc_rnvp_layout": (ctypes.c_int, [ctypes.POINTER(FmcRealNVP), ctypes.POINTER(ctypes.c_int64),
                                       ctypes.POINTER(ctypes.c_int64)]),
    "fmc_rnvp_workspace_size": (ctypes.c_int, [ctypes.POINTER(FmcRealNVP), ctypes.c_int64, ctypes.c_int32,
                                               ctypes.POINTER(ctypes.c_size_t)]),
    "fmc_rnvp_forward": (ctypes.c_int, [ctypes.POINTER(FmcRealNVP), ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "fmc_rnvp_inverse": (ctypes.c_int, [ctypes.POINTER(FmcRealNVP), ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "fmc_rnvp_log_prob": (ctypes.c_int, [ctypes.POINTER(FmcRealNVP), ctypes.c_void_p, ctypes.c_int64,
                                         ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "fmc_rnvp_sample": (ctypes.c_int, [ctypes.POINTER(FmcRealNVP), ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p,
                                       ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                       ctypes.c_void_p]),
    "fmc_rnvp_loss_grad": (ctypes.c_int, [ctypes.POINTER(FmcRealNVP), ctypes.c_void_p, ctypes.c_int64,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                          ctypes.c_void_p]),
}
for _name, (_res, _args) in _SIGS.items():
    _lib.register_extra(_name, _res, _args)


def realnvp_masks(d: int, n_layers: int) -> np.ndarray:
    """realNVP.py:163-169: ones with the first int(d/2) set to 0, flipped on even layers."""
    out = np.empty((n_layers, d), np.float32)
    for i in range(n_layers):
        m = np.ones(d, np.float32)
        m[: int(d / 2)] = 0.0
        out[i] = 1.0 - m if i % 2 == 0 else m
    return out


class RealNVP(NFModel):
    """RealNVP model defined in the paper https://arxiv.org/abs/1605.08803."""

    def __repr__(self):
        return "RealNVP with n_features=" + str(self._n_features) + ", n_layers=" + str(self.n_layers)

    def __init__(self, n_features: int, n_layers: int, n_hidden: int, key: PRNGKey, device=None, **kwargs):
        self._n_features = d = int(n_features)
        self.n_layers = L = int(n_layers)
        self.n_hidden = H = int(n_hidden)
        self.dt = 1.0
        self.precision = "float32"
        self.device = torch.device(device) if device is not None else (
            torch.device("cuda") if torch.cuda.is_available() else torch.device("cpu"))
        self.per_layer = 2 * H * d + 2 * H + 2 * (d * H + d)
        self.n_params = self.per_layer * L
        # the reference's initialisation (common.py:84-107 with scale 1e-4 and
        # relu): the hidden Linear's weights ~ N(0, 1e-4 / d); its bias and the
        # output Linear keep Equinox's default U(-1/sqrt(in), 1/sqrt(in))
        gen = np.random.default_rng(key.value if isinstance(key, PRNGKey) else int(key))
        layers = []
        for _l in range(L):
            lay = {}
            for name in ("scale", "shift"):
                W1 = gen.normal(size=(H, d)) * math.sqrt(1e-4 / d)
                b1 = gen.uniform(-1 / math.sqrt(d), 1 / math.sqrt(d), size=H)
                W2 = gen.uniform(-1 / math.sqrt(H), 1 / math.sqrt(H), size=(d, H))
                b2 = gen.uniform(-1 / math.sqrt(H), 1 / math.sqrt(H), size=d)
                lay[name] = {"W": [W1, W2], "b": [b1, b2]}
            layers.append(lay)
        mean = kwargs.get("data_mean")
        cov = kwargs.get("data_cov")
        aux = np.zeros(2 * d + 2 + L * d, np.float32)
        aux[:d] = 0.0 if mean is None else np.asarray(torch.as_tensor(mean).cpu(), np.float32)
        aux[d:2 * d] = 1.0 if cov is None else np.diag(np.atleast_2d(np.asarray(torch.as_tensor(cov).cpu())))
        aux[2 * d] = 1.0            # base Gaussian covariance scale (Gaussian(0, I))
        aux[2 * d + 1] = 1.0
        aux[2 * d + 2:] = realnvp_masks(d, L).ravel()
        self.theta = torch.zeros(self.n_params, dtype=torch.float32, device=self.device)
        self.aux = torch.tensor(aux, device=self.device)
        self._ws = _lib.Workspace()
        self.load_layers(layers)

    # ------------------------------------------------------------ parameters
    @property
    def n_features(self):
        return self._n_features

    @property
    def data_mean(self):
        return self.aux[: self._n_features]

    @property
    def data_cov(self):
        return torch.diag(self.aux[self._n_features: 2 * self._n_features])

    @property
    def masks(self) -> torch.Tensor:
        d = self._n_features
        return self.aux[2 * d + 2:].reshape(self.n_layers, d)

    def load_layers(self, layers: list):
        """layers[l] = {"scale": {"W": [W1 [H, d], W2 [d, H]], "b": [b1, b2]},
        "shift": {...}} in Equinox's Linear layout."""
        d, H = self._n_features, self.n_hidden
        vec = np.empty(self.n_params, np.float32)
        for l, lay in enumerate(layers):
            o = l * self.per_layer
            s, t = lay["scale"], lay["shift"]
            parts = [s["W"][0], t["W"][0], s["b"][0], t["b"][0], s["W"][1], s["b"][1], t["W"][1], t["b"][1]]
            shapes = [(H, d), (H, d), (H,), (H,), (d, H), (d,), (d, H), (d,)]
            for a, shp in zip(parts, shapes):
                a = np.asarray(a, np.float32)
                if a.shape != shp:
                    raise ValueError(f"layer {l}: parameter of shape {a.shape}, expected {shp}")
                vec[o:o + a.size] = a.ravel()
                o += a.size
        self.theta.copy_(torch.from_numpy(vec))

    def layers_numpy(self) -> list:
        """The inverse of load_layers (numpy arrays)."""
        d, H = self._n_features, self.n_hidden
        vec = self.theta.detach().cpu().numpy()
        out = []
        for l in range(self.n_layers):
            o = l * self.per_layer

            def take(shape):
                nonlocal o
                k = int(np.prod(shape))
                a = vec[o:o + k].reshape(shape).copy()
                o += k
                return a
            W1s, W1t, b1s, b1t = take((H, d)), take((H, d)), take((H,)), take((H,))
            W2s, b2s, W2t, b2t = take((d, H)), take((d,)), take((d, H)), take((d,))
            out.append({"scale": {"W": [W1s, W2s], "b": [b1s, b2s]}, "shift": {"W": [W1t, W2t], "b": [b1t, b2t]}})
        return out

    def c_struct(self) -> FmcRealNVP:
        s = FmcRealNVP()
        s.n_dim, s.n_layers, s.n_hidden, s.dt = self._n_features, self.n_layers, self.n_hidden, self.dt
        s.theta = _lib.ptr(self.theta)
        s.aux = _lib.ptr(self.aux)
        return s

    def sync_bf16(self):
        """FP32 model: nothing to re-pack."""

    # ------------------------------------------------------------ compute
    def _ws_get(self, n: int, mode: int, ws=None):
        s = self.c_struct()
        nb = ctypes.c_size_t()
        _lib.check(_lib.lib().fmc_rnvp_workspace_size(ctypes.byref(s), int(n), int(mode), ctypes.byref(nb)))
        ptr, size = (ws or self._ws).get(nb.value, self.device)
        return s, ptr, size

    def _as_rows(self, x):
        x = torch.as_tensor(x, dtype=torch.float32, device=self.device)
        single = x.dim() == 1
        x = (x.reshape(1, -1) if single else x).contiguous()
        if x.shape[1] != self._n_features:
            raise ValueError(f"inputs have {x.shape[1]} features, model has {self._n_features}")
        return x, single

    def _transform(self, x, fn):
        x, single = self._as_rows(x)
        n = x.shape[0]
        y = torch.empty_like(x)
        ld = torch.empty(n, device=self.device)
        s, ptr, size = self._ws_get(n, 0)
        _lib.check(getattr(_lib.lib(), fn)(ctypes.byref(s), x.data_ptr(), n, y.data_ptr(), ld.data_ptr(), ptr, size,
                                           _lib.stream_handle(self.device)))
        return (y[0], ld[0]) if single else (y, ld)

    def forward(self, x, key=None, condition=None):
        """realNVP.py:180-194: x -> (y, log_det), no standardisation."""
        return self._transform(x, "fmc_rnvp_forward")

    def inverse(self, x, condition=None):
        """realNVP.py:196-207: layers in reverse order."""
        return self._transform(x, "fmc_rnvp_inverse")

    def log_prob(self, x):
        """realNVP.py:215-222."""
        x, single = self._as_rows(x)
        n = x.shape[0]
        lp = torch.empty(n, device=self.device)
        s, ptr, size = self._ws_get(n, 0)
        _lib.check(_lib.lib().fmc_rnvp_log_prob(ctypes.byref(s), x.data_ptr(), n, lp.data_ptr(), ptr, size,
                                                _lib.stream_handle(self.device)))
        return lp[0] if single else lp

    def sample(self, rng_key: PRNGKey, n_samples: int, z=None):
        """realNVP.py:209-213; z [n, d] optionally gives the base normals."""
        n = int(n_samples)
        out = torch.empty(n, self._n_features, device=self.device)
        s, ptr, size = self._ws_get(n, 0)
        zp = None
        if z is not None:
            z = _lib.require_cuda_f32(torch.as_tensor(z, dtype=torch.float32, device=self.device).contiguous(), "z",
                                      (n, self._n_features))
            zp = z.data_ptr()
        _lib.check(_lib.lib().fmc_rnvp_sample(ctypes.byref(s), rng_key.value, 0, zp, n, out.data_ptr(), ptr, size,
                                              _lib.stream_handle(self.device)))
        return out

    def loss_and_grad(self, x, loss=None, grad=None):
        """-mean(log_prob(x)) and its gradient w.r.t. theta (nf_model/base.py:98-100)."""
        x = _lib.require_cuda_f32(torch.as_tensor(x).contiguous(), "x")
        n = x.shape[0]
        if not hasattr(self, "_ws_train"):
            self._ws_train = _lib.Workspace()
        s, ptr, size = self._ws_get(n, 1, self._ws_train)
        if loss is None:
            loss = torch.empty((), device=self.device)
        if grad is None:
            grad = torch.empty(self.n_params, device=self.device)
        _lib.check(_lib.lib().fmc_rnvp_loss_grad(ctypes.byref(s), x.data_ptr(), n, loss.data_ptr(), grad.data_ptr(),
                                                 ptr, size, _lib.stream_handle(self.device)))
        return loss, grad

    def print_parameters(self):
        print("RealNVP parameters:")
        print(f"Data mean: {self.data_mean}")
        print(f"Data covariance: {self.data_cov}")

    def save_model(self, path: str):
        from .eqx_format import save_eqx_realnvp
        save_eqx_realnvp(self, path + ".eqx")

    def load_model(self, path: str):
        from .eqx_format import load_eqx_realnvp
        return load_eqx_realnvp(self, path if path.endswith(".eqx") else path + ".eqx")

    save_resource = save_model
    load_resource = load_model
