"""Golden vectors from the reference's own source code.

Runs flowMC v0.4.5's MALA, HMC and GaussianRandomWalk kernels
(resource/kernel/MALA.py:26-89, HMC.py:98-151, Gaussian_random_walk.py:25-61),
its RQSpline bijection (knots, forward and inverse:
resource/model/nf_model/rqSpline.py:20-239, 296-362), the whole
MaskedCouplingRQSpline (rqSpline.py:450-504), TakeSerialSteps.__call__ with
thinning into the reference's Buffers over several calls
(strategy/take_steps.py:60-180, resource/buffers.py:24-41), TrainModel's
training-data selection (strategy/train_model.py:66-80), NFProposal.kernel with its
batched and unbatched proposal draws (resource/kernel/NF_proposal.py:27-172),
RealNVP's layers (nf_model/realNVP.py:180-222), AdamOptimization.optimize
(strategy/optimization.py:85-164) and its
ParallelTempering ensemble step, exchange sweep and temperature adaptation
(strategy/parallel_tempering.py:205-436, on resource/logPDF.py's TemperedPDF)
on scripted normals and uniforms, and saves inputs and outputs to ``reference_vectors.npz`` beside
this file. JAX is not installed here, so the reference modules run against
the stand-ins under ``_standin/`` (float64 torch tensors, autograd for
``jax.value_and_grad``/``jax.grad``, Python loops for ``lax.scan`` and
``vmap``, random keys that return the scripted draws). The targets are the
oracle's targets written with ``jax.numpy`` calls, so the reference kernels
differentiate them themselves.

Run with REFERENCE_SRC set to the src/ directory of a flowMC v0.4.5
checkout:  REFERENCE_SRC=<checkout>/src python tests/golden/make_golden.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("REFERENCE_SRC")
if not REF or not os.path.isdir(os.path.join(REF, "flowMC")):
    sys.exit("set REFERENCE_SRC to the src/ directory of a flowMC v0.4.5 checkout")
sys.path.insert(0, os.path.join(HERE, "_standin"))
sys.path.insert(0, REF)

import numpy as np  # noqa: E402
import torch  # noqa: E402

import jax.numpy as jnp  # noqa: E402
from jax import random as jr  # noqa: E402
from flowMC.resource.kernel.Gaussian_random_walk import GaussianRandomWalk  # noqa: E402
from flowMC.resource.kernel.HMC import HMC  # noqa: E402
from flowMC.resource.kernel.MALA import MALA  # noqa: E402
from flowMC.resource.model.nf_model.rqSpline import RQSpline  # noqa: E402
from flowMC.resource.logPDF import TemperedPDF  # noqa: E402
from flowMC.strategy.parallel_tempering import ParallelTempering  # noqa: E402
from flowMC.strategy.optimization import AdamOptimization  # noqa: E402
from flowMC.resource.model.common import MLP, MLPAffine, MaskedCouplingLayer, ScalarAffine, Gaussian  # noqa: E402
from flowMC.resource.model.nf_model.rqSpline import MaskedCouplingRQSpline  # noqa: E402
from flowMC.resource.kernel.NF_proposal import NFProposal  # noqa: E402
from flowMC.resource.buffers import Buffer  # noqa: E402
from flowMC.resource.states import State  # noqa: E402
from flowMC.strategy.take_steps import TakeSerialSteps  # noqa: E402
from flowMC.strategy.train_model import TrainModel  # noqa: E402
from flowMC.resource.optimizer import Optimizer  # noqa: E402
from flowMC.resource.model.nf_model.realNVP import RealNVP  # noqa: E402
import jax  # noqa: E402


def jnp_target(t):
    """The oracle's target dict as a function of one position, in jax.numpy calls."""
    k = t["kind"]
    if k == "diag_gaussian":
        m, iv = torch.tensor(t["mean"]), torch.tensor(t["inv_var"])
        return lambda x, data: -0.5 * jnp.sum((x - m) ** 2 * iv) + t["const"]
    if k == "rosenbrock":
        a, b, c = t["a"], t["b"], t["c"]
        return lambda x, data: -jnp.sum((b - x[:-1]) ** 2 / a + c * (x[1:] - x[:-1] ** 2) ** 2)
    if k == "dual_moon":
        r0, sr, mu, s0 = t["r0"], t["sr"], t["mu"], t["s0"]

        def f(x, data):
            r = jnp.sqrt(jnp.sum(x * x))
            za, zb = (x[0] + mu) / s0, (x[0] - mu) / s0
            return -0.5 * ((r - r0) / sr) ** 2 + jnp.log(jnp.exp(-0.5 * za * za) + jnp.exp(-0.5 * zb * zb))
        return f
    raise ValueError(k)


def run_kernel(kernel, logpdf, x0, noise, unif):
    """TakeSerialSteps semantics for one chain: lp0 = logpdf(x0), then S kernel
    calls; step s uses key path s<c>.<s> whose split children get xi and u."""
    x = torch.tensor(x0)
    lp = logpdf(x, None)
    pos, lps, accs = [], [], []
    for s in range(noise.shape[0]):
        key = jr.Key(f"step{s}")
        jr.DRAWS[f"step{s}.0"] = noise[s]
        jr.DRAWS[f"step{s}.1"] = unif[s]
        x, lp, acc = kernel.kernel(key, x, lp, logpdf, None)
        x, lp = torch.as_tensor(x).detach(), torch.as_tensor(lp).detach()
        pos.append(x.numpy().copy())
        lps.append(float(lp))
        accs.append(float(bool(acc)))
    return np.array(pos), np.array(lps), np.array(accs)


def run_parallel_tempering(kernel, f, prior, temps, x0, noise, unif, u_ex):
    """ParallelTempering's ensemble step and exchange sweep for each chain
    (strategy/parallel_tempering.py:250-398), then the temperature adaptation
    on all chains' swap flags (400-436). Key paths: chain c's ensemble key
    pt<c> splits into one key per temperature, whose step-s subkey is
    <key>.0^s.1 (split children .0 normals, .1 uniform); the exchange key
    ex<c> gives step i the uniform at ex<c>.0^i.1."""
    C, Tn, S, d = noise.shape
    pt = ParallelTempering(n_steps=S, tempered_logpdf_name="tempered_logpdf", kernel_name="local_sampler",
                           tempered_buffer_names=["tempered_positions", "temperatures"], state_name="sampler_state")
    tlp = TemperedPDF(f, prior, n_dims=d, n_temps=Tn)
    tt = torch.tensor(temps)
    ens_x, ens_lp, ens_acc, ex_x, ex_lp, ex_acc = [], [], [], [], [], []
    for c in range(C):
        for t in range(Tn):
            for st in range(S):
                path = f"pt{c}.{t}" + ".0" * st + ".1"
                jr.DRAWS[path + ".0"] = noise[c, t, st]
                jr.DRAWS[path + ".1"] = unif[c, t, st]
        pos, lp, acc = pt._ensemble_step(kernel, jr.Key(f"pt{c}"), torch.tensor(x0[c]), tlp, tt, None)
        ens_x.append(pos.detach().numpy())
        ens_lp.append(lp.detach().numpy())
        ens_acc.append(torch.as_tensor(acc, dtype=torch.float64).numpy())
        for i in range(Tn - 1):
            jr.DRAWS[f"ex{c}" + ".0" * i + ".1"] = u_ex[c, i]
        pos2, lp2, acc2 = pt._exchange(jr.Key(f"ex{c}"), pos.detach(), tlp, tt, None)
        ex_x.append(pos2.detach().numpy())
        ex_lp.append(lp2.detach().numpy())
        ex_acc.append(torch.as_tensor(acc2, dtype=torch.float64).numpy())
    ex_acc = np.stack(ex_acc)
    new_t = pt._adapt_temperature(tt, torch.tensor(ex_acc)).numpy()
    return (np.stack(ens_x), np.stack(ens_lp), np.stack(ens_acc), np.stack(ex_x), np.stack(ex_lp), ex_acc, new_t)


class _Linear:
    """eqx.nn.Linear's call: weight @ x + bias."""

    def __init__(self, W, b):
        self.weight, self.bias = torch.tensor(W), torch.tensor(b)
        self.out_features, self.in_features = self.weight.shape

    def __call__(self, x):
        return self.weight @ x + self.bias


def _mlp(W1, b1, W2, b2):
    """The reference's MLP object with given weights (common.py:68-112: layers
    Linear, relu, Linear), built without Equinox's Linear constructor."""
    m = object.__new__(MLP)
    m.layers = [_Linear(W1, b1), jax.nn.relu, _Linear(W2, b2)]
    return m


def _mlp_tanh(Ws, bs):
    """The reference's MLP object (common.py:68-112) with given weights and
    tanh between the Linears, as MaskedCouplingRQSpline builds it."""
    m = object.__new__(MLP)
    m.layers = []
    for i, (W, b) in enumerate(zip(Ws, bs)):
        m.layers.append(_Linear(W, b))
        if i < len(Ws) - 1:
            m.layers.append(jax.nn.tanh)
    return m


def _rqspline_flow(layers, n_bins, mean, var, d):
    """A MaskedCouplingRQSpline whose attributes are set directly
    (rqSpline.py:392-443 without Equinox's stacking): per layer the pair
    [MaskedCouplingLayer(ScalarAffine(scale, shift), 0), MaskedCouplingLayer(
    RQSpline(MLP), mask)] of the reference's own classes, the base
    Gaussian(0, I), data_mean and diag data_cov. Masks are float 0/1, which
    the reference's bool masks promote to in (1 - mask) and x * mask."""
    flow = object.__new__(MaskedCouplingRQSpline)
    flow.layers = []
    for L in layers:
        spline = RQSpline(_mlp_tanh(L["W"], L["b"]), -10.0, 10.0)
        flow.layers.append([MaskedCouplingLayer(ScalarAffine(L["scale"], L["shift"]), torch.zeros(d, dtype=torch.float64)),
                            MaskedCouplingLayer(spline, torch.tensor(L["mask"], dtype=torch.float64))])
    flow.base_dist = Gaussian(torch.zeros(d, dtype=torch.float64), torch.eye(d, dtype=torch.float64), learnable=False)
    flow._data_mean = torch.tensor(mean)
    flow._data_cov = torch.diag(torch.tensor(var))
    flow._n_features = d
    return flow


class _RealNVPStandIn:
    """What RealNVP.forward / inverse / log_prob see (realNVP.py:180-222): the
    scan over the stacked layers is a loop over the reference's own
    MaskedCouplingLayer(MLPAffine(...)) objects."""

    def __init__(self, layers, mean, cov, d):
        self.layers, self.data_mean, self.data_cov, self.n_features = layers, mean, cov, d

    def __call__(self, x):
        return self.forward(x)

    def forward(self, x):
        ld = 0.0
        for lay in self.layers:
            x, ldi = lay(x, None)
            ld = ld + ldi
        return x, ld

    def inverse(self, x):
        ld = 0.0
        for lay in reversed(self.layers):
            x, ldi = lay.inverse(x, None)
            ld = ld + ldi
        return x, ld


class _Conditioner:
    """Stands in for the spline's MLP: returns fixed raw parameters."""

    def __init__(self, raw, n_in, n_out):
        self.raw, self.n_input, self.n_output, self.dtype = raw, n_in, n_out, torch.float64

    def __call__(self, condition):
        return self.raw


def main():
    rng = np.random.default_rng(20261204)
    out, cases = {}, []
    targets = {
        "dual_moon5": {"kind": "dual_moon", "n_dim": 5, "r0": 2.0, "sr": 0.1, "mu": 3.0, "s0": 0.6},
        "rosenbrock6": {"kind": "rosenbrock", "n_dim": 6, "a": 20.0, "b": 1.0, "c": 5.0},
        "diag4": {"kind": "diag_gaussian", "n_dim": 4, "mean": [0.5, -1.0, 0.0, 2.0],
                  "inv_var": [1.0, 2.0, 0.5, 4.0], "const": 0.0},
    }
    M_spd = None
    plans = [("mala", "dual_moon5", 0.2, 0, None), ("mala", "rosenbrock6", 0.35, 0, None),
             ("mala", "diag4", 0.4, 0, None), ("hmc", "rosenbrock6", 0.02, 5, "eye"),
             ("hmc", "diag4", 0.15, 4, "spd"), ("grw", "dual_moon5", 0.1, 0, None), ("grw", "diag4", 0.6, 0, None)]
    S, C = 20, 3
    for kind, tname, step, nlf, mass in plans:
        t = targets[tname]
        d = t["n_dim"]
        x0 = rng.normal(size=(C, d))
        if tname == "dual_moon5":
            x0 = x0 / np.linalg.norm(x0, axis=1, keepdims=True) * 2.0
        if tname == "rosenbrock6":
            x0 = 0.3 * x0 + 0.5
        noise = rng.normal(size=(C, S, d))
        unif = rng.uniform(1e-6, 1.0, size=(C, S))
        M = None
        if kind == "hmc":
            if mass == "eye":
                M = np.eye(d)
            else:
                Q, _ = np.linalg.qr(rng.normal(size=(d, d)))
                M = Q @ np.diag(rng.uniform(0.5, 2.0, size=d)) @ Q.T
            kern = HMC(condition_matrix=torch.tensor(M), step_size=step, n_leapfrog=nlf)
        elif kind == "mala":
            kern = MALA(step)
        else:
            kern = GaussianRandomWalk(step)
        f = jnp_target(t)
        res = [run_kernel(kern, f, x0[c], noise[c], unif[c]) for c in range(C)]
        name = f"{kind}_{tname}"
        out[f"{name}/x0"] = x0
        out[f"{name}/noise"] = noise
        out[f"{name}/unif"] = unif
        out[f"{name}/pos"] = np.stack([r[0] for r in res])
        out[f"{name}/logp"] = np.stack([r[1] for r in res])
        out[f"{name}/acc"] = np.stack([r[2] for r in res])
        if M is not None:
            out[f"{name}/M"] = M
        cases.append({"name": name, "kind": kind, "target": t, "step_size": step, "n_leapfrog": nlf})
    # RQSpline: knots from raw conditioner outputs, forward and inverse (tails included)
    for K, scale in ((8, 1.0), (12, 2.5)):
        d = 7
        P = 3 * K + 1
        raw = rng.normal(size=(d * P,)) * scale
        x = np.concatenate([rng.normal(size=d - 2) * 4.0, [-11.5, 12.0]])
        sp = RQSpline(_Conditioner(torch.tensor(raw), d, d * P), -10.0, 10.0)
        y, ldf = sp.forward(torch.tensor(x), None)
        xi, ldi = sp.inverse(torch.tensor(x), None)
        name = f"rqspline_K{K}"
        out[f"{name}/raw"] = raw.reshape(d, P)
        out[f"{name}/x"] = x
        out[f"{name}/fwd_y"] = y.numpy()
        out[f"{name}/fwd_logdet"] = ldf.numpy()
        out[f"{name}/inv_x"] = xi.numpy()
        out[f"{name}/inv_logdet"] = ldi.numpy()
        cases.append({"name": name, "kind": "rqspline", "n_bins": K})
    # ParallelTempering: tempered ensemble steps, exchange sweep, adaptation
    pt_plans = [("mala", "dual_moon5", 0.25, 0, None, 5.0), ("grw", "diag4", 0.8, 0, "gauss", 8.0),
                ("hmc", "rosenbrock6", 0.02, 4, None, 3.0)]
    C, Tn, S = 3, 4, 6
    for kind, tname, step, nlf, prior_kind, tmax in pt_plans:
        t = targets[tname]
        d = t["n_dim"]
        temps = np.linspace(1.0, tmax, Tn)
        x0 = rng.normal(size=(C, Tn, d))
        if tname == "dual_moon5":
            x0 = x0 / np.linalg.norm(x0, axis=-1, keepdims=True) * 2.0
        if tname == "rosenbrock6":
            x0 = 0.3 * x0 + 0.5
        noise = rng.normal(size=(C, Tn, S, d))
        unif = rng.uniform(1e-6, 1.0, size=(C, Tn, S))
        u_ex = rng.uniform(1e-6, 1.0, size=(C, Tn - 1))
        if kind == "mala":
            kern = MALA(step)
        elif kind == "grw":
            kern = GaussianRandomWalk(step)
        else:
            kern = HMC(condition_matrix=torch.eye(d, dtype=torch.float64), step_size=step, n_leapfrog=nlf)
        prior = {"mean": rng.normal(size=d) * 0.5, "inv_var": rng.uniform(0.2, 1.0, size=d), "const": -0.75} \
            if prior_kind == "gauss" else None
        if prior is None:
            prior_f = lambda x, _: 0.0  # noqa: E731  (the bundle's default prior)
        else:
            pm, piv, pc = torch.tensor(prior["mean"]), torch.tensor(prior["inv_var"]), prior["const"]
            prior_f = lambda x, _: -0.5 * jnp.sum((x - pm) ** 2 * piv) + pc  # noqa: E731
        res = run_parallel_tempering(kern, jnp_target(t), prior_f, temps, x0, noise, unif, u_ex)
        name = f"pt_{kind}_{tname}"
        for key, val in zip(("x0", "noise", "unif", "u_exchange", "temps"), (x0, noise, unif, u_ex, temps)):
            out[f"{name}/{key}"] = val
        for key, val in zip(("ens_x", "ens_lp", "ens_acc", "ex_x", "ex_lp", "ex_acc", "new_temps"), res):
            out[f"{name}/{key}"] = val
        case = {"name": name, "kind": "pt", "local": kind, "target": t, "step_size": step, "n_leapfrog": nlf}
        if prior is not None:
            case["prior"] = {k: np.asarray(v).tolist() for k, v in prior.items()}
        cases.append(case)
    # temperature adaptation alone on many chains (damping of order one)
    pt = ParallelTempering(1, "tempered_logpdf", "local_sampler", ["tempered_positions", "temperatures"],
                           "sampler_state")
    temps = np.array([1.0, 1.7, 2.9, 4.4, 6.0, 9.0])
    flags = (rng.uniform(size=(200, 5)) < np.array([0.9, 0.6, 0.75, 0.3, 0.5])).astype(np.float64)
    out["pt_adapt/temps"] = temps
    out["pt_adapt/flags"] = flags
    out["pt_adapt/new_temps"] = pt._adapt_temperature(torch.tensor(temps), torch.tensor(flags)).numpy()
    cases.append({"name": "pt_adapt", "kind": "pt_adapt"})
    # AdamOptimization.optimize: chain c's key is root.1.c, step s's gradient
    # noise the scalar normal at root.1.c.0^s.1 (optimization.py:117-157)
    for tname, n_steps, lr, nl, bounds in (("rosenbrock6", 25, 0.05, 0.5, "per_dim"),
                                           ("dual_moon5", 30, 0.1, 2.0, "broadcast")):
        t = targets[tname]
        d = t["n_dim"]
        C = 3
        x0 = rng.normal(size=(C, d))
        xi = rng.normal(size=(C, n_steps))
        if bounds == "per_dim":
            b = np.stack([np.full(d, -0.4), np.full(d, 0.6)], axis=1)
            b[::2, 0] = -np.inf
        else:
            b = np.array([[-1.5, 1.5]])
        for c in range(C):
            for st in range(n_steps):
                jr.DRAWS[f"opt.1.{c}" + ".0" * st + ".1"] = xi[c, st]
        opt = AdamOptimization(jnp_target(t), n_steps=n_steps, learning_rate=lr, noise_level=nl,
                               bounds=torch.tensor(b))
        f = jnp_target(t)
        _, xo, lpo = opt.optimize(jr.Key("opt"), lambda p, data: -f(p, data), torch.tensor(x0), None)
        name = f"adam_{tname}"
        for key, val in (("x0", x0), ("xi", xi), ("bounds", b), ("x", xo.detach().numpy()),
                         ("logp", lpo.detach().numpy())):
            out[f"{name}/{key}"] = val
        cases.append({"name": name, "kind": "adam", "target": t, "n_steps": n_steps, "learning_rate": lr,
                      "noise_level": nl})
    # RealNVP: the reference's MaskedCouplingLayer / MLPAffine / MLP and
    # RealNVP.log_prob on fixed weights; masks as float leaves, one case with
    # weight-decayed masks (0.9999 / 1e-4 instead of 1 / 0 would not arise, but
    # decay scales the ones: 1 -> 0.9998)
    for name, d, L, H, decay in (("realnvp_d5", 5, 4, 8, 1.0), ("realnvp_d6_decayed", 6, 3, 16, 0.9998)):
        masks, Ws = [], []
        for l in range(L):
            m = np.ones(d)
            m[: int(d / 2)] = 0.0
            m = 1 - m if l % 2 == 0 else m
            masks.append(m * decay)
            Ws.append([rng.normal(size=(H, d)) * 0.5, rng.normal(size=H) * 0.3, rng.normal(size=(d, H)) * 0.3,
                       rng.normal(size=d) * 0.3, rng.normal(size=(H, d)) * 0.5, rng.normal(size=H) * 0.3,
                       rng.normal(size=(d, H)) * 0.3, rng.normal(size=d) * 0.3])
        layers = [MaskedCouplingLayer(MLPAffine(_mlp(*w[:4]), _mlp(*w[4:])), torch.tensor(m))
                  for w, m in zip(Ws, masks)]
        mean, var = rng.normal(size=d) * 0.5, rng.uniform(0.5, 2.0, size=d)
        flow = _RealNVPStandIn(layers, torch.tensor(mean), torch.diag(torch.tensor(var)), d)
        x = rng.normal(size=(7, d)) * 1.5
        fy, fld, iy, ild, lp = [], [], [], [], []
        for row in x:
            y, ld = flow.forward(torch.tensor(row))
            fy.append(y.numpy()), fld.append(float(ld))
            xi, ldi = flow.inverse(torch.tensor(row))
            iy.append(xi.numpy()), ild.append(float(ldi))
            lp.append(float(RealNVP.log_prob(flow, torch.tensor(row))))
        out[f"{name}/x"] = x
        out[f"{name}/masks"] = np.stack(masks)
        out[f"{name}/mean"], out[f"{name}/var"] = mean, var
        for i, key in enumerate(("W1s", "b1s", "W2s", "b2s", "W1t", "b1t", "W2t", "b2t")):
            out[f"{name}/{key}"] = np.stack([w[i] for w in Ws])
        out[f"{name}/fwd_y"], out[f"{name}/fwd_logdet"] = np.stack(fy), np.array(fld)
        out[f"{name}/inv_x"], out[f"{name}/inv_logdet"] = np.stack(iy), np.array(ild)
        out[f"{name}/log_prob"] = np.array(lp)
        cases.append({"name": name, "kind": "realnvp", "n_dim": d, "n_layers": L, "n_hidden": H})
    # MaskedCouplingRQSpline: the reference's forward, inverse (its layer and
    # ScalarAffine order) and log_prob (standardisation, base Gaussian) on
    # fixed weights with non-zero ScalarAffine scale and shift; inputs reach
    # both spline tails
    for name, d, L, hidden, K in (("rqsflow_d5", 5, 3, [8, 8], 4), ("rqsflow_d6", 6, 2, [12], 5)):
        P = 3 * K + 1
        layers = []
        for l in range(L):
            shape = [d] + hidden + [d * P]
            layers.append({"W": [rng.normal(size=(b, a)) * 0.6 for a, b in zip(shape[:-1], shape[1:])],
                           "b": [rng.normal(size=b) * 0.3 for b in shape[1:]],
                           "scale": float(rng.normal() * 0.3), "shift": float(rng.normal() * 0.5),
                           "mask": ((np.arange(d) + l) % 2).astype(np.float64)})
        mean, var = rng.normal(size=d) * 0.5, rng.uniform(0.5, 2.0, size=d)
        flow = _rqspline_flow(layers, K, mean, var, d)
        x = rng.normal(size=(9, d)) * 4.0
        x[0, 0], x[1, 1] = 30.0, -30.0          # beyond the spline range after standardising
        fy, fld, iy, ild, lp = [], [], [], [], []
        for row in x:
            y, ld = MaskedCouplingRQSpline.forward(flow, torch.tensor(row))
            fy.append(y.numpy()), fld.append(float(ld))
            xi, ldi = MaskedCouplingRQSpline.inverse(flow, torch.tensor(row))
            iy.append(xi.numpy()), ild.append(float(ldi))
            lp.append(float(MaskedCouplingRQSpline.log_prob(flow, torch.tensor(row))))
        out[f"{name}/x"] = x
        out[f"{name}/mean"], out[f"{name}/var"] = mean, var
        for l, Ld in enumerate(layers):
            for i, (W, b) in enumerate(zip(Ld["W"], Ld["b"])):
                out[f"{name}/W{l}_{i}"], out[f"{name}/b{l}_{i}"] = W, b
        out[f"{name}/scale"] = np.array([Ld["scale"] for Ld in layers])
        out[f"{name}/shift"] = np.array([Ld["shift"] for Ld in layers])
        out[f"{name}/fwd_y"], out[f"{name}/fwd_logdet"] = np.stack(fy), np.array(fld)
        out[f"{name}/inv_x"], out[f"{name}/inv_logdet"] = np.stack(iy), np.array(ild)
        out[f"{name}/log_prob"] = np.array(lp)
        cases.append({"name": name, "kind": "rqsflow", "n_dim": d, "n_layers": L, "hidden": hidden, "n_bins": K})
    # NFProposal.kernel (NF_proposal.py:27-172) per chain on a 5-D dual moon
    # with a MaskedCouplingRQSpline proposal: once with the proposals drawn in
    # one batch, once through sample_flow's batched scan (n_batch_size 3 for
    # 7 steps: three draws of 3 rows, the last two rows dropped) and the
    # chunked target evaluation. The normals each chain's proposals start
    # from are saved as the [S, d] rows the proposals use.
    t_nf = targets["dual_moon5"]
    for name, bs in (("nfprop_dual_moon5", 100), ("nfprop_dual_moon5_batched", 3)):
        d, L, hidden, K, C, S = 5, 2, [8], 6, 3, 7
        P = 3 * K + 1
        layers = []
        for l in range(L):
            shape = [d] + hidden + [d * P]
            layers.append({"W": [rng.normal(size=(b, a)) * 0.3 for a, b in zip(shape[:-1], shape[1:])],
                           "b": [rng.normal(size=b) * 0.2 for b in shape[1:]],
                           "scale": float(0.35 + 0.05 * rng.normal()), "shift": float(0.1 * rng.normal()),
                           "mask": ((np.arange(d) + l) % 2).astype(np.float64)})
        mean, var = rng.normal(size=d) * 0.2, rng.uniform(0.8, 1.5, size=d)
        flow = _rqspline_flow(layers, K, mean, var, d)
        prop = object.__new__(NFProposal)
        prop.model, prop.n_batch_size = flow, bs
        f = jnp_target(t_nf)
        # chains start far outside the target's shell, so proposals nearer it
        # are accepted and the accept/reject mix is not one-sided
        x0 = rng.normal(size=(C, d)) * 4.0
        unif = rng.uniform(size=(C, S))
        z_used = np.empty((C, S, d))
        pos, lps, accs = [], [], []
        for c in range(C):
            if S > bs:
                n_batch = -(-S // bs)
                n_sample = -(-S // n_batch)
                zb = rng.normal(size=(n_batch, n_sample, d))
                for b in range(n_batch):
                    jr.DRAWS[f"nf{name}{c}.1" + ".0" * b + ".1"] = zb[b]
                z_used[c] = zb.reshape(-1, d)[:S]
            else:
                z_used[c] = rng.normal(size=(S, d))
                jr.DRAWS[f"nf{name}{c}.1"] = z_used[c]
            for s in range(S):
                jr.DRAWS[f"nf{name}{c}.0" + ".0" * s + ".1"] = unif[c, s]
            xc = torch.tensor(x0[c])
            lp0 = f(xc, None)                                         # take_steps.py:200-206
            px, plp, pacc = prop.kernel(jr.Key(f"nf{name}{c}"), xc, lp0, f, {"n_steps": S})
            pos.append(torch.as_tensor(px).detach().numpy())
            lps.append(torch.as_tensor(plp).detach().numpy())
            accs.append(torch.as_tensor(pacc, dtype=torch.float64).numpy())
        out[f"{name}/x0"], out[f"{name}/z"], out[f"{name}/unif"] = x0, z_used, unif
        out[f"{name}/mean"], out[f"{name}/var"] = mean, var
        for l, Ld in enumerate(layers):
            for i, (W, b) in enumerate(zip(Ld["W"], Ld["b"])):
                out[f"{name}/W{l}_{i}"], out[f"{name}/b{l}_{i}"] = W, b
        out[f"{name}/scale"] = np.array([Ld["scale"] for Ld in layers])
        out[f"{name}/shift"] = np.array([Ld["shift"] for Ld in layers])
        out[f"{name}/pos"], out[f"{name}/logp"], out[f"{name}/acc"] = np.stack(pos), np.stack(lps), np.stack(accs)
        cases.append({"name": name, "kind": "nfproposal", "target": t_nf, "n_dim": d, "n_layers": L,
                      "hidden": hidden, "n_bins": K, "n_batch_size": bs})
    # TakeSerialSteps.__call__ (take_steps.py:60-180) with MALA and thinning 3
    # over 7 steps, called three times into the reference's Buffers of 6 rows:
    # each call writes ceil(7/3) = 3 rows but advances the cursor by 7 // 3 = 2,
    # and the third call's start (4) is clamped to 3 by the buffer update
    name, S, thin, n_calls, R = "takesteps_mala_thin3", 7, 3, 3, 6
    t = targets["dual_moon5"]
    C, d = 3, 5
    f = jnp_target(t)
    res = {"MALA": MALA(0.2), "logpdf": f,
           "p": Buffer("p", (C, R, d), 1), "l": Buffer("l", (C, R), 1), "a": Buffer("a", (C, R), 1),
           "state": State({"p": "p", "l": "l", "a": "a"}, name="state")}
    strat = TakeSerialSteps("logpdf", "MALA", "state", ["p", "l", "a"], n_steps=S, thinning=thin)
    x = torch.tensor(rng.normal(size=(C, d)) * 1.5)
    x0 = x.numpy().copy()
    noise = rng.normal(size=(n_calls, C, S, d))
    unif = rng.uniform(size=(n_calls, C, S))
    lasts, cursors = [], []
    for k in range(n_calls):
        for c in range(C):
            for s in range(S):
                path = f"ts{k}.1.{c}" + ".0" * s + ".1"
                jr.DRAWS[path + ".0"] = noise[k, c, s]
                jr.DRAWS[path + ".1"] = unif[k, c, s]
        _, res, x = strat(jr.Key(f"ts{k}"), res, x, None)
        x = torch.as_tensor(x).detach()
        lasts.append(x.numpy().copy())
        cursors.append(strat.current_position)
    out[f"{name}/x0"], out[f"{name}/noise"], out[f"{name}/unif"] = x0, noise, unif
    out[f"{name}/pos_buf"] = torch.as_tensor(res["p"].data).numpy()
    out[f"{name}/logp_buf"] = torch.as_tensor(res["l"].data).numpy()
    out[f"{name}/acc_buf"] = torch.as_tensor(res["a"].data).numpy()
    out[f"{name}/last"], out[f"{name}/cursor"] = np.stack(lasts), np.array(cursors)
    cases.append({"name": name, "kind": "takesteps", "local": "mala", "target": t, "step_size": 0.2,
                  "n_steps": S, "thinning": thin, "n_calls": n_calls, "buf_rows": R})
    # TrainModel.__call__'s data selection (train_model.py:66-80): a buffer
    # with unfilled (-inf) rows, the history window, and scripted
    # jax.random.choice indices; the model's train() is replaced by a recorder
    # of the rows it was given
    name, C, Sb, d, window, n_max = "train_select", 4, 9, 3, 5, 23
    buf = rng.normal(size=(C, Sb, d))
    buf[:, 7:] = -np.inf                                   # two rows per chain not yet written
    choice = rng.integers(0, C * window, size=n_max)
    jr.DRAWS["tm.1"] = choice
    seen = {}

    def _record(rng, data, optim, state, num_epochs, batch_size, verbose):
        seen["data"] = torch.as_tensor(data).numpy().copy()
        return rng, model, state, torch.zeros(num_epochs, dtype=torch.float64)
    model = object.__new__(MaskedCouplingRQSpline)
    model.train = _record
    opt = object.__new__(Optimizer)
    opt.optim, opt.optim_state = None, None
    data_buf = Buffer("data", (C, Sb, d), 1)
    data_buf.data = torch.tensor(buf)
    tm = TrainModel("model", "data", "opt", n_epochs=2, batch_size=8, n_max_examples=n_max,
                    history_window=window)
    tm(jr.Key("tm"), {"model": model, "data": data_buf, "opt": opt}, torch.zeros(C, d), None)
    out[f"{name}/buf"], out[f"{name}/choice"], out[f"{name}/selected"] = buf, choice, seen["data"]
    cases.append({"name": name, "kind": "train_select", "history_window": window, "n_max_examples": n_max})
    # NFModel.loss_fn (nf_model/base.py:98-100), -mean(vmap(log_prob)(x)), run
    # by the reference's own code on a flow of the reference's classes; its
    # gradient with respect to every trainable leaf (per layer ScalarAffine
    # scale and shift, each conditioner Linear's weight and bias) comes from
    # autograd, the stand-in for eqx.filter_value_and_grad. Inputs reach both
    # spline tails.
    name, d, L, hidden, K = "nfloss_d5", 5, 3, [8, 8], 4
    P = 3 * K + 1
    layers = []
    for l in range(L):
        shape = [d] + hidden + [d * P]
        layers.append({"W": [rng.normal(size=(b, a)) * 0.6 for a, b in zip(shape[:-1], shape[1:])],
                       "b": [rng.normal(size=b) * 0.3 for b in shape[1:]],
                       "scale": float(rng.normal() * 0.3), "shift": float(rng.normal() * 0.5),
                       "mask": ((np.arange(d) + l) % 2).astype(np.float64)})
    mean, var = rng.normal(size=d) * 0.5, rng.uniform(0.5, 2.0, size=d)
    flow = _rqspline_flow(layers, K, mean, var, d)
    x = rng.normal(size=(13, d)) * 3.0
    x[0, 0], x[1, 1] = 30.0, -30.0
    leaves = []
    for aff, spl in flow.layers:
        for t in (aff.bijector.scale, aff.bijector.shift):
            t.requires_grad_(True)
        lins = [m for m in spl.bijector.conditioner.layers if isinstance(m, _Linear)]
        for lin in lins:
            lin.weight.requires_grad_(True)
            lin.bias.requires_grad_(True)
        leaves.append((aff.bijector.scale, aff.bijector.shift, lins))
    loss = flow.loss_fn(torch.tensor(x))
    flat = [t for sc, sh, lins in leaves for t in [sc, sh] + [u for lin in lins for u in (lin.weight, lin.bias)]]
    grads = torch.autograd.grad(loss, flat)
    out[f"{name}/x"], out[f"{name}/mean"], out[f"{name}/var"] = x, mean, var
    for l, Ld in enumerate(layers):
        for i, (W, b) in enumerate(zip(Ld["W"], Ld["b"])):
            out[f"{name}/W{l}_{i}"], out[f"{name}/b{l}_{i}"] = W, b
    out[f"{name}/scale"] = np.array([Ld["scale"] for Ld in layers])
    out[f"{name}/shift"] = np.array([Ld["shift"] for Ld in layers])
    out[f"{name}/loss"] = np.array(float(loss.detach()))
    out[f"{name}/grad"] = np.concatenate([g.detach().numpy().ravel() for g in grads])
    cases.append({"name": name, "kind": "nfloss", "n_dim": d, "n_layers": L, "hidden": hidden, "n_bins": K})
    for c in cases:
        if c["kind"] == "nfproposal":
            print(f"{c['name']}: acceptance {out[c['name'] + '/acc'].mean():.2f}")
        if c["kind"] in ("mala", "hmc", "grw"):
            print(f"{c['name']}: acceptance {out[c['name'] + '/acc'].mean():.2f}")
        if c["kind"] == "pt":
            print(f"{c['name']}: step acceptance {out[c['name'] + '/ens_acc'].mean():.2f}, "
                  f"swaps {out[c['name'] + '/ex_acc'].mean():.2f}")
    out["cases"] = np.array(json.dumps(cases))
    path = os.path.join(HERE, "reference_vectors.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {len(cases)} cases")


if __name__ == "__main__":
    main()
