"""Golden vectors from the reference's own source code.

Runs flowMC v0.4.5's MALA, HMC and GaussianRandomWalk kernels
(resource/kernel/MALA.py:26-89, HMC.py:98-151, Gaussian_random_walk.py:25-61)
and its RQSpline bijection (knots, forward and inverse:
resource/model/nf_model/rqSpline.py:20-239, 296-362) on scripted normals and
uniforms, and saves inputs and outputs to ``reference_vectors.npz`` beside
this file. JAX is not installed here, so the reference modules run against
the stand-ins under ``_standin/`` (float64 torch tensors, autograd for
``jax.value_and_grad``/``jax.grad``, Python loops for ``lax.scan`` and
``vmap``, random keys that return the scripted draws). The targets are the
oracle's targets written with ``jax.numpy`` calls, so the reference kernels
differentiate them themselves.

Run in a checkout that has the reference source (REFERENCE_SRC, default
/root/reference/src):  python tests/golden/make_golden.py
"""
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REF = os.environ.get("REFERENCE_SRC", "/root/reference/src")
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
    for c in cases:
        if c["kind"] in ("mala", "hmc", "grw"):
            print(f"{c['name']}: acceptance {out[c['name'] + '/acc'].mean():.2f}")
    out["cases"] = np.array(json.dumps(cases))
    path = os.path.join(HERE, "reference_vectors.npz")
    np.savez_compressed(path, **out)
    print(f"wrote {path}: {len(cases)} cases")


if __name__ == "__main__":
    main()
