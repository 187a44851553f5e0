"""AdamOptimization (strategy/optimization.py of the reference): the oracle
against golden vectors made by running the reference's own optimize() on
scripted gradient noise (tests/golden/make_golden.py), the strategy's
argument checks, and the fused CUDA optimiser against both."""
import json
import os

import numpy as np
import pytest
import torch

from flowmc_gb300 import targets as TG
from flowmc_gb300.random import PRNGKey
from flowmc_gb300.strategy.optimization import AdamOptimization
from oracle import optimization as OPT

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz")


def _cases():
    z = np.load(GOLD)
    return [c for c in json.loads(str(z["cases"])) if c["kind"] == "adam"]


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c["name"])
def test_oracle_adam_matches_reference_source(case):
    z = np.load(GOLD)
    n = case["name"]
    x, lp = OPT.adam_optimize(case["target"], z[f"{n}/x0"], case["n_steps"], case["learning_rate"],
                              case["noise_level"], z[f"{n}/xi"], z[f"{n}/bounds"])
    np.testing.assert_allclose(x, z[f"{n}/x"], rtol=1e-10, atol=1e-12)
    np.testing.assert_allclose(lp, z[f"{n}/logp"], rtol=1e-10, atol=1e-12)
    if case["target"]["kind"] == "dual_moon":
        # this fixture ends on its box, so the projection is exercised
        b = z[f"{n}/bounds"]
        assert (np.abs(z[f"{n}/x"]) == b[0, 1]).any()


def test_adam_strategy_argument_checks():
    tgt = TG.DiagGaussian(3, device="cpu")
    opt = AdamOptimization(tgt)
    assert repr(opt) == "AdamOptimization" and opt.bounds.shape == (1, 2)
    with pytest.raises(ValueError, match="bounds must have shape"):
        AdamOptimization(tgt, bounds=np.array([-1.0, 1.0]))
    with pytest.raises(ValueError, match="bounds must have shape"):
        AdamOptimization(tgt, bounds=np.zeros((3, 3)))
    with pytest.raises(NotImplementedError):
        opt.optimize(PRNGKey(0), lambda p, d: -p.sum(), np.zeros((2, 3)), {})


def _f32(a):
    return torch.tensor(np.asarray(a), dtype=torch.float32, device="cuda")


def _dev_target(t):
    if t["kind"] == "rosenbrock":
        return TG.Rosenbrock(t["n_dim"], a=t["a"], b=t["b"], c=t["c"])
    if t["kind"] == "dual_moon":
        return TG.DualMoon(t["n_dim"], r0=t["r0"], sr=t["sr"], mu=t["mu"], s0=t["s0"])
    raise ValueError(t["kind"])


@pytest.mark.gpu
@pytest.mark.parametrize("case", _cases(), ids=lambda c: c["name"])
def test_cuda_adam_matches_reference_source(cuda, case):
    z = np.load(GOLD)
    n = case["name"]
    opt = AdamOptimization(_dev_target(case["target"]), n_steps=case["n_steps"],
                           learning_rate=case["learning_rate"], noise_level=case["noise_level"],
                           bounds=z[f"{n}/bounds"])
    _, x, lp = opt.optimize(PRNGKey(0), None, _f32(z[f"{n}/x0"]), {}, noise=_f32(z[f"{n}/xi"]))
    # float32 Adam: 1 - 0.999^t loses about 4 digits at small t, so positions
    # agree to about 1e-4 of the step scale
    np.testing.assert_allclose(x.cpu().numpy(), z[f"{n}/x"], rtol=2e-4, atol=2e-4)
    np.testing.assert_allclose(lp.cpu().numpy(), z[f"{n}/logp"], rtol=1e-3, atol=1e-3)


@pytest.mark.gpu
def test_cuda_adam_matches_oracle_mixture(cuda):
    rng = np.random.default_rng(4)
    d, C, S = 20, 96, 60
    tgt = TG.GaussianMixture(rng.normal(size=(3, d)) * 2, np.full((3, d), 0.8), [0.3, 0.3, 0.4])
    x0 = rng.normal(size=(C, d)) * 2
    xi = rng.normal(size=(C, S))
    b = np.stack([np.full(d, -2.5), np.full(d, 2.5)], axis=1)
    x_ref, lp_ref = OPT.adam_optimize(tgt.describe(), x0, S, 0.05, 0.3, xi, b)
    opt = AdamOptimization(tgt, n_steps=S, learning_rate=0.05, noise_level=0.3, bounds=b)
    _, x, lp = opt.optimize(PRNGKey(1), None, _f32(x0), {}, noise=_f32(xi))
    np.testing.assert_allclose(x.cpu().numpy(), x_ref, rtol=5e-4, atol=5e-4)
    np.testing.assert_allclose(lp.cpu().numpy(), lp_ref, rtol=1e-3, atol=1e-3)


@pytest.mark.gpu
def test_cuda_adam_philox_reaches_the_mode(cuda):
    """In-kernel noise: Adam with mild gradient noise drives every chain to
    the mode of a Gaussian; the strategy call returns the positions."""
    d, C = 7, 2048
    mean = np.linspace(-1, 1, d)
    tgt = TG.DiagGaussian(d, mean=mean, inv_var=np.linspace(0.5, 2, d))
    opt = AdamOptimization(tgt, n_steps=600, learning_rate=0.02, noise_level=0.2)
    g = torch.Generator(device="cuda").manual_seed(0)
    # Adam moves about one learning rate per step: start within reach
    _, _, x = opt(PRNGKey(2), {}, torch.randn(C, d, device="cuda", generator=g), {})
    # Adam at a fixed rate with noisy gradients settles in a band of a few
    # learning rates; the band's far tail (one coordinate in 10^4) reaches
    # about 0.1
    dev = np.abs(x.cpu().numpy() - mean)
    assert np.quantile(dev, 0.999) < 0.08
    assert dev.max() < 0.25
    np.testing.assert_allclose(x.cpu().numpy().mean(axis=0), mean, atol=0.01)
    # a different key gives different noise, so different (but converged) paths
    _, _, x2 = opt(PRNGKey(3), {}, torch.randn(C, d, device="cuda", generator=g), {})
    assert not torch.equal(x, x2)
