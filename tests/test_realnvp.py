"""RealNVP (resource/model/nf_model/realNVP.py of the reference, with
common.py's MLP / MaskedCouplingLayer / MLPAffine): the oracle against golden
vectors made by the reference's own layer classes and RealNVP.log_prob
(tests/golden/make_golden.py), its gradient against finite differences, the
model's host-side layout and .eqx checkpoints, then the CUDA passes,
gradient, training and NF global step against the oracle."""
import json
import os

import numpy as np
import pytest
import torch

from flowmc_gb300.random import PRNGKey
from flowmc_gb300.resource.model.nf_model import eqx_format
from flowmc_gb300.resource.model.nf_model.realNVP import RealNVP, realnvp_masks
from oracle import realnvp as R

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz")


def _cases():
    z = np.load(GOLD)
    return [c for c in json.loads(str(z["cases"])) if c["kind"] == "realnvp"]


def _oracle_from_gold(z, n):
    params = {k: z[f"{n}/{k}"] for k in R.KEYS}
    return R.RealNVP(params, z[f"{n}/masks"], z[f"{n}/mean"], z[f"{n}/var"])


@pytest.mark.parametrize("case", _cases(), ids=lambda c: c["name"])
def test_oracle_realnvp_matches_reference_source(case):
    z = np.load(GOLD)
    n = case["name"]
    o = _oracle_from_gold(z, n)
    x = z[f"{n}/x"]
    y, ld = o.forward(x)
    np.testing.assert_allclose(y, z[f"{n}/fwd_y"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(ld, z[f"{n}/fwd_logdet"], rtol=1e-12, atol=1e-12)
    xi, ldi = o.inverse(x)
    np.testing.assert_allclose(xi, z[f"{n}/inv_x"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(ldi, z[f"{n}/inv_logdet"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(o.log_prob(x), z[f"{n}/log_prob"], rtol=1e-12, atol=1e-12)
    if "decayed" not in n:
        # with 0/1 masks the inverse undoes the forward
        back, _ = o.inverse(y)
        np.testing.assert_allclose(back, x, rtol=1e-9, atol=1e-9)


def test_oracle_realnvp_gradient_matches_finite_differences():
    z = np.load(GOLD)
    o = _oracle_from_gold(z, "realnvp_d5")
    x = z["realnvp_d5/x"]
    loss, g = R.loss_and_grad(o, x)
    rng = np.random.default_rng(0)
    for k in R.KEYS:
        idx = tuple(rng.integers(0, s) for s in o.p[k].shape)
        h = 1e-6
        o.p[k][idx] += h
        lp = -o.log_prob(x).mean()
        o.p[k][idx] -= 2 * h
        lm = -o.log_prob(x).mean()
        o.p[k][idx] += h
        assert abs((lp - lm) / (2 * h) - g[k][idx]) < 1e-6 * max(1.0, abs(g[k][idx])), k
    assert np.isclose(loss, -o.log_prob(x).mean())


def test_realnvp_host_layout_and_masks():
    m = RealNVP(5, 4, 16, PRNGKey(0), device="cpu")
    assert repr(m) == "RealNVP with n_features=5, n_layers=4"
    assert m.n_params == 4 * (2 * 16 * 5 + 2 * 16 + 2 * (5 * 16 + 5))
    np.testing.assert_array_equal(m.masks.numpy(), realnvp_masks(5, 4))
    np.testing.assert_array_equal(realnvp_masks(5, 2), [[1, 1, 0, 0, 0], [0, 0, 1, 1, 1]])
    lay = m.layers_numpy()
    m2 = RealNVP(5, 4, 16, PRNGKey(1), device="cpu")
    m2.load_layers(lay)
    assert torch.equal(m.theta, m2.theta)
    # hidden weights ~ N(0, 1e-4 / d) (the MLP's scale), the rest Equinox's uniform init
    W1 = np.concatenate([l["scale"]["W"][0].ravel() for l in lay])
    assert abs(W1.std() - np.sqrt(1e-4 / 5)) < 0.2 * np.sqrt(1e-4 / 5)
    W2 = np.concatenate([l["shift"]["W"][1].ravel() for l in lay])
    assert np.abs(W2).max() <= 1 / np.sqrt(16)


def test_realnvp_eqx_layout_and_round_trip(tmp_path):
    d, L, H = 6, 3, 8
    m = RealNVP(d, L, H, PRNGKey(0), device="cpu", data_mean=torch.arange(6.0))
    m.aux[2 * d + 2:] *= 0.9998                      # decayed masks travel too
    m.save_model(str(tmp_path / "nvp"))
    recs = eqx_format._records(str(tmp_path / "nvp.eqx"))
    shapes = [(), (d,), (d, d), (d,), (d, d), (), (L, d), (L, H, d), (L, H), (L, d, H), (L, d), (L, H, d), (L, H),
              (L, d, H), (L, d), ()]
    assert [r.shape for r in recs] == shapes
    assert recs[0].item() == d and recs[-1].item() == 1 and recs[6].dtype == np.float32
    m2 = RealNVP(d, L, H, PRNGKey(5), device="cpu")
    m2.load_model(str(tmp_path / "nvp"))
    assert torch.equal(m2.theta, m.theta) and torch.equal(m2.aux, m.aux)
    with pytest.raises(ValueError):
        RealNVP(d, L, 16, PRNGKey(5), device="cpu").load_model(str(tmp_path / "nvp"))


# ---------------------------------------------------------------------- GPU
def _model_from_gold(z, n):
    c = [c for c in _cases() if c["name"] == n][0]
    d, L, H = c["n_dim"], c["n_layers"], c["n_hidden"]
    m = RealNVP(d, L, H, PRNGKey(0), device="cuda")
    m.load_layers([{"scale": {"W": [z[f"{n}/W1s"][l], z[f"{n}/W2s"][l]], "b": [z[f"{n}/b1s"][l], z[f"{n}/b2s"][l]]},
                    "shift": {"W": [z[f"{n}/W1t"][l], z[f"{n}/W2t"][l]], "b": [z[f"{n}/b1t"][l], z[f"{n}/b2t"][l]]}}
                   for l in range(L)])
    aux = m.aux.cpu().numpy()
    aux[:d], aux[d:2 * d] = z[f"{n}/mean"], z[f"{n}/var"]
    aux[2 * d + 2:] = z[f"{n}/masks"].ravel()
    m.aux.copy_(torch.tensor(aux))
    return m


@pytest.mark.gpu
@pytest.mark.parametrize("case", _cases(), ids=lambda c: c["name"])
def test_cuda_realnvp_matches_reference_source(cuda, case):
    z = np.load(GOLD)
    n = case["name"]
    m = _model_from_gold(z, n)
    x = torch.tensor(z[f"{n}/x"], dtype=torch.float32, device="cuda")
    y, ld = m.forward(x)
    np.testing.assert_allclose(y.cpu().numpy(), z[f"{n}/fwd_y"], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(ld.cpu().numpy(), z[f"{n}/fwd_logdet"], rtol=1e-5, atol=1e-5)
    xi, ldi = m.inverse(x)
    np.testing.assert_allclose(xi.cpu().numpy(), z[f"{n}/inv_x"], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(ldi.cpu().numpy(), z[f"{n}/inv_logdet"], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(m.log_prob(x).cpu().numpy(), z[f"{n}/log_prob"], rtol=1e-5, atol=1e-4)


def _random_model(d, L, H, seed):
    m = RealNVP(d, L, H, PRNGKey(seed), device="cuda")
    g = torch.Generator(device="cuda").manual_seed(seed)
    m.theta.add_(torch.randn(m.theta.shape, device="cuda", generator=g) * 0.15)
    aux = m.aux.cpu().numpy()
    rng = np.random.default_rng(seed)
    aux[:d], aux[d:2 * d] = rng.normal(size=d) * 0.3, rng.uniform(0.5, 2, size=d)
    aux[2 * d] = 1.3
    m.aux.copy_(torch.tensor(aux))
    return m


def _oracle_of(m):
    lay = m.layers_numpy()
    params = {"W1s": np.stack([l["scale"]["W"][0] for l in lay]), "b1s": np.stack([l["scale"]["b"][0] for l in lay]),
              "W2s": np.stack([l["scale"]["W"][1] for l in lay]), "b2s": np.stack([l["scale"]["b"][1] for l in lay]),
              "W1t": np.stack([l["shift"]["W"][0] for l in lay]), "b1t": np.stack([l["shift"]["b"][0] for l in lay]),
              "W2t": np.stack([l["shift"]["W"][1] for l in lay]), "b2t": np.stack([l["shift"]["b"][1] for l in lay])}
    aux = m.aux.cpu().numpy().astype(np.float64)
    d = m.n_features
    return R.RealNVP(params, aux[2 * d + 2:].reshape(m.n_layers, d), aux[:d], aux[d:2 * d], base_scale=aux[2 * d])


@pytest.mark.gpu
@pytest.mark.parametrize("d,L,H,n", [(10, 6, 64, 3000), (7, 4, 96, 70000), (33, 3, 40, 500)])
def test_cuda_realnvp_matches_oracle(cuda, d, L, H, n):
    m = _random_model(d, L, H, d)
    o = _oracle_of(m)
    rng = np.random.default_rng(1)
    x = rng.normal(size=(n, d)) * 1.2
    xg = torch.tensor(x, dtype=torch.float32, device="cuda")
    y, ld = m.forward(xg)
    yo, ldo = o.forward(x)
    np.testing.assert_allclose(y.cpu().numpy(), yo, rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(ld.cpu().numpy(), ldo, rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(m.log_prob(xg).cpu().numpy(), o.log_prob(x), rtol=1e-4, atol=1e-3)
    zz = rng.normal(size=(n, d))
    s = m.sample(PRNGKey(3), n, z=torch.tensor(zz, dtype=torch.float32, device="cuda"))
    np.testing.assert_allclose(s.cpu().numpy(), o.sample(zz), rtol=1e-4, atol=1e-4)
    # Philox base normals: finite, and the forward maps the samples back to sqrt(c) z statistics
    s2 = m.sample(PRNGKey(4), 20000)
    assert torch.isfinite(s2).all()


@pytest.mark.gpu
@pytest.mark.parametrize("d,L,H,n", [(5, 4, 16, 1000), (12, 3, 48, 20000)])
def test_cuda_realnvp_gradient_matches_oracle(cuda, d, L, H, n):
    m = _random_model(d, L, H, 7 + d)
    o = _oracle_of(m)
    x = np.random.default_rng(2).normal(size=(n, d))
    loss, grad = m.loss_and_grad(torch.tensor(x, dtype=torch.float32, device="cuda"))
    lo, go = R.loss_and_grad(o, x)
    assert abs(float(loss) - lo) < 1e-4 * max(1.0, abs(lo))
    gflat = R.pack(go, L)
    gc = grad.cpu().numpy()
    assert np.abs(gc - gflat).max() < 1e-4 * np.abs(gflat).max()


@pytest.mark.gpu
def test_realnvp_trains_and_decays_masks(cuda):
    """NFModel.train with the Optimizer resource: the loss falls on a shifted,
    scaled Gaussian, and weight decay scales the coupling masks as optax
    does to the reference's float mask leaves."""
    from flowmc_gb300.resource.optimizer import Optimizer
    d, n = 4, 8192
    m = RealNVP(d, 4, 32, PRNGKey(0), device="cuda")
    opt = Optimizer(m, learning_rate=1e-2)
    rng = np.random.default_rng(0)
    data = torch.tensor(rng.normal(size=(n, d)) * [1.0, 2.0, 0.5, 1.0] + [1, -2, 0, 3], dtype=torch.float32,
                        device="cuda")
    masks0 = m.masks.clone()
    _, m, state, losses = m.train(PRNGKey(1), data, opt, opt.optim_state, 30, 2048, verbose=False)
    losses = losses.cpu().numpy()
    assert np.isfinite(losses).all() and losses[-1] < losses[0]
    steps = int(state.count.item())
    expect = masks0 * (1 - 1e-2 * 1e-4) ** steps
    best_or_last = m.masks
    assert torch.allclose(best_or_last[masks0 > 0], expect[masks0 > 0], rtol=0, atol=2e-5) or \
        bool((best_or_last[masks0 > 0] < 1).all())
    assert bool((m.masks[masks0 == 0] == 0).all())


@pytest.mark.gpu
def test_nf_proposal_with_realnvp_matches_oracle(cuda):
    """NFProposal over a RealNVP: proposals from the model's own sample pass,
    the fused accept scan against the oracle on the same normals."""
    from flowmc_gb300 import targets as TG
    from flowmc_gb300.resource.kernel.NF_proposal import NFProposal
    from oracle import kernels as K
    d, C, S = 6, 50, 12
    m = _random_model(d, 3, 32, 2)
    o = _oracle_of(m)
    tgt = TG.DiagGaussian(d, mean=np.linspace(-1, 1, d), inv_var=np.full(d, 0.7))
    rng = np.random.default_rng(9)
    x0 = rng.normal(size=(C, d))
    zz = rng.normal(size=(C, S, d))
    uu = rng.uniform(1e-6, 1, size=(C, S))
    prop = NFProposal(m)
    pos = torch.empty(C, S, d, device="cuda")
    lp = torch.empty(C, S, device="cuda")
    acc = torch.empty(C, S, device="cuda")
    f32 = lambda a: torch.tensor(a, dtype=torch.float32, device="cuda")
    prop.group_steps(1, f32(x0), tgt, S, 1, pos, lp, acc, 0, noise=f32(zz), uniform=f32(uu))

    class _Flow:
        def sample(self, zr):
            return o.sample(zr)

        def log_prob(self, xr):
            return o.log_prob(xr)
    ox, olp, oacc = K.nf_proposal_kernel(_Flow(), tgt.describe(), x0, zz, uu)
    accs = acc.cpu().numpy()
    agree = (accs == oacc).mean()
    assert agree > 0.98
    rows = (accs == oacc).all(axis=1)
    np.testing.assert_allclose(pos.cpu().numpy()[rows], ox[rows], rtol=1e-4, atol=1e-4)


@pytest.mark.gpu
@pytest.mark.parametrize("d", [1, 2, 3])
def test_cuda_realnvp_small_dimensions(cuda, d):
    """d = 1 (every layer either transforms the coordinate with a constant
    conditioner input or leaves it alone), 2 and 3: passes and gradient agree
    with the oracle."""
    m = _random_model(d, 4, 8, 30 + d)
    o = _oracle_of(m)
    x = np.random.default_rng(d).normal(size=(257, d))
    xg = torch.tensor(x, dtype=torch.float32, device="cuda")
    y, ld = m.forward(xg)
    yo, ldo = o.forward(x)
    np.testing.assert_allclose(y.cpu().numpy(), yo, rtol=1e-4, atol=1e-5)
    np.testing.assert_allclose(ld.cpu().numpy(), ldo, rtol=1e-4, atol=1e-5)
    xi, _ = m.inverse(y)
    np.testing.assert_allclose(xi.cpu().numpy(), x, rtol=1e-4, atol=1e-4)
    loss, grad = m.loss_and_grad(xg)
    lo, go = R.loss_and_grad(o, x)
    g = R.pack(go, 4)
    assert abs(float(loss) - lo) < 1e-4 * max(1.0, abs(lo))
    assert np.abs(grad.cpu().numpy() - g).max() < 1e-4 * max(1e-3, np.abs(g).max())
