"""Flow kernels (K3/K4/K6), optimiser, training-data selection and the NF
global step (K5) on the GPU against the oracle, through the C ABI.

Tolerances: FP32 flow log-probs within 1e-4 (relative to max(1, |logp|)),
forward/inverse outputs within 1e-4, gradients within 1e-4 of the largest
gradient entry (FP64 autograd oracle, itself pinned to central finite
differences in test_oracle.py), AdamW updates within 1e-6 relative.
"""
import numpy as np
import pytest
import torch

from oracle import flow as F
from oracle import flow_torch as FT
from oracle import kernels as K

pytestmark = pytest.mark.gpu


def rand_flow(d, L, hidden, nb, seed=0, wscale=0.4):
    rng = np.random.default_rng(seed)
    P = 3 * nb + 1
    layers = []
    for i in range(L):
        shape = [d, *hidden, d * P]
        Ws = [rng.normal(size=(b, a)) * wscale / np.sqrt(a) * 2 for a, b in zip(shape[:-1], shape[1:])]
        bs = [rng.normal(size=b) * 0.2 for b in shape[1:]]
        layers.append({"W": Ws, "b": bs, "scale": 0.05 * rng.normal(), "shift": 0.1 * rng.normal(),
                       "mask": ((np.arange(d) + i) % 2).astype(bool)})
    mean = rng.normal(size=d) * 0.3
    var = rng.uniform(0.5, 2.0, size=d)
    return F.Flow(layers, nb, mean, np.diag(var))


def to_f32(fl: F.Flow) -> F.Flow:
    """The oracle flow with float32-rounded parameters (what the GPU holds)."""
    g = F.clone(fl)
    for L in g.layers:
        L["W"] = [w.astype(np.float32).astype(np.float64) for w in L["W"]]
        L["b"] = [b.astype(np.float32).astype(np.float64) for b in L["b"]]
        L["scale"] = float(np.float32(L["scale"]))
        L["shift"] = float(np.float32(L["shift"]))
    g.data_mean = g.data_mean.astype(np.float32).astype(np.float64)
    g.data_cov = np.diag(np.diag(g.data_cov).astype(np.float32).astype(np.float64))
    return g


def gpu_model(fl: F.Flow, hidden, precision="float32"):
    from flowmc_gb300.random import PRNGKey
    from flowmc_gb300.resource.model.nf_model.rqSpline import MaskedCouplingRQSpline
    d = fl.d
    m = MaskedCouplingRQSpline(d, len(fl.layers), list(hidden), fl.n_bins, PRNGKey(0), precision=precision,
                               device="cuda")
    m.load_full(fl.layers)
    m.aux[:d] = torch.tensor(fl.data_mean, dtype=torch.float32)
    m.aux[d:2 * d] = torch.tensor(np.diag(fl.data_cov), dtype=torch.float32)
    m.aux[2 * d] = float(fl.base_cov_scale)
    m.check_layout()
    return m


CONFIGS = [(3, 2, (16, 16), 8), (5, 4, (32, 32), 8), (7, 3, (9, 11), 4), (32, 8, (128, 128), 10),
           (16, 2, (24,), 12), (6, 2, (8, 8, 8), 5)]


@pytest.mark.parametrize("d,L,hidden,nb", CONFIGS, ids=[f"d{c[0]}L{c[1]}K{c[3]}" for c in CONFIGS])
def test_flow_passes_match_oracle(cuda, d, L, hidden, nb):
    fl = to_f32(rand_flow(d, L, hidden, nb, seed=d * 100 + L))
    m = gpu_model(fl, hidden)
    rng = np.random.default_rng(1)
    x = (rng.normal(size=(300, d)) * 2.5).astype(np.float32)
    x[:5] *= 6.0                                    # some rows in the linear tails
    xt = torch.tensor(x, device="cuda")
    # forward (no standardisation)
    y, ld = m.forward(xt)
    oy, old = fl.forward(x.astype(np.float64))
    np.testing.assert_allclose(y.cpu().numpy(), oy, rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(ld.cpu().numpy(), old, rtol=1e-4, atol=1e-4 * max(1, np.abs(old).max()))
    # inverse (the reference's in-layer order)
    xi, ldi = m.inverse(xt)
    oxi, oldi = fl.inverse(x.astype(np.float64))
    np.testing.assert_allclose(xi.cpu().numpy(), oxi, rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(ldi.cpu().numpy(), oldi, rtol=1e-4, atol=1e-4 * max(1, np.abs(oldi).max()))
    # log_prob (data space)
    lp = m.log_prob(xt).cpu().numpy()
    olp = fl.log_prob(x.astype(np.float64))
    np.testing.assert_allclose(lp, olp, rtol=1e-4, atol=1e-4 * np.maximum(1, np.abs(olp)).max())
    # sample with explicit base normals
    z = rng.normal(size=(200, d)).astype(np.float32)
    s = m.sample(__import__("flowmc_gb300.random", fromlist=["PRNGKey"]).PRNGKey(3), 200,
                 z=torch.tensor(z, device="cuda")).cpu().numpy()
    np.testing.assert_allclose(s, fl.sample(z.astype(np.float64)), rtol=1e-4, atol=1e-4)


def test_flow_sample_philox_statistics(cuda):
    # an identity-like flow (zero last layer => standard spline is identity inside the range)
    from flowmc_gb300.random import PRNGKey
    fl = rand_flow(4, 2, (8, 8), 8, seed=1)
    for Lr in fl.layers:
        Lr["W"][-1][:] = 0
        Lr["b"][-1][:] = 0
        Lr["scale"] = 0.0
        Lr["shift"] = 0.0
    fl.data_mean = np.array([1.0, -2.0, 0.5, 0.0])
    fl.data_cov = np.diag([1.0, 4.0, 0.25, 1.0])
    m = gpu_model(fl, (8, 8))
    s = m.sample(PRNGKey(7), 200000).double()
    np.testing.assert_allclose(s.mean(0).cpu().numpy(), fl.data_mean, atol=0.02)
    np.testing.assert_allclose(s.var(0).cpu().numpy(), np.diag(fl.data_cov), rtol=0.02)


@pytest.mark.parametrize("d,L,hidden,nb", [(3, 2, (16, 16), 8), (5, 4, (32, 32), 8), (7, 3, (9, 11), 4),
                                           (32, 4, (128, 128), 10)])
def test_flow_gradient_matches_autograd(cuda, d, L, hidden, nb):
    fl = to_f32(rand_flow(d, L, hidden, nb, seed=7 + d))
    m = gpu_model(fl, hidden)
    x = (np.random.default_rng(4).normal(size=(257, d)) * 2).astype(np.float32)
    loss, grad = m.loss_and_grad(torch.tensor(x, device="cuda"))
    oloss, ograd_full = FT.loss_and_grad(fl, x.astype(np.float64))
    assert abs(loss.item() - oloss) <= 1e-4 * max(1, abs(oloss))
    # map the oracle's full-layout gradient into the packed layout
    gpu_full = gpu_grad_to_full(m, grad)
    scale = np.abs(ograd_full).max()
    np.testing.assert_allclose(gpu_full, ograd_full, atol=1e-4 * scale, rtol=0)


def gpu_grad_to_full(m, grad):
    """Packed GPU gradient -> the oracle's full flat layout (zeros where unused)."""
    saved = m.theta.clone()
    m.theta.copy_(grad)
    dec = m.aux[2 * m.n_features + 1].item()
    m.aux[2 * m.n_features + 1] = 0.0      # packed-out entries -> 0
    full = m.to_full()
    m.theta.copy_(saved)
    m.aux[2 * m.n_features + 1] = dec
    tmp = F.Flow([dict(Lr, mask=((np.arange(m.n_features) + i) % 2).astype(bool)) for i, Lr in enumerate(full)],
                 m.num_bins, np.zeros(m.n_features), np.eye(m.n_features))
    return F.flatten(tmp)


def test_adamw_step_matches_oracle(cuda):
    from flowmc_gb300.resource.optimizer import Optimizer
    fl = to_f32(rand_flow(5, 2, (8, 8), 4, seed=3))
    m = gpu_model(fl, (8, 8))
    opt = Optimizer(m, learning_rate=1e-2)
    st = opt.optim_state
    rng = np.random.default_rng(0)
    p = m.theta.double().cpu().numpy()
    ost = F.AdamWState(np.zeros(p.size), np.zeros(p.size))
    aux0 = m.aux.double().cpu().numpy()
    for k in range(5):
        g = rng.normal(size=p.size) * (0.01 if k % 2 else 1.0)   # clipped and unclipped steps
        gt = torch.tensor(g, dtype=torch.float32, device="cuda")
        opt.apply(m, gt, st)
        p, decay = F.adamw_update(p, g.astype(np.float32).astype(np.float64), ost, lr=1e-2)
    np.testing.assert_allclose(m.theta.double().cpu().numpy(), p, rtol=2e-5, atol=1e-6)
    np.testing.assert_allclose(m.aux.double().cpu().numpy(), aux0 * (1 - 1e-2 * 1e-4) ** 5, rtol=1e-6)
    assert int(st.count.item()) == 5


def test_select_training_data_matches_oracle(cuda):
    from flowmc_gb300.strategy.train_model import TrainModel
    rng = np.random.default_rng(0)
    C, S, d = 6, 40, 3
    buf = np.full((C, S, d), -np.inf, np.float32)
    buf[:, :25] = rng.normal(size=(C, 25, d))
    tm = TrainModel("model", "data", "opt", n_max_examples=500, history_window=10)
    idx = rng.integers(0, C * 10, size=500)
    out = tm.select(0, torch.tensor(buf, device="cuda"), torch.tensor(idx, device="cuda"))
    np.testing.assert_array_equal(out.cpu().numpy(), F.select_training_data(buf, 10, idx).astype(np.float32))
    # Philox draws: every selected row comes from the window
    out2 = tm.select(5, torch.tensor(buf, device="cuda")).cpu().numpy()
    window = buf[:, 15:25].reshape(-1, d)
    assert all((np.abs(window - r).sum(1) == 0).any() for r in out2[:50])
    tm.check_errors()
    # uneven finite rows -> error flag, like the reference's reshape
    buf[0, 3] = np.nan
    tm.select(1, torch.tensor(buf, device="cuda"))
    with pytest.raises(ValueError):
        tm.check_errors()


def test_nf_global_step_matches_oracle(cuda):
    from flowmc_gb300 import targets as TG
    from flowmc_gb300.resource.kernel.NF_proposal import NFProposal
    d = 5
    fl = to_f32(rand_flow(d, 3, (16, 16), 8, seed=11, wscale=0.2))
    m = gpu_model(fl, (16, 16))
    tgt = TG.DualMoon(d)
    C, S = 7, 13
    rng = np.random.default_rng(2)
    x0 = rng.normal(size=(C, d)).astype(np.float32)
    z = rng.normal(size=(C, S, d)).astype(np.float32)
    u = rng.uniform(1e-6, 1, size=(C, S)).astype(np.float32)
    dev = "cuda"
    pos = torch.full((C, S + 4, d), -np.inf, device=dev)
    lp = torch.full((C, S + 4), -np.inf, device=dev)
    acc = torch.full((C, S + 4), -np.inf, device=dev)
    prop = NFProposal(m)
    xl = prop.group_steps(9, torch.tensor(x0, device=dev), tgt, S, 1, pos, lp, acc, 2,
                          noise=torch.tensor(z, device=dev), uniform=torch.tensor(u, device=dev))
    ox, olp, oacc = K.nf_proposal_kernel(fl, tgt.describe(), x0.astype(np.float64), z.astype(np.float64),
                                         u.astype(np.float64))
    # accept decisions identical away from ties (the flow densities enter the ratio)
    np.testing.assert_array_equal(acc[:, 2:2 + S].cpu().numpy(), oacc)
    np.testing.assert_allclose(pos[:, 2:2 + S].cpu().numpy(), ox, rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(lp[:, 2:2 + S].cpu().numpy(), olp, rtol=1e-4, atol=1e-3)
    np.testing.assert_allclose(xl.cpu().numpy(), ox[:, -1], rtol=1e-4, atol=1e-4)
    assert np.isinf(pos[:, :2].cpu().numpy()).all()


def test_training_reduces_loss_and_keeps_best(cuda):
    from flowmc_gb300.random import PRNGKey
    from flowmc_gb300.resource.model.nf_model.rqSpline import MaskedCouplingRQSpline
    from flowmc_gb300.resource.optimizer import Optimizer
    rng = np.random.default_rng(0)
    # bimodal data: standardisation alone cannot fit it, the splines must
    lab = rng.integers(0, 2, size=4000)
    raw = rng.normal(size=(4000, 2)) * 0.3 + np.stack([np.where(lab, 2.0, -2.0), np.zeros(4000)], 1)
    data = torch.tensor(raw + [1.0, -1.0], dtype=torch.float32, device="cuda")
    m = MaskedCouplingRQSpline(2, 4, [32, 32], 4, PRNGKey(10), device="cuda")
    opt = Optimizer(m, learning_rate=3e-3)
    _, m, st, losses = m.train(PRNGKey(1), data, opt, opt.optim_state, 30, 500, verbose=False)
    losses = losses.cpu().numpy()
    assert losses[-1] < losses[0] - 0.3, losses
    best = losses.min()
    lp = m.log_prob(data)
    # the restored model is the best epoch's (its loss is the last step's loss of that epoch)
    assert abs(-lp.mean().item() - best) < 0.2
    np.testing.assert_allclose(m.data_mean.cpu().numpy(), raw.mean(0) + [1.0, -1.0], atol=1e-3)


def test_train_step_matches_oracle_sequence(cuda):
    """Two epochs of NFModel.train with the same batches: GPU vs oracle."""
    from flowmc_gb300.random import PRNGKey
    from flowmc_gb300.resource.optimizer import Optimizer
    d = 3
    fl = to_f32(rand_flow(d, 2, (8, 8), 4, seed=21))
    m = gpu_model(fl, (8, 8))
    opt = Optimizer(m, learning_rate=1e-2)
    data = np.random.default_rng(1).normal(size=(64, d)).astype(np.float32)
    # full-batch steps (batch_size > N) so no permutation is involved (base.py:148-149)
    _, m, st, losses = m.train(PRNGKey(0), torch.tensor(data, device="cuda"), opt, opt.optim_state, 4, 128,
                               verbose=False)
    ost = F.AdamWState(np.zeros(F.flatten(fl).size), np.zeros(F.flatten(fl).size))
    best, _, olosses = F.train(fl, data.astype(np.float64), FT.loss_and_grad, ost, 4, 128, 1e-2)
    np.testing.assert_allclose(losses.cpu().numpy(), olosses, rtol=1e-4, atol=1e-4)
    np.testing.assert_allclose(gpu_grad_to_full_params(m), F.flatten(best), rtol=1e-3, atol=1e-5)
    np.testing.assert_allclose(m.data_mean.cpu().numpy(), best.data_mean, rtol=1e-5, atol=1e-6)


def gpu_grad_to_full_params(m):
    full = m.to_full()
    tmp = F.Flow([dict(Lr, mask=((np.arange(m.n_features) + i) % 2).astype(bool)) for i, Lr in enumerate(full)],
                 m.num_bins, np.zeros(m.n_features), np.eye(m.n_features))
    return F.flatten(tmp)


# (700, 2, ...): 350 transformed coordinates, more bias rows than the fused
# spline kernel stages in shared memory (its global-load path)
BF16_CONFIGS = [(32, 4, (128, 128), 10), (128, 2, (512, 512), 12), (5, 2, (32, 32), 8), (64, 3, (256, 256), 8),
                (700, 2, (64, 64), 12)]


@pytest.mark.parametrize("d,L,hidden,nb", BF16_CONFIGS, ids=[f"d{c[0]}L{c[1]}K{c[3]}" for c in BF16_CONFIGS])
def test_flow_bf16_conditioner_matches_oracle(cuda, d, L, hidden, nb):
    """BF16 conditioner GEMMs (tcgen05) with FP32 spline: log-probs within 2e-2."""
    from flowmc_gb300 import _lib
    fl = to_f32(rand_flow(d, L, hidden, nb, seed=d + L, wscale=0.3))
    m = gpu_model(fl, hidden, precision="bf16")
    rng = np.random.default_rng(2)
    x = (rng.normal(size=(1000, d)) * 1.5).astype(np.float32)
    xt = torch.tensor(x, device="cuda")
    lp = m.log_prob(xt).cpu().numpy()
    olp = fl.log_prob(x.astype(np.float64))
    assert _lib.device_error() == 0
    err = np.abs(lp - olp) / np.maximum(1.0, np.abs(olp))
    assert err.max() <= 2e-2, err.max()
    y, ld = m.forward(xt)
    oy, old = fl.forward(x.astype(np.float64))
    assert np.abs(y.cpu().numpy() - oy).max() <= 2e-2 * max(1, np.abs(oy).max())
    z = rng.normal(size=(500, d)).astype(np.float32)
    from flowmc_gb300.random import PRNGKey
    s = m.sample(PRNGKey(1), 500, z=torch.tensor(z, device="cuda")).cpu().numpy()
    os_ = fl.sample(z.astype(np.float64))
    assert np.abs(s - os_).max() <= 2e-2 * max(1, np.abs(os_).max())


@pytest.mark.parametrize("d,L,hidden,nb,xs", [(32, 3, (128, 128), 10, 1.5), (128, 2, (512, 512), 12, 1.5),
                                               (7, 3, (40, 24), 4, 1.5), (16, 2, (64, 64), 6, 8.0)])
def test_flow_bf16_gradient_tracks_autograd(cuda, d, L, hidden, nb, xs):
    """BF16 tensor-core training gradient: BF16 rounding of activations and
    adjoints bounds the error to a few 1e-2 of the largest entry; direction
    within 0.999 cosine of the FP64 autograd gradient. xs = 8 puts many
    inputs in the spline's linear tails."""
    from flowmc_gb300 import _lib
    fl = to_f32(rand_flow(d, L, hidden, nb, seed=5 + d, wscale=0.3))
    m = gpu_model(fl, hidden, precision="bf16")
    x = (np.random.default_rng(4).normal(size=(1000, d)) * xs).astype(np.float32)
    loss, grad = m.loss_and_grad(torch.tensor(x, device="cuda"))
    assert _lib.device_error() == 0
    oloss, og = FT.loss_and_grad(fl, x.astype(np.float64))
    assert abs(loss.item() - oloss) <= 2e-2 * max(1, abs(oloss))
    gg = gpu_grad_to_full(m, grad)
    cos = float(gg @ og / (np.linalg.norm(gg) * np.linalg.norm(og)))
    assert cos > 0.999, cos
    assert np.abs(gg - og).max() <= 5e-2 * np.abs(og).max()


@pytest.mark.parametrize("n", [40, 64, 200])
def test_flow_bf16_gradient_small_batches(cuda, n):
    """BF16 training gradient at batch sizes below and around one 64-row
    K block of the weight-gradient GEMMs (their MN-major operand maps cover
    64 rows, the rows past the batch held at zero), after a larger batch has
    left other values in the workspace rows past n."""
    from flowmc_gb300 import _lib
    d, L, hidden, nb = 16, 2, (64, 64), 6
    fl = to_f32(rand_flow(d, L, hidden, nb, seed=31, wscale=0.3))
    m = gpu_model(fl, hidden, precision="bf16")
    rng = np.random.default_rng(8)
    big = (rng.normal(size=(1000, d)) * 1.5).astype(np.float32)
    m.loss_and_grad(torch.tensor(big, device="cuda"))
    x = (rng.normal(size=(n, d)) * 1.5).astype(np.float32)
    loss, grad = m.loss_and_grad(torch.tensor(x, device="cuda"))
    assert _lib.device_error() == 0
    oloss, og = FT.loss_and_grad(fl, x.astype(np.float64))
    assert abs(loss.item() - oloss) <= 2e-2 * max(1, abs(oloss))
    gg = gpu_grad_to_full(m, grad)
    cos = float(gg @ og / (np.linalg.norm(gg) * np.linalg.norm(og)))
    assert cos > 0.999, cos


def test_training_bf16_reduces_loss(cuda):
    from flowmc_gb300.random import PRNGKey
    from flowmc_gb300.resource.model.nf_model.rqSpline import MaskedCouplingRQSpline
    from flowmc_gb300.resource.optimizer import Optimizer
    rng = np.random.default_rng(0)
    lab = rng.integers(0, 2, size=8192)
    raw = rng.normal(size=(8192, 8)) * 0.3
    raw[:, 0] += np.where(lab, 2.0, -2.0)
    data = torch.tensor(raw, dtype=torch.float32, device="cuda")
    m = MaskedCouplingRQSpline(8, 4, [64, 64], 8, PRNGKey(10), precision="bf16", device="cuda")
    opt = Optimizer(m, learning_rate=3e-3)
    _, m, st, losses = m.train(PRNGKey(1), data, opt, opt.optim_state, 25, 1024, verbose=False)
    losses = losses.cpu().numpy()
    assert np.isfinite(losses).all()
    assert losses[-1] < losses[0] - 0.3, losses


@pytest.mark.parametrize("n,d", [(2, 1), (1000, 7), (300000, 128), (5000, 1500)])
def test_column_stats_matches_numpy(cuda, n, d):
    """fmc_column_stats (data standardisation before training, nf_model/base.py:
    data mean and variance): two-stage block merge against float64 numpy,
    on columns with a large offset and a small spread."""
    from flowmc_gb300 import _lib
    rng = np.random.default_rng(n + d)
    x = (rng.normal(size=(n, d)) * rng.uniform(1e-2, 3.0, size=d) + rng.uniform(-100, 100, size=d)).astype(np.float32)
    xt = torch.tensor(x, device="cuda")
    mean = torch.empty(d, device="cuda")
    var = torch.empty(d, device="cuda")
    _lib.column_stats(xt, mean, var, _lib.Workspace())
    x64 = x.astype(np.float64)
    np.testing.assert_allclose(mean.cpu().numpy(), x64.mean(0), rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(var.cpu().numpy(), x64.var(0, ddof=1), rtol=2e-4, atol=1e-6)


@pytest.mark.parametrize("d,L,hidden,nb", [(128, 2, (512, 512), 12), (64, 2, (256, 256), 8), (6, 2, (64, 64), 3)],
                         ids=["d128K12", "d64K8", "d6K3"])
def test_spline_cta_pair_tiles_match_single_cta(cuda, d, L, hidden, nb):
    """The fused last Linear + spline on CTA pairs (tcgen05 cta_group::2,
    256-row tiles, half the group's weights per CTA) against one-CTA 128-row
    tiles: the same products in the same K order, so forward and inverse
    outputs agree to float32 rounding (1e-6 relative), at row counts that
    leave the last pair's second CTA partly or wholly past the end. The
    one-CTA kernel adds its log-det partials per coordinate group before the
    row reduction (the pair kernel leaves one partial per warp), so log_prob
    and the log-determinants agree to a summation-order bound, 1e-5."""
    fl = to_f32(rand_flow(d, L, hidden, nb, seed=d + 3 * L, wscale=0.3))
    m = gpu_model(fl, hidden, precision="bf16")
    rng = np.random.default_rng(5)
    for n in (50, 128, 300, 1000, 70000):
        x = torch.tensor((rng.normal(size=(n, d)) * 1.5).astype(np.float32), device="cuda")
        outs = {}
        for tile in (128, 256):
            m.tile_rows = tile
            y, ld = m.forward(x)
            xi, ldi = m.inverse(x)
            outs[tile] = [m.log_prob(x), y, ld, xi, ldi]
        from flowmc_gb300 import _lib
        assert _lib.device_error() == 0
        for k, (a, b) in enumerate(zip(outs[128], outs[256])):
            tol = 1e-6 if k in (1, 3) else 1e-5   # outputs / log-densities and log-dets
            torch.testing.assert_close(b, a, rtol=tol, atol=tol)
    m.tile_rows = 0
