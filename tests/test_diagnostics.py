"""The measurement code on the CPU: the ESS estimator, the moment error, the
quadrature moments the moment error is taken against, and the plain FP32
form's target gradients (the comparison arm of the bench)."""
import math

import numpy as np
import pytest
import torch

from flowmc_gb300 import diagnostics as D
from flowmc_gb300 import plain as PL
from oracle import targets as OT


def test_ess_iid_draws():
    g = torch.Generator().manual_seed(0)
    x = torch.randn(16, 2000, 3, generator=g, dtype=torch.float64)
    ess = D.ess_bulk(x)
    n = 16 * 2000
    assert torch.all(ess > 0.8 * n) and torch.all(ess < 1.25 * n)


def test_ess_ar1_draws():
    # AR(1) with coefficient rho has integrated autocorrelation time (1 + rho) / (1 - rho)
    rho = 0.9
    g = torch.Generator().manual_seed(1)
    e = torch.randn(16, 4000, 2, generator=g, dtype=torch.float64)
    x = torch.empty_like(e)
    x[:, 0] = e[:, 0] / math.sqrt(1 - rho * rho)
    for t in range(1, e.shape[1]):
        x[:, t] = rho * x[:, t - 1] + e[:, t]
    ess = D.ess_bulk(x)
    expect = 16 * 4000 * (1 - rho) / (1 + rho)
    assert torch.all(ess > 0.75 * expect) and torch.all(ess < 1.33 * expect)


def test_ess_stuck_chains():
    # chains that never mix between two locations: ESS far below the draw count
    g = torch.Generator().manual_seed(2)
    x = torch.randn(8, 1000, 1, generator=g, dtype=torch.float64) * 0.1
    x[:4] += 5.0
    assert float(D.ess_bulk(x)[0]) < 100


def test_moment_error():
    # six draws per coordinate; the variance is the unbiased one (6/5 here)
    x = torch.zeros(2, 3, 2, dtype=torch.float64)
    x[0, :, 0], x[1, :, 0] = 1.0, 3.0          # mean 2, variance 1.2
    x[0, :, 1], x[1, :, 1] = -1.0, 1.0         # mean 0, variance 1.2
    assert D.moment_error(x, [2.0, 0.0], [1.2, 1.2]) == pytest.approx(0.0, abs=1e-12)
    assert D.moment_error(x, [2.0, 0.6], [1.2, 1.2]) == pytest.approx(0.6 / 1.2 ** 0.5, abs=1e-12)
    assert D.moment_error(x, [2.0, 0.0], [1.2, 0.6]) == pytest.approx(1.0, abs=1e-12)


def test_rosenbrock_moments_two_dims():
    # d = 2: x0 ~ N(b, a/2) exactly (the pair factor integrates to a constant),
    # x1 | x0 ~ N(x0^2, 1/(2c))
    a, b, c = 20.0, 1.0, 5.0
    mean, var = D.rosenbrock_chain_moments(2, a, b, c, lo=-25.0, hi=27.0, m=8000)
    s2 = a / 2
    m2 = b * b + s2
    m4 = b ** 4 + 6 * b * b * s2 + 3 * s2 * s2
    assert mean[0] == pytest.approx(b, rel=1e-6)
    assert var[0] == pytest.approx(s2, rel=1e-6)
    assert mean[1] == pytest.approx(m2, rel=1e-6)
    assert var[1] == pytest.approx(m4 - m2 * m2 + 1 / (2 * c), rel=1e-6)


def test_dual_moon_moments_importance_sampling():
    """Quadrature against importance sampling with the radial shell as the
    proposal: x = r u, r ~ N(r0, sr), u uniform on the sphere."""
    d, r0, sr, mu, s0 = 5, 2.0, 0.1, 3.0, 0.6
    mean, var = D.dual_moon_moments(d, r0, sr, mu, s0, m_r=800, m_phi=1600)
    rng = np.random.default_rng(0)
    n = 400_000
    u = rng.normal(size=(n, d))
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    r = rng.normal(r0, sr, size=n)
    r = r[r > 0]
    x = r[:, None] * u[: r.size]
    lw = np.logaddexp(-0.5 * ((x[:, 0] + mu) / s0) ** 2, -0.5 * ((x[:, 0] - mu) / s0) ** 2) \
        + (d - 1) * np.log(r)
    w = np.exp(lw - lw.max())
    w /= w.sum()
    is_var = (w[:, None] * x ** 2).sum(0)
    assert np.all(mean == 0.0)
    assert var[0] == pytest.approx(is_var[0], rel=0.01)
    assert var[1:].mean() == pytest.approx(is_var[1:].mean(), rel=0.01)
    # the same integral on a finer grid
    _, var_f = D.dual_moon_moments(d, r0, sr, mu, s0, m_r=1600, m_phi=3200)
    np.testing.assert_allclose(var, var_f, rtol=1e-6)


@pytest.mark.parametrize("kind", ["dual_moon", "rosenbrock", "mixture"])
def test_plain_target_value_grad(kind):
    rng = np.random.default_rng(3)
    if kind == "dual_moon":
        t = {"kind": "dual_moon", "n_dim": 5, "r0": 2.0, "sr": 0.1, "mu": 3.0, "s0": 0.6}
        x = rng.normal(size=(9, 5)) * 1.5
        fn = PL.dual_moon_value_grad
    elif kind == "rosenbrock":
        t = {"kind": "rosenbrock", "n_dim": 7, "a": 20.0, "b": 1.0, "c": 5.0}
        x = rng.normal(size=(9, 7))
        fn = PL.rosenbrock_value_grad
    else:
        means = rng.normal(size=(4, 6)) * 3
        iv = rng.uniform(0.5, 2.0, size=(4, 6))
        lw = np.log(np.full(4, 0.25)) + 0.5 * np.log(iv / (2 * np.pi)).sum(1)
        t = {"kind": "mixture", "mean": means, "inv_var": iv, "log_w": lw}
        x = rng.normal(size=(9, 6)) * 3
        fn = lambda z: PL.mixture_value_grad(z, torch.tensor(means), torch.tensor(iv), torch.tensor(lw))
    v_ref, g_ref = OT.value_grad(t, x)
    v, g = fn(torch.tensor(x))
    np.testing.assert_allclose(v.numpy(), v_ref, rtol=1e-12, atol=1e-10)
    np.testing.assert_allclose(g.numpy(), g_ref, rtol=1e-12, atol=1e-10)


def test_streaming_oracle_matches_batch_definitions():
    """The streaming oracle (Welford per chain, merged) equals the plain
    float64 definitions on the same draws: mean and variance of all draws,
    R-hat from within/between-chain variances, and the variance of the
    complete batch means behind the batch-means ESS -- over updates whose
    sizes do not line up with the batches."""
    import numpy as np
    from oracle.streaming import StreamingOracle
    rng = np.random.default_rng(3)
    C, n, d, b = 7, 53, 4, 10
    x = rng.normal(size=(C, n, d)) * [1.0, 2.0, 0.5, 3.0] + [0.0, 1.0, -2.0, 5.0]
    so = StreamingOracle(C, d, b)
    for lo, hi in ((0, 3), (3, 17), (17, 40), (40, 53)):
        so.update(x[:, lo:hi])
    mu, var, ess, rhat = so.finalize()
    flat = x.reshape(-1, d)
    np.testing.assert_allclose(mu, flat.mean(0), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(var, flat.var(0, ddof=1), rtol=1e-12)
    W = x.var(1, ddof=1).mean(0)
    B_n = x.mean(1).var(0, ddof=1)
    np.testing.assert_allclose(rhat, np.sqrt(((n - 1) / n * W + B_n) / W), rtol=1e-12)
    k = n // b
    bm = x[:, :k * b].reshape(C, k, b, d).mean(2).reshape(-1, d)
    tau = b * bm.var(0, ddof=1) / flat.var(0, ddof=1)
    np.testing.assert_allclose(ess, np.minimum(C * n / tau, C * n), rtol=1e-10)


def test_streaming_oracle_ess_of_ar1():
    """Batch-means ESS of AR(1) chains x_t = rho x_{t-1} + e_t (integrated
    autocorrelation time (1 + rho) / (1 - rho)) within 15 % of N / tau with
    batches of 25 tau, and near N for independent draws."""
    import numpy as np
    from oracle.streaming import StreamingOracle
    rng = np.random.default_rng(11)
    C, n, d = 64, 4000, 2
    for rho in (0.0, 0.8):
        e = rng.normal(size=(C, n, d))
        x = np.empty_like(e)
        x[:, 0] = e[:, 0] / np.sqrt(1 - rho ** 2)
        for t in range(1, n):
            x[:, t] = rho * x[:, t - 1] + e[:, t]
        tau = (1 + rho) / (1 - rho)
        so = StreamingOracle(C, d, int(25 * tau))
        so.update(x)
        _, _, ess, rhat = so.finalize()
        assert np.all(np.abs(ess / (C * n / tau) - 1) < 0.15), (rho, ess, C * n / tau)
        assert np.all(np.abs(rhat - 1) < 0.01)
