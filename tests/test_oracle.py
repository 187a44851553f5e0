"""The oracle against the reference's own known-answer pins (CPU only).

The reference tests hold no numeric golden vectors; these are its
behavioural pins, restated for the oracle:
  * acceptance -> 1 at tiny steps   test/unit/test_kernels.py:111-133, 221-239, 324-342
  * N(0, I) moments within 3e-2     test_kernels.py:135-184, 241-288, 344-392
  * leapfrog reversibility          test_kernels.py:63-109
  * determinism                     test_kernels.py:37-61, 199-219, 303-322
  * flow shapes                     test/unit/test_nf.py:55-73
plus analytic checks: target gradients vs finite differences, the flow
gradient (autograd) vs central finite differences, spline round trips.
"""
import numpy as np
import pytest

from oracle import flow as F
from oracle import kernels as K
from oracle import targets as T

STD2 = {"kind": "diag_gaussian", "mean": np.zeros(2), "inv_var": np.ones(2), "const": 0.0}


def _fd_grad(t, x, h=1e-6):
    g = np.zeros_like(x)
    for j in range(x.shape[1]):
        e = np.zeros_like(x)
        e[:, j] = h
        g[:, j] = (T.value(t, x + e) - T.value(t, x - e)) / (2 * h)
    return g


ALL_TARGETS = [
    STD2,
    {"kind": "dual_moon", "n_dim": 5, "r0": 2.0, "sr": 0.1, "mu": 3.0, "s0": 0.6},
    {"kind": "mixture", "mean": np.random.default_rng(0).normal(size=(4, 6)),
     "inv_var": np.random.default_rng(1).uniform(0.5, 2.0, size=(4, 6)), "log_w": np.log(np.full(4, 0.25))},
    {"kind": "rosenbrock", "n_dim": 7, "a": 20.0, "b": 1.0, "c": 5.0},
    {"kind": "dense_gaussian", "mean": np.arange(3.0), "precision": np.array([[2., .3, 0], [.3, 1., .2], [0, .2, .5]]),
     "const": 0.0},
]


@pytest.mark.parametrize("t", ALL_TARGETS, ids=lambda t: t["kind"])
def test_target_gradients_match_finite_differences(t):
    rng = np.random.default_rng(3)
    x = rng.normal(size=(5, T.n_dim(t))) * 0.7 + 0.3
    _, g = T.value_grad(t, x)
    np.testing.assert_allclose(g, _fd_grad(t, x), rtol=1e-6, atol=1e-6)


@pytest.mark.parametrize("kind,step", [("mala", 1e-5), ("hmc", 1e-7), ("grw", 1e-5)])
def test_acceptance_goes_to_one(kind, step):
    rng = np.random.default_rng(42)
    x = rng.normal(size=(100, 2))
    pos, lp, acc, _ = K.take_serial_steps(kind, STD2, x, 1, rng.normal(size=(100, 1, 2)),
                                          rng.uniform(size=(100, 1)), step_size=step, n_leapfrog=5)
    assert acc.all()


@pytest.mark.parametrize("kind,step,n", [("mala", 1.0, 20000), ("hmc", 0.1, 10000), ("grw", 1.0, 20000)])
def test_moments_standard_normal(kind, step, n):
    # the reference runs one chain for 30-50k steps; 8 chains x n steps here
    rng = np.random.default_rng(7)
    C = 8
    x0 = rng.normal(size=(C, 2))
    pos, _, _, _ = K.take_serial_steps(kind, STD2, x0, n, rng.normal(size=(C, n, 2)), rng.uniform(size=(C, n)),
                                       step_size=step, n_leapfrog=5)
    assert abs(pos.mean()) < 3e-2
    assert abs(pos.var() - 1) < 3e-2


def test_leapfrog_reversible():
    rng = np.random.default_rng(42)
    x = rng.normal(size=(1, 2))
    p = rng.normal(size=(1, 2))
    x1, p1 = K.leapfrog(STD2, x, p, 1.0, 5, np.eye(2))
    x2, _ = K.leapfrog(STD2, x1, -p1, 1.0, 5, np.eye(2))
    np.testing.assert_allclose(x2, x, atol=1e-8)
    np.testing.assert_allclose(T.value(STD2, x2), T.value(STD2, x), atol=1e-8)


def test_leapfrog_table_matches_reference_layout():
    c = K.leapfrog_coefs(5)
    assert c.shape == (7, 2)
    assert list(c[0]) == [0, 0.5] and list(c[-1]) == [1, 0.5] and (c[1:-1] == 1).all()


def test_thinning_and_last_position():
    rng = np.random.default_rng(0)
    C, S = 3, 10
    pos, lp, acc, last = K.take_serial_steps("mala", STD2, rng.normal(size=(C, 2)), S, rng.normal(size=(C, S, 2)),
                                             rng.uniform(size=(C, S)), step_size=0.5, thinning=4)
    assert pos.shape == (C, 3, 2)                       # ceil(10 / 4)
    full, _, _, _ = K.take_serial_steps("mala", STD2, rng.normal(size=(C, 2)) * 0, 1, np.zeros((C, 1, 2)),
                                        np.ones((C, 1)), step_size=0.5)
    np.testing.assert_array_equal(last, pos[:, -1])


def test_buffer_update_clamps_start():
    buf = np.full((2, 5), -np.inf)
    out = K.buffer_update(buf, np.ones((2, 3)), 4, axis=1)   # clamped to start 2
    assert np.isinf(out[:, :2]).all() and (out[:, 2:] == 1).all()


# ----------------------------------------------------------------- flow
def make_flow(d=3, L=2, hidden=(16, 16), K=8, seed=10, scale_shift=True):
    rng = np.random.default_rng(seed)
    P = 3 * K + 1
    layers = []
    for i in range(L):
        shape = [d, *hidden, d * P]
        Ws, bs = [], []
        for a, b in zip(shape[:-1], shape[1:]):
            Ws.append(rng.normal(size=(b, a)) * 0.3)
            bs.append(rng.normal(size=b) * 0.1)
        layers.append({"W": Ws, "b": bs, "scale": 0.1 * (i + 1) if scale_shift else 0.0,
                       "shift": -0.2 * i if scale_shift else 0.0,
                       "mask": ((np.arange(d) + i) % 2).astype(bool)})
    return F.Flow(layers, K, rng.normal(size=d) * 0.1, np.diag(rng.uniform(0.5, 2, size=d)))


def test_flow_shapes():
    fl = make_flow()
    z = np.random.default_rng(0).normal(size=(2, 3))
    s = fl.sample(z)
    assert s.shape == (2, 3)
    assert fl.log_prob(s).shape == (2,)


def test_spline_roundtrip_and_logdet():
    rng = np.random.default_rng(5)
    raw = rng.normal(size=(200, 25))
    xp, yp, sl = F.spline_params(raw, 8)
    x = rng.uniform(-12, 12, size=200)
    y, ld = F.rqs_forward(x, xp, yp, sl)
    x2, ld2 = F.rqs_inverse(y, xp, yp, sl)
    np.testing.assert_allclose(x2, x, atol=1e-9)
    np.testing.assert_allclose(ld2, -ld, atol=1e-9)
    h = 1e-6
    fd = (F.rqs_forward(x + h, xp, yp, sl)[0] - F.rqs_forward(x - h, xp, yp, sl)[0]) / (2 * h)
    np.testing.assert_allclose(np.log(fd), ld, atol=1e-6)


def test_flow_inverse_is_exact_without_affine():
    # with ScalarAffine at its initial (0, 0) the in-layer order does not matter
    fl = make_flow(scale_shift=False)
    x = np.random.default_rng(1).normal(size=(50, 3))
    y, ld = fl.forward(x)
    x2, ld2 = fl.inverse(y)
    np.testing.assert_allclose(x2, x, atol=1e-9)
    np.testing.assert_allclose(ld2, -ld, atol=1e-9)


def test_flow_inverse_order_quirk():
    # rqSpline.py:470-488 applies ScalarAffine.inverse before the spline inverse
    # inside each layer, so inverse(forward(x)) != x once scale/shift != 0
    fl = make_flow(scale_shift=True)
    x = np.random.default_rng(1).normal(size=(50, 3))
    y, _ = fl.forward(x)
    x2, _ = fl.inverse(y)
    assert np.abs(x2 - x).max() > 1e-3


def test_flow_gradient_autograd_vs_finite_differences():
    from oracle import flow_torch as FT
    fl = make_flow(d=3, L=2, hidden=(5, 4), K=4)
    x = np.random.default_rng(2).normal(size=(16, 3))
    loss, g = FT.loss_and_grad(fl, x)
    assert abs(loss - F.loss(fl, x)) < 1e-12
    p0 = F.flatten(fl)
    rng = np.random.default_rng(0)
    idx = rng.choice(p0.size, size=40, replace=False)
    h = 1e-6
    for i in idx:
        f2 = F.clone(fl)
        p = p0.copy()
        p[i] += h
        F.unflatten(f2, p)
        lp = F.loss(f2, x)
        p[i] -= 2 * h
        F.unflatten(f2, p)
        lm = F.loss(f2, x)
        fd = (lp - lm) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_adamw_matches_definition():
    p = np.array([1.0, -2.0, 0.5])
    g = np.array([0.1, 0.2, -0.3])
    st = F.AdamWState(np.zeros(3), np.zeros(3))
    p1, decay = F.adamw_update(p, g, st, lr=1e-3)
    # first step: mhat = g, vhat = g^2 -> update = sign(g) (up to eps)
    expect = p - 1e-3 * (g / (np.abs(g) + 1e-8) + 1e-4 * p)
    np.testing.assert_allclose(p1, expect, rtol=1e-12)
    assert decay == 1 - 1e-7
    # clipping: a large gradient is rescaled to norm 1 before the moments
    st2 = F.AdamWState(np.zeros(3), np.zeros(3))
    F.adamw_update(p, g * 100, st2, lr=1e-3)
    np.testing.assert_allclose(st2.m, 0.1 * g * 100 / np.linalg.norm(g * 100), rtol=1e-12)


def test_select_training_data():
    rng = np.random.default_rng(0)
    buf = np.full((3, 6, 2), -np.inf)
    buf[:, :4] = rng.normal(size=(3, 4, 2))
    sel = F.select_training_data(buf, 2, np.array([0, 5, 3]))
    flat = buf[:, 2:4].reshape(-1, 2)
    np.testing.assert_array_equal(sel, flat[[0, 5, 3]])
