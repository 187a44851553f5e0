"""K1 (fused local steps) on the GPU against the oracle, through the C ABI.

Parity: the same explicit normals and uniforms go to both sides; positions
and log-densities must agree within 1e-5 relative (atol 1e-5 for values near
zero) and accept decisions must be identical except at ties, i.e. where the
oracle's |log u - log_ratio| < 1e-4 (the FP32 kernel and the FP64 oracle can
then legitimately disagree). After a tie-flip the trajectories diverge, so
comparison stops at the first tie of a chain.
"""
import zlib

import numpy as np
import pytest
import torch

from oracle import kernels as K
from oracle import targets as T

pytestmark = pytest.mark.gpu

RTOL = 1e-5
ATOL = 1e-5


def make_targets():
    from flowmc_gb300 import targets as TG
    rng = np.random.default_rng(11)
    Q, _ = np.linalg.qr(rng.normal(size=(6, 6)))
    P = Q @ np.diag(rng.uniform(0.5, 2.0, 6)) @ Q.T
    return {
        "diag": TG.DiagGaussian(3, mean=[0.5, -1.0, 0.0], inv_var=[1.0, 2.0, 0.5]),
        "std2": TG.DiagGaussian(2),
        "dual_moon": TG.DualMoon(5),
        "mixture": TG.GaussianMixture(rng.normal(size=(4, 9)) * 2, 0.5),
        "rosenbrock": TG.Rosenbrock(12),
        "rosenbrock128": TG.Rosenbrock(128),
        "dense": TG.DenseGaussian(P, mean=rng.normal(size=6)),
        "mixture64": TG.GaussianMixture(rng.normal(size=(4, 64)), 0.5),
        # d % 4 == 0 with d < lanes x coordinates: the shared-memory tables are read as
        # float4 and the last lane's chunks straddle the end of the row
        "mixture20": TG.GaussianMixture(rng.normal(size=(3, 20)), rng.uniform(0.3, 1.0, size=(3, 20))),
        "diag20": TG.DiagGaussian(20, mean=rng.normal(size=20), inv_var=rng.uniform(0.5, 2.0, size=20)),
        # default chain blocks whose last lane straddles d: d = 18 with 8 lanes x 4
        # (float2 row stores) and d = 132 with 32 lanes x 8 (float4 row stores)
        "diag18": TG.DiagGaussian(18, mean=rng.normal(size=18), inv_var=rng.uniform(0.5, 2.0, size=18)),
        "mixture132": TG.GaussianMixture(rng.normal(size=(2, 132)), 0.7),
    }


@pytest.fixture(scope="module")
def tgts(cuda):
    return make_targets()


def _run_gpu(kernel, tgt, x0, noise, unif, n_steps, thinning=1, cursor=0, buf_len=None, lanes=0):
    from flowmc_gb300.resource.kernel.base import run_local_steps
    C, d = x0.shape
    R = -(-n_steps // thinning)
    buf_len = buf_len or R
    dev = torch.device("cuda")
    kernel.lanes_per_chain = lanes
    pos = torch.full((C, buf_len, d), -np.inf, device=dev)
    lp = torch.full((C, buf_len), -np.inf, device=dev)
    acc = torch.full((C, buf_len), -np.inf, device=dev)
    xl, ll = run_local_steps(kernel, tgt, torch.tensor(x0, dtype=torch.float32, device=dev), n_steps, thinning,
                             1234, 0, pos, lp, acc, cursor,
                             noise=torch.tensor(noise, dtype=torch.float32, device=dev),
                             uniform=torch.tensor(unif, dtype=torch.float32, device=dev))
    torch.cuda.synchronize()
    return pos.cpu().numpy(), lp.cpu().numpy(), acc.cpu().numpy(), xl.cpu().numpy(), ll.cpu().numpy()


def _oracle_ratios(kind, t, x0, noise, unif, n_steps, step, n_leapfrog):
    """Per-step |log u - log_ratio| margins of the oracle (for tie detection)."""
    x = x0.astype(np.float64)
    lp = T.value(t, x)
    margins = np.zeros((x.shape[0], n_steps))
    for s in range(n_steps):
        xi, u = noise[:, s].astype(np.float64), unif[:, s].astype(np.float64)
        if kind == "mala":
            dt2 = step * step
            lp0, g0 = T.value_grad(t, x)
            prop = x + dt2 * g0 / 2 + step * xi
            lp1, g1 = T.value_grad(t, prop)
            r = lp1 - lp0 + (np.sum((prop - x - dt2 * g0 / 2) ** 2, -1) - np.sum((x - prop - dt2 * g1 / 2) ** 2, -1)) / (2 * dt2)
            x2, lp2, _ = K.mala_kernel(t, x, step, xi, u)
        elif kind == "hmc":
            xq, pq = K.leapfrog(t, x, xi, step, n_leapfrog, np.eye(x.shape[1]))
            lpq = T.value(t, xq)
            r = (-lp + 0.5 * np.sum(xi * xi, -1)) - (-lpq + 0.5 * np.sum(pq * pq, -1))
            x2, lp2, _ = K.hmc_kernel(t, x, lp, step, n_leapfrog, np.eye(x.shape[1]), xi, u)
        else:
            prop = x + xi * step
            r = T.value(t, prop) - lp
            x2, lp2, _ = K.grw_kernel(t, x, lp, step, xi, u)
        margins[:, s] = np.abs(np.log(u) - r) / (1 + np.abs(r))
        x, lp = x2, lp2
    return margins


CASES = [
    ("mala", "std2", 0.5, 0), ("mala", "diag", 0.3, 0), ("mala", "dual_moon", 0.1, 0), ("mala", "mixture", 0.3, 0),
    ("mala", "rosenbrock", 0.05, 0), ("mala", "dense", 0.3, 0), ("mala", "mixture64", 0.2, 0),
    ("mala", "rosenbrock128", 0.01, 0),
    ("hmc", "std2", 0.3, 5), ("hmc", "diag", 0.2, 4), ("hmc", "dual_moon", 0.02, 3), ("hmc", "mixture", 0.1, 6),
    ("hmc", "rosenbrock", 0.01, 10), ("hmc", "dense", 0.1, 5), ("hmc", "rosenbrock128", 0.01, 16),
    ("grw", "std2", 1.0, 0), ("grw", "dual_moon", 0.05, 0), ("grw", "mixture", 0.5, 0),
    ("grw", "rosenbrock", 0.05, 0), ("grw", "mixture64", 0.1, 0),
    ("mala", "mixture20", 0.2, 0), ("grw", "diag20", 0.3, 0), ("hmc", "diag20", 0.1, 3),
    ("grw", "diag18", 0.3, 0), ("mala", "mixture132", 0.05, 0),
]


def _kernel(kind, step, nlf):
    from flowmc_gb300.resource.kernel.Gaussian_random_walk import GaussianRandomWalk
    from flowmc_gb300.resource.kernel.HMC import HMC
    from flowmc_gb300.resource.kernel.MALA import MALA
    if kind == "mala":
        return MALA(step)
    if kind == "hmc":
        return HMC(step_size=step, n_leapfrog=nlf)
    return GaussianRandomWalk(step)


@pytest.mark.parametrize("kind,tname,step,nlf", CASES, ids=[f"{c[0]}-{c[1]}" for c in CASES])
def test_trajectory_parity(tgts, kind, tname, step, nlf):
    tgt = tgts[tname]
    t = tgt.describe()
    d = tgt.n_dim
    C, S = 9, 25
    rng = np.random.default_rng(zlib.crc32(f"{kind}-{tname}".encode()))
    x0 = rng.normal(size=(C, d)).astype(np.float32)
    if tname.startswith("rosenbrock"):
        x0 = (0.3 * x0 + 0.5).astype(np.float32)
    noise = rng.normal(size=(C, S, d)).astype(np.float32)
    unif = rng.uniform(1e-6, 1, size=(C, S)).astype(np.float32)
    pos, lp, acc, xl, ll = _run_gpu(_kernel(kind, step, nlf), tgt, x0, noise, unif, S)
    opos, olp, oacc, olast = K.take_serial_steps(kind, t, x0.astype(np.float64), S, noise.astype(np.float64),
                                                 unif.astype(np.float64), step_size=step, n_leapfrog=nlf)
    margins = _oracle_ratios(kind, t, x0.astype(np.float64), noise, unif, S, step, nlf)
    n_cmp = 0
    for c in range(C):
        ties = np.nonzero(margins[c] < 1e-4)[0]
        upto = ties[0] if len(ties) else S
        sl = slice(0, upto)
        np.testing.assert_array_equal(acc[c, sl], oacc[c, sl], err_msg=f"chain {c}")
        np.testing.assert_allclose(pos[c, sl], opos[c, sl], rtol=RTOL, atol=ATOL, err_msg=f"chain {c}")
        np.testing.assert_allclose(lp[c, sl], olp[c, sl], rtol=RTOL, atol=ATOL * max(1, np.abs(olp[c, sl]).max()),
                                   err_msg=f"chain {c}")
        n_cmp += upto
    assert n_cmp >= 0.8 * C * S
    if not np.any(margins < 1e-4):
        np.testing.assert_allclose(xl, olast, rtol=RTOL, atol=ATOL)
    # acceptance must be neither all-reject nor trivially all-accept for the test to mean something
    assert 0 < acc.mean() <= 1


@pytest.mark.parametrize("tname", ["mixture", "mixture20"])
@pytest.mark.parametrize("lanes", [4, 8, 16, 32])
def test_lane_shapes_agree(tgts, lanes, tname):
    tgt = tgts[tname]
    C, S, d = 6, 12, tgt.n_dim
    rng = np.random.default_rng(5)
    x0 = rng.normal(size=(C, d)).astype(np.float32)
    noise = rng.normal(size=(C, S, d)).astype(np.float32)
    unif = rng.uniform(size=(C, S)).astype(np.float32)
    ref = _run_gpu(_kernel("mala", 0.3, 0), tgt, x0, noise, unif, S, lanes=0)
    out = _run_gpu(_kernel("mala", 0.3, 0), tgt, x0, noise, unif, S, lanes=lanes)
    np.testing.assert_allclose(out[0], ref[0], rtol=1e-5, atol=1e-6)
    np.testing.assert_array_equal(out[2], ref[2])


def test_thinning_cursor_and_clamp(tgts):
    tgt = tgts["std2"]
    C, S, d = 4, 10, 2
    rng = np.random.default_rng(9)
    x0 = rng.normal(size=(C, d)).astype(np.float32)
    noise = rng.normal(size=(C, S, d)).astype(np.float32)
    unif = rng.uniform(size=(C, S)).astype(np.float32)
    full = _run_gpu(_kernel("mala", 0.5, 0), tgt, x0, noise, unif, S)
    thin = _run_gpu(_kernel("mala", 0.5, 0), tgt, x0, noise, unif, S, thinning=4, cursor=5, buf_len=7)
    # 3 rows, cursor 5 clamps to 4 (buf_len 7 - 3)
    np.testing.assert_array_equal(thin[0][:, 4:7], full[0][:, ::4])
    assert np.isinf(thin[0][:, :4]).all()
    np.testing.assert_array_equal(thin[3], full[0][:, 8])      # last thinned row, not the last step


def test_determinism_and_philox_statistics(tgts):
    from flowmc_gb300.resource.kernel.base import run_local_steps
    tgt = tgts["std2"]
    dev = torch.device("cuda")
    C, S = 4096, 400
    x0 = torch.randn(C, 2, device=dev)
    outs = []
    for _ in range(2):
        pos = torch.empty(C, S, 2, device=dev)
        lp = torch.empty(C, S, device=dev)
        acc = torch.empty(C, S, device=dev)
        run_local_steps(_kernel("mala", 1.0, 0), tgt, x0, S, 1, 42, 7, pos, lp, acc, 0)
        outs.append((pos, lp, acc))
    assert torch.equal(outs[0][0], outs[1][0]) and torch.equal(outs[0][2], outs[1][2])
    p = outs[0][0][:, 100:].double()
    assert abs(p.mean().item()) < 1e-2 and abs(p.var().item() - 1) < 2e-2
    np.testing.assert_allclose(outs[0][1].cpu().numpy(), -0.5 * (outs[0][0] ** 2).sum(-1).cpu().numpy(), rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("kind,step", [("mala", 1e-5), ("hmc", 1e-7), ("grw", 1e-5)])
def test_acceptance_goes_to_one(tgts, kind, step):
    from flowmc_gb300.random import PRNGKey
    k = _kernel(kind, step, 5)
    x = torch.randn(100, 2, device="cuda")
    _, _, acc = k.kernel(PRNGKey(42), x, tgts["std2"](x), tgts["std2"])
    assert bool(acc.all())


@pytest.mark.parametrize("rounds", [10, 7])
@pytest.mark.parametrize("kind,step,nlf", [("mala", 1.0, 0), ("hmc", 0.1, 5), ("grw", 1.0, 0)])
def test_moments_standard_normal_philox(tgts, kind, step, nlf, rounds):
    """test_kernels.py:135-184 (N(0, I) moments within 3e-2), with the
    default Philox-4x32-10 noise and the opt-in Philox-4x32-7 noise."""
    from flowmc_gb300.resource.kernel.base import run_local_steps
    dev = torch.device("cuda")
    C, S = 2048, 1000
    x0 = torch.randn(C, 2, device=dev)
    pos = torch.empty(C, S, 2, device=dev)
    lp = torch.empty(C, S, device=dev)
    acc = torch.empty(C, S, device=dev)
    k = _kernel(kind, step, nlf)
    k.philox_rounds = rounds
    run_local_steps(k, tgts["std2"], x0, S, 1, 3, 0, pos, lp, acc, 0)
    p = pos.double()
    assert abs(p.mean().item()) < 3e-2
    assert abs(p.var().item() - 1) < 3e-2


def test_philox7_moments_64d_mixture_directions(tgts):
    """Philox-4x32-7 noise at a width where every lane draws several blocks
    (64-D standard normal, GRW, 16 lanes x 4 coordinates): per-coordinate
    means and variances within 4 standard errors of their targets, the
    cross-coordinate correlation near 0, and a stream different from the
    10-round one."""
    from flowmc_gb300 import targets as TG
    from flowmc_gb300.resource.kernel.base import run_local_steps
    dev = torch.device("cuda")
    tgt = TG.DiagGaussian(64, device=dev)
    C, S = 4096, 400
    x0 = torch.randn(C, 64, device=dev)
    res = {}
    for rounds in (10, 7):
        pos = torch.empty(C, S, 64, device=dev)
        lp = torch.empty(C, S, device=dev)
        acc = torch.empty(C, S, device=dev)
        k = _kernel("grw", 0.3, 0)
        k.philox_rounds = rounds
        run_local_steps(k, tgt, x0, S, 1, 11, 0, pos, lp, acc, 0)
        res[rounds] = pos[:, 200:].reshape(-1, 64).double()
    p = res[7]
    assert not torch.equal(res[7], res[10])
    # effective sample size is well below C * 200 (autocorrelated chains):
    # compare with a generous bound from the 10-round run's spread
    m, v = p.mean(0), p.var(0)
    m10, v10 = res[10].mean(0), res[10].var(0)
    tol_m = 6 * float(m10.abs().mean()) + 1e-2
    tol_v = 6 * float((v10 - 1).abs().mean()) + 1e-2
    assert float(m.abs().max()) < tol_m, (float(m.abs().max()), tol_m)
    assert float((v - 1).abs().max()) < tol_v, (float((v - 1).abs().max()), tol_v)
    c = torch.corrcoef(p[::7, :8].T)
    off = c - torch.eye(8, dtype=c.dtype, device=c.device)
    assert float(off.abs().max()) < 0.05


def test_errors_are_reported_not_raised_on_device(tgts):
    from flowmc_gb300 import _lib
    from flowmc_gb300.resource.kernel.base import run_local_steps
    dev = torch.device("cuda")
    x0 = torch.zeros(3, 2, device=dev)
    pos = torch.empty(3, 2, 2, device=dev)
    lp = torch.empty(3, 2, device=dev)
    acc = torch.empty(3, 2, device=dev)
    with pytest.raises(_lib.FlowMCError, match="INVALID_ARG"):
        run_local_steps(_kernel("mala", 0.1, 0), tgts["std2"], x0, 5, 1, 0, 0, pos, lp, acc, 0)  # 5 rows > 2
    with pytest.raises(RuntimeError, match="CUDA tensor"):
        run_local_steps(_kernel("mala", 0.1, 0), tgts["std2"], x0.cpu(), 1, 1, 0, 0, pos, lp, acc, 0)
    with pytest.raises(ValueError):
        run_local_steps(_kernel("mala", 0.1, 0), tgts["dual_moon"], x0, 1, 1, 0, 0, pos, lp, acc, 0)


def test_target_value_grad_entry(tgts):
    for name, tgt in tgts.items():
        t = tgt.describe()
        x = np.random.default_rng(1).normal(size=(33, tgt.n_dim)).astype(np.float32)
        lp, g = tgt.value_and_grad(torch.tensor(x, device="cuda"))
        olp, og = T.value_grad(t, x.astype(np.float64))
        np.testing.assert_allclose(lp.cpu().numpy(), olp, rtol=1e-5, atol=1e-4, err_msg=name)
        np.testing.assert_allclose(g.cpu().numpy(), og, rtol=1e-4, atol=1e-4, err_msg=name)


def _spd(d, seed):
    rng = np.random.default_rng(seed)
    Q, _ = np.linalg.qr(rng.normal(size=(d, d)))
    return Q @ np.diag(rng.uniform(0.5, 2.0, size=d)) @ Q.T


@pytest.mark.gpu
@pytest.mark.parametrize("tname,step,nlf,lanes", [("diag20", 0.3, 3, 0), ("mixture", 0.5, 3, 0), ("dense", 0.4, 3, 0),
                                                  ("diag20", 0.3, 3, 4), ("diag20", 0.3, 3, 32),
                                                  ("mixture132", 0.3, 3, 0)])
def test_hmc_dense_mass_matches_oracle(tgts, tname, step, nlf, lanes):
    """HMC with a dense condition matrix (HMC.py:133-137): momentum
    xi @ cholesky(inv(M)).T, kinetic energy with M's column sums; the fused
    kernel against the oracle on the same normals and uniforms."""
    from flowmc_gb300.resource.kernel.HMC import HMC
    tgt = tgts[tname]
    t = tgt.describe()
    d = tgt.n_dim
    M = _spd(d, d)
    C, S = 9, 20
    rng = np.random.default_rng(7 + d)
    x0 = rng.normal(size=(C, d)).astype(np.float32)
    noise = rng.normal(size=(C, S, d)).astype(np.float32)
    unif = rng.uniform(1e-6, 1, size=(C, S)).astype(np.float32)
    kern = HMC(condition_matrix=M, step_size=step, n_leapfrog=nlf)
    pos, lp, acc, xl, ll = _run_gpu(kern, tgt, x0, noise, unif, S, lanes=lanes)
    opos, olp, oacc, _ = K.take_serial_steps("hmc", t, x0.astype(np.float64), S, noise.astype(np.float64),
                                             unif.astype(np.float64), step_size=step, n_leapfrog=nlf, M=M)
    margins = K.accept_margins("hmc", t, x0, noise, unif, step_size=step, n_leapfrog=nlf, M=M)
    checked = 0
    for c in range(C):
        ties = np.nonzero(margins[c] < 1e-4)[0]
        upto = ties[0] if len(ties) else S
        np.testing.assert_array_equal(acc[c, :upto], oacc[c, :upto], err_msg=f"chain {c}")
        np.testing.assert_allclose(pos[c, :upto], opos[c, :upto], rtol=1e-4, atol=1e-4, err_msg=f"chain {c}")
        checked += upto
    assert checked >= C * S // 2
    assert 0 < oacc.mean() < 1   # both outcomes of the accept test occur
