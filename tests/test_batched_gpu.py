"""Batched dense-Gaussian local steps (many targets of uneven dimension in one
launch) against the oracle, through the C ABI: same explicit noise, 1e-5
relative trajectories with identical accepts away from ties; with Philox
noise, sample covariances against the analytic ones."""
import numpy as np
import pytest
import torch

from oracle import kernels as K

pytestmark = pytest.mark.gpu


def make(dims, seed=1):
    from flowmc_gb300 import targets as TG
    rng = np.random.default_rng(seed)
    ts, covs = [], []
    for d in dims:
        Q, R = np.linalg.qr(rng.normal(size=(d, d)))
        Q = Q * np.sign(np.diag(R))
        lam = np.exp(rng.uniform(np.log(0.05), np.log(2.0), size=d))
        cov = Q @ np.diag(lam) @ Q.T
        ts.append(TG.DenseGaussian(np.linalg.inv(cov), device="cuda"))
        covs.append(cov)
    return ts, covs


@pytest.mark.parametrize("kind,nlf", [("mala", 0), ("hmc", 6)])
def test_batched_trajectories_match_oracle(cuda, kind, nlf):
    from flowmc_gb300.batched import BatchedDenseLocalSteps
    dims, chains = [5, 40, 130, 256], [40, 70, 33, 9]
    ts, covs = make(dims)
    steps = [0.3 * np.sqrt(np.linalg.eigvalsh(c).min()) for c in covs]
    S = 12
    rng = np.random.default_rng(3)
    xs = [rng.normal(size=(c, d)).astype(np.float32) for c, d in zip(chains, dims)]
    nz = [rng.normal(size=(c, S, d)).astype(np.float32) for c, d in zip(chains, dims)]
    un = [rng.uniform(1e-6, 1, size=(c, S)).astype(np.float32) for c in chains]
    b = BatchedDenseLocalSteps(ts, chains, steps, kind=kind, n_leapfrog=nlf)
    outs, xl, ll = b.run([torch.tensor(x, device="cuda") for x in xs], S, seed=5,
                         noise=[torch.tensor(z, device="cuda") for z in nz],
                         uniform=[torch.tensor(u, device="cuda") for u in un])
    torch.cuda.synchronize()
    for t in range(len(dims)):
        pos, lp, acc = (o.cpu().numpy() for o in outs[t])
        opos, olp, oacc, olast = K.take_serial_steps(kind, ts[t].describe(), xs[t].astype(np.float64), S,
                                                     nz[t].astype(np.float64), un[t].astype(np.float64),
                                                     step_size=steps[t], n_leapfrog=nlf, M=np.eye(dims[t]))
        agree = (acc == oacc).mean()
        assert agree >= 0.97, (t, agree)
        ok = (acc == oacc).all(1)           # chains without a tie flip
        np.testing.assert_allclose(pos[ok], opos[ok], rtol=1e-4, atol=1e-4)
        np.testing.assert_allclose(lp[ok], olp[ok], rtol=1e-4, atol=1e-3)
        assert ok.mean() >= 0.9


def test_batched_moments_philox(cuda):
    from flowmc_gb300.batched import BatchedDenseLocalSteps
    dims, chains = [8, 33, 64], [1024, 700, 1200]
    ts, covs = make(dims, seed=7)
    steps = [0.5 * np.sqrt(np.linalg.eigvalsh(c).min()) * d ** (-1 / 3) for c, d in zip(covs, dims)]
    S = 600
    b = BatchedDenseLocalSteps(ts, chains, steps, kind="hmc", n_leapfrog=10)
    xs = [torch.randn(c, d, device="cuda") for c, d in zip(chains, dims)]
    outs, _, _ = b.run(xs, S, seed=11)
    for t, cov in enumerate(covs):
        pos = outs[t][0][:, 100:].reshape(-1, dims[t]).double().cpu().numpy()
        emp = np.cov(pos.T)
        rel = np.linalg.norm(emp - cov) / np.linalg.norm(cov)
        assert rel < 0.1, (t, rel)
        assert np.abs(pos.mean(0)).max() < 0.15 * np.sqrt(np.diag(cov)).max()


def test_batched_rejects_non_dense(cuda):
    from flowmc_gb300 import targets as TG
    from flowmc_gb300.batched import BatchedDenseLocalSteps
    with pytest.raises(TypeError):
        BatchedDenseLocalSteps([TG.DiagGaussian(3)], [4], [0.1])
