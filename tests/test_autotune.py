"""Chain-block autotuner: candidate shapes and that every tuned shape samples the same chains."""
import pytest
import torch

from flowmc_gb300 import autotune


def test_candidates_cover_valid_shapes():
    assert autotune.candidates(2) == [4, 8, 16, 32]
    assert autotune.candidates(64) == [8, 16, 32]
    assert autotune.candidates(128) == [16, 32]
    assert autotune.candidates(256) == [32]
    for d in (3, 17, 100, 200):
        for g in autotune.candidates(d):
            v = 1
            while g * v < d:
                v *= 2
            assert v <= 8


@pytest.mark.gpu
@pytest.mark.parametrize("kname", ["MALA", "GRW", "HMC"])
def test_tuned_shape_matches_default_shape(cuda, kname):
    from flowmc_gb300.resource.kernel.base import run_local_steps
    from flowmc_gb300.resource.kernel.MALA import MALA
    from flowmc_gb300.resource.kernel.HMC import HMC
    from flowmc_gb300.resource.kernel.Gaussian_random_walk import GaussianRandomWalk
    from flowmc_gb300.targets import GaussianMixture
    d, C, S = 48, 1024, 6
    g = torch.Generator().manual_seed(3)
    tgt = GaussianMixture(torch.randn(4, d, generator=g), torch.full((4, d), 0.5), torch.ones(4) / 4, device="cuda")
    kern = {"MALA": lambda: MALA(step_size=0.05), "GRW": lambda: GaussianRandomWalk(step_size=0.1),
            "HMC": lambda: HMC(step_size=0.05, n_leapfrog=4)}[kname]()
    best = autotune.tune_local_kernel(kern, tgt, C, probe_steps=4, reps=1)
    assert best in autotune.candidates(d)
    x0 = torch.randn(C, d, generator=g).cuda()
    outs = []
    for lanes in autotune.candidates(d):
        kern.lanes_per_chain = lanes
        pos = torch.empty(C, S, d, device="cuda")
        lp = torch.empty(C, S, device="cuda")
        acc = torch.empty(C, S, device="cuda")
        run_local_steps(kern, tgt, x0, S, 1, 11, 0, pos, lp, acc, 0)
        outs.append((pos, lp, acc))
    # the noise is indexed by (chain, step, coordinate), so shapes differ only in reduction order
    for pos, lp, acc in outs[1:]:
        same = (acc == outs[0][2]).float().mean().item()
        assert same > 0.99
        ok = (acc == outs[0][2]).all(dim=1)
        torch.testing.assert_close(pos[ok], outs[0][0][ok], rtol=1e-3, atol=1e-3)
        torch.testing.assert_close(lp[ok], outs[0][1][ok], rtol=1e-3, atol=1e-3)


@pytest.mark.gpu
def test_flow_gemm_tile_width_is_tuned_and_changes_no_result(cuda):
    """The BF16 hidden-layer GEMMs give the same log-densities with 128- and
    256-column tiles (each output's K reduction is the same); the tuner
    picks one of them and records it on the model."""
    import torch
    from flowmc_gb300.autotune import tune_flow_gemm
    from flowmc_gb300.random import PRNGKey
    from flowmc_gb300.resource.model.nf_model.rqSpline import MaskedCouplingRQSpline
    m = MaskedCouplingRQSpline(24, 3, [512, 512], 8, PRNGKey(0), precision="bf16", device="cuda")
    m.theta.add_(torch.randn_like(m.theta) * 0.02)
    m.sync_bf16()
    x = torch.randn(5000, 24, device="cuda")
    out = {}
    for bn in (256, 128):
        m.gemm_bn = bn
        out[bn] = m.log_prob(x)
    torch.testing.assert_close(out[128], out[256], rtol=0, atol=0)
    # the K >= 256 hidden GEMMs' ring depth: identical outputs
    m.gemm_bn, m.tile_rows = 256, 128
    for stages in (3, 4):
        m.gemm_stages = stages
        out[stages] = m.log_prob(x)
    torch.testing.assert_close(out[3], out[4], rtol=0, atol=0)
    torch.testing.assert_close(out[3], out[256], rtol=0, atol=0)
    pick = tune_flow_gemm(m, n_rows=8192, reps=1)
    assert pick in (128, 256) and m.gemm_bn == pick
    assert m.tile_rows in (128, 256) and m.gemm_stages in (0, 3, 4)
    assert len(m.tile_timings_ms) in (4, 6)


@pytest.mark.gpu
def test_flow_wgrad_split_is_tuned_and_changes_no_more_than_rounding(cuda):
    """The BF16 training's weight-gradient GEMMs with different K-slice counts
    give the same gradient up to float32 summation order; the tuner picks a
    candidate and records the timings."""
    import torch
    from flowmc_gb300.autotune import tune_flow_train
    from flowmc_gb300.random import PRNGKey
    from flowmc_gb300.resource.model.nf_model.rqSpline import MaskedCouplingRQSpline
    m = MaskedCouplingRQSpline(24, 3, [256, 256], 8, PRNGKey(1), precision="bf16", device="cuda")
    m.theta.add_(torch.randn_like(m.theta) * 0.02)
    m.sync_bf16()
    x = torch.randn(6000, 24, device="cuda")
    grads = {}
    for sl in (0, 1, 4, 16):
        m.wgrad_splits = sl
        loss, g = m.loss_and_grad(x)
        grads[sl] = g.clone()
    for sl in (1, 4, 16):
        torch.testing.assert_close(grads[sl], grads[0], rtol=1e-4, atol=1e-5 * float(grads[0].abs().max()))
    pick = tune_flow_train(m, n_rows=4096, reps=1, candidates=(0, 2, 8))
    assert pick in (0, 2, 8) and m.wgrad_splits == pick and len(m.train_timings_ms) == 3
