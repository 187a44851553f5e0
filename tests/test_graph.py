"""The sampling schedule as one CUDA graph (Sampler.capture / sample with
cuda_graph=True) and the library's random-stream epoch word.

A replay re-executes the captured launches, advancing the epoch word first:
with the word set so that the replay runs at epoch E, the replay must
reproduce an eager run at epoch E bit for bit (every kernel of the path is
deterministic); the next replay draws fresh numbers."""
import numpy as np
import pytest
import torch

from flowmc_gb300 import _lib
from flowmc_gb300 import targets as TG
from flowmc_gb300.random import PRNGKey, split
from flowmc_gb300.resource_strategy_bundle.RQSpline_MALA import RQSpline_MALA_Bundle
from flowmc_gb300.resource_strategy_bundle.RQSpline_MALA_PT import RQSpline_MALA_PT_Bundle
from flowmc_gb300.Sampler import Sampler

BUFS = ("positions_training", "log_prob_training", "local_accs_training", "global_accs_training",
        "positions_production", "log_prob_production", "local_accs_production", "global_accs_production",
        "loss_buffer")


def _sampler(precision, pt=False):
    d, C = 5, 64
    key, sub = split(PRNGKey(0))
    kw = dict(mala_step_size=0.1, rq_spline_hidden_units=[32, 32], rq_spline_n_bins=8, rq_spline_n_layers=3,
              batch_size=4096, n_max_examples=4096, precision=precision, device="cuda")
    if pt:
        b = RQSpline_MALA_PT_Bundle(sub, C, d, TG.DualMoon(d), 10, 10, 2, 2, 3, n_temperatures=3, **kw)
    else:
        b = RQSpline_MALA_Bundle(sub, C, d, TG.DualMoon(d), 10, 10, 2, 2, 3, **kw)
    return Sampler(d, C, key, resource_strategy_bundles=b), b


def _snapshot(bundle):
    return {k: bundle.resources[k].data.clone() for k in BUFS}


@pytest.mark.gpu
@pytest.mark.parametrize("precision,pt", [("float32", False), ("bf16", False), ("float32", True)])
def test_graph_replay_reproduces_eager_run(cuda, precision, pt):
    epoch = _lib.rng_epoch()
    x0 = torch.randn(64, 5, generator=torch.Generator().manual_seed(1)).cuda()
    sa, ba = _sampler(precision, pt)
    epoch.fill_(5)
    out_a = sa.sample(x0, {})
    torch.cuda.synchronize()
    ref = _snapshot(ba)
    sb, bb = _sampler(precision, pt)
    cap = sb.capture(x0, {})
    epoch.fill_(4)                           # the replay advances it to 5 first
    out_b = cap.replay(x0)
    torch.cuda.synchronize()
    assert int(epoch.item()) == 5
    for k in BUFS:
        assert torch.equal(bb.resources[k].data, ref[k]), k
    assert torch.equal(out_b, out_a)
    assert torch.isfinite(ref["positions_production"]).all()
    # the next replay (epoch 6) draws fresh numbers and still fills every row
    out_c = sb.sample(x0, {}, cuda_graph=True)
    torch.cuda.synchronize()
    assert int(epoch.item()) == 6
    assert not torch.equal(bb.resources["positions_production"].data, ref["positions_production"])
    assert torch.isfinite(bb.resources["positions_production"].data).all() and torch.isfinite(out_c).all()
    epoch.zero_()


@pytest.mark.gpu
def test_epoch_zero_leaves_streams_unchanged(cuda):
    """A zero epoch word is the library's plain stream: the local kernel
    draws the same numbers with the word attached as without it."""
    from flowmc_gb300.resource.kernel.MALA import MALA
    from flowmc_gb300.resource.kernel.base import run_local_steps
    tgt = TG.DiagGaussian(6)
    x0 = torch.randn(256, 6, device="cuda")
    outs = []
    for attach in (False, True):
        _lib.check(_lib.lib().fmc_rng_epoch_attach(_lib.rng_epoch().data_ptr() if attach else None))
        _lib.rng_epoch().zero_() if attach else None
        pos = torch.empty(256, 20, 6, device="cuda")
        lp = torch.empty(256, 20, device="cuda")
        acc = torch.empty(256, 20, device="cuda")
        run_local_steps(MALA(0.3), tgt, x0, 20, 1, 99, 0, pos, lp, acc, 0)
        outs.append(pos.clone())
    assert torch.equal(outs[0], outs[1])
    w = _lib.rng_epoch()
    w.fill_(3)
    pos = torch.empty(256, 20, 6, device="cuda")
    run_local_steps(MALA(0.3), tgt, x0, 20, 1, 99, 0, pos, lp, acc, 0)
    assert not torch.equal(pos, outs[0])
    w.zero_()
