"""Streaming FP64 diagnostics on the device (fmc_welford_ess_update /
fmc_welford_ess_finalize) against the float64 oracle (oracle/streaming.py),
through the C ABI: the same per-chain Welford recurrences, so per-coordinate
means, variances, R-hat and batch-means ESS agree to 1e-12 relative (the
chain merge is a tree on the device and a sequential sum in the oracle)."""
import numpy as np
import pytest
import torch

from oracle.streaming import StreamingOracle

pytestmark = pytest.mark.gpu


def _close(got, ref):
    np.testing.assert_allclose(got.cpu().numpy(), ref, rtol=1e-12, atol=1e-12 * max(1.0, np.abs(ref).max()))


@pytest.mark.parametrize("C,d,S,batch,calls", [(37, 5, 90, 7, [(0, 13), (13, 50), (50, 90)]),
                                               (2048, 64, 240, 50, [(0, 100), (100, 240)])])
def test_streaming_moments_match_oracle(cuda, C, d, S, batch, calls):
    from flowmc_gb300.diagnostics import StreamingMoments
    rng = np.random.default_rng(C + d)
    buf = (rng.normal(size=(C, S, d)) * rng.uniform(0.2, 3.0, size=d) + rng.uniform(-5, 5, size=d))
    buf = buf.astype(np.float32)
    bt = torch.tensor(buf, device="cuda")
    sm = StreamingMoments(C, d, batch)
    so = StreamingOracle(C, d, batch)
    for lo, hi in calls:
        sm.update(bt, lo, hi - lo)
        so.update(buf[:, lo:hi])
    got = sm.finalize()
    mu, var, ess, rhat = so.finalize()
    assert sm.draws() == S
    _close(got["mean"], mu)
    _close(got["var"], var)
    _close(got["ess"], ess)
    _close(got["rhat"], rhat)
    # reset starts over
    sm.reset()
    assert sm.draws() == 0


def test_streaming_update_replays_in_a_graph(cuda):
    """An update captured in a CUDA graph reads the draw count from the
    device state, so two replays equal two eager updates of the same rows."""
    from flowmc_gb300.diagnostics import StreamingMoments
    C, d, S = 128, 16, 30
    buf = torch.randn(C, S, d, device="cuda")
    a, b = StreamingMoments(C, d, 12), StreamingMoments(C, d, 12)
    a.update(buf, 0, S)
    a.update(buf, 0, S)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        b.update(buf, 0, S)
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    assert b.draws() == 2 * S
    ra, rb = a.finalize(), b.finalize()
    for k in ra:
        torch.testing.assert_close(rb[k], ra[k], rtol=0, atol=0, equal_nan=True)


def test_bundle_streaming_diagnostics_equal_posthoc(cuda):
    """RQSpline_MALA_Bundle(streaming_diagnostics=True) accumulates every
    production row once: its means and variances equal the post-hoc float64
    moments of positions_production, eager and as a captured schedule."""
    from flowmc_gb300 import diagnostics as D
    from flowmc_gb300 import targets as TG
    from flowmc_gb300.random import PRNGKey, split
    from flowmc_gb300.resource_strategy_bundle.RQSpline_MALA import RQSpline_MALA_Bundle
    from flowmc_gb300.Sampler import Sampler
    d, C = 5, 64
    for graph in (False, True):
        key, sub = split(PRNGKey(0))
        b = RQSpline_MALA_Bundle(sub, C, d, TG.DualMoon(d), 10, 10, 2, 3, 3, mala_step_size=0.1,
                                 rq_spline_hidden_units=[16, 16], rq_spline_n_bins=8, rq_spline_n_layers=2,
                                 batch_size=1000, n_max_examples=1000, device="cuda", streaming_diagnostics=True)
        s = Sampler(d, C, key, resource_strategy_bundles=b)
        s.sample(torch.randn(C, d), {}, cuda_graph=graph)
        torch.cuda.synchronize()
        pos = b.resources["positions_production"].data
        assert torch.isfinite(pos).all()
        st = b.production_moments.finalize()
        mu, var = D.moments(pos)
        torch.testing.assert_close(st["mean"], mu, rtol=1e-9, atol=1e-9)
        torch.testing.assert_close(st["var"], var, rtol=1e-9, atol=1e-9)
        assert b.production_moments.draws() == pos.shape[1]
        assert torch.isfinite(st["ess"]).all() and (st["ess"] > 0).all()
