"""RQSpline_MALA_Bundle and Sampler (mirrors test/unit/test_bundle.py:10-32,
test/integration/test_quickstart.py:28-51 and the strategy tests of
test/unit/test_strategies.py): construction on the host, then full runs of
the training -> production schedule on the GPU."""
import numpy as np
import pytest
import torch

from flowmc_gb300 import targets as TG
from flowmc_gb300.random import PRNGKey, split
from flowmc_gb300.resource_strategy_bundle.RQSpline_MALA import RQSpline_MALA_Bundle
from flowmc_gb300.Sampler import Sampler


def _bundle(device, **kw):
    args = dict(rng_key=PRNGKey(0), n_chains=2, n_dims=3, logpdf=TG.DiagGaussian(3, device=device),
                n_local_steps=10, n_global_steps=5, n_training_loops=2, n_production_loops=1, n_epochs=3,
                device=device)
    args.update(kw)
    return RQSpline_MALA_Bundle(**args)


def test_bundle_initialization_cpu():
    b = _bundle("cpu")
    assert repr(b) == "RQSpline_MALA Bundle"
    assert b.resources["positions_training"].shape == (2, 2 * (10 + 5), 3)
    assert b.resources["positions_production"].shape == (2, 10 + 5, 3)
    assert b.resources["loss_buffer"].shape == (6,)
    assert b.strategy_order[:6] == ["local_stepper", "update_global_step", "model_trainer", "update_model",
                                    "global_stepper", "update_local_step"]
    assert b.strategy_order[12:14] == ["reset_steppers", "update_state"]
    assert len(b.strategy_order) == 2 * 6 + 2 + 4
    assert torch.isinf(b.resources["positions_training"].data).all()


def test_sampler_requires_bundle_or_resources():
    with pytest.raises(ValueError):
        Sampler(3, 2, PRNGKey(0))


def test_sampler_unknown_strategy_name():
    b = _bundle("cpu")
    s = Sampler(3, 2, PRNGKey(0), resource_strategy_bundles=b)
    s.strategy_order = ["nope"]
    with pytest.raises(ValueError, match="Invalid strategy name"):
        s.sample(torch.zeros(2, 3), {})


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["float32", "bf16"])
def test_dual_moon_bundle_runs_end_to_end(cuda, precision):
    """The 5-D dual-moon bundle (20 chains, MALA 0.1, 30 local + 30 global
    steps), shortened to 3 + 2 loops: every buffer row is filled, values are
    finite, the losses were recorded and the chains move."""
    d, C = 5, 20
    key, sub = split(PRNGKey(0))
    b = RQSpline_MALA_Bundle(sub, C, d, TG.DualMoon(d), 30, 30, 3, 2, 5, mala_step_size=0.1,
                             rq_spline_hidden_units=[32, 32], rq_spline_n_bins=8, rq_spline_n_layers=4,
                             batch_size=10000, n_max_examples=10000, precision=precision, device="cuda")
    s = Sampler(d, C, key, resource_strategy_bundles=b)
    x0 = torch.tensor(np.random.default_rng(0).normal(size=(C, d)), dtype=torch.float32)
    last = s.sample(x0, {})
    torch.cuda.synchronize()
    r = s.resources
    for name in ("positions_training", "positions_production", "log_prob_training", "log_prob_production"):
        assert torch.isfinite(r[name].data).all(), name
    la = r["local_accs_production"].data.reshape(C, 2, 60)[:, :, :30]
    ga = r["global_accs_production"].data.reshape(C, 2, 60)[:, :, 30:]
    assert 0.2 < float(la.mean()) <= 1.0
    assert torch.isfinite(ga).all()
    assert torch.isfinite(r["loss_buffer"].data).all()
    assert r["loss_buffer"].data.shape == (15,)
    assert last.shape == (C, d)
    assert r["sampler_state"].data["training"] is False
    # reset to 0 before production, then two loops of 30 local + 30 global rows
    assert s.strategies["local_stepper"].current_position == 2 * 60


@pytest.mark.gpu
def test_take_serial_steps_kernel_switching(cuda):
    """test/unit/test_strategies.py:117-158: one TakeSerialSteps strategy run
    with MALA, then GRW, then HMC, with buffer cursors moving."""
    from flowmc_gb300.resource.buffers import Buffer
    from flowmc_gb300.resource.kernel.Gaussian_random_walk import GaussianRandomWalk
    from flowmc_gb300.resource.kernel.HMC import HMC
    from flowmc_gb300.resource.kernel.MALA import MALA
    from flowmc_gb300.resource.logPDF import LogPDF
    from flowmc_gb300.resource.states import State
    from flowmc_gb300.strategy.take_steps import TakeSerialSteps
    n_chains, n_steps, n_dims, n_batch = 5, 25, 2, 5
    res = {
        "test_position": Buffer("test_position", (n_chains, n_steps, n_dims), 1, device="cuda"),
        "test_log_prob": Buffer("test_log_prob", (n_chains, n_steps), 1, device="cuda"),
        "test_acceptance": Buffer("test_acceptance", (n_chains, n_steps), 1, device="cuda"),
        "logpdf": LogPDF(TG.DiagGaussian(n_dims, mean=[0.0, 1.0], device="cuda"), n_dims=n_dims),
        "MALA": MALA(1.0), "GRW": GaussianRandomWalk(1.0), "HMC": HMC(np.eye(n_dims), 0.1, 10),
        "sampler_state": State({"test_position": "test_position", "test_log_prob": "test_log_prob",
                                "test_acceptance": "test_acceptance"}, name="sampler_state"),
    }
    st = TakeSerialSteps("logpdf", "MALA", "sampler_state", ["test_position", "test_log_prob", "test_acceptance"],
                         n_batch)
    key = PRNGKey(42)
    pos = torch.zeros(n_chains, n_dims, device="cuda")
    for _ in range(n_batch):
        key, sub, _ = split(key, 3)
        _, res, pos = st(sub, res, pos, {})
    assert st.current_position == n_batch * n_batch
    assert torch.isfinite(res["test_position"].data).all()
    st.kernel_name = "GRW"
    st.set_current_position(0)
    _, res, pos = st(key, res, pos, {})
    st.kernel_name = "HMC"
    _, res, pos = st(key, res, pos, {})
    assert pos.shape == (n_chains, n_dims)
    assert st.current_position == 2 * n_batch


@pytest.mark.gpu
def test_take_group_steps_nf_proposal(cuda):
    """test/unit/test_strategies.py:251-319: TakeGroupSteps with NFProposal
    for 11 and 5 steps; the proposal's own model is the target."""
    from flowmc_gb300.resource.buffers import Buffer
    from flowmc_gb300.resource.kernel.NF_proposal import NFProposal
    from flowmc_gb300.resource.logPDF import LogPDF
    from flowmc_gb300.resource.model.nf_model.rqSpline import MaskedCouplingRQSpline
    from flowmc_gb300.resource.states import State
    from flowmc_gb300.strategy.take_steps import TakeGroupSteps
    C, S, d = 5, 25, 2
    model = MaskedCouplingRQSpline(d, 3, [16, 16], 8, PRNGKey(10), device="cuda")
    res = {"p": Buffer("p", (C, S, d), 1, device="cuda"), "l": Buffer("l", (C, S), 1, device="cuda"),
           "a": Buffer("a", (C, S), 1, device="cuda"), "NFProposal": NFProposal(model, n_NFproposal_batch_size=5),
           "logpdf": LogPDF(TG.DiagGaussian(d, device="cuda"), n_dims=d),
           "sampler_state": State({"p": "p", "l": "l", "a": "a"}, name="sampler_state")}
    for n in (11, 5):
        st = TakeGroupSteps("logpdf", "NFProposal", "sampler_state", ["p", "l", "a"], n_steps=n)
        _, res, last = st(PRNGKey(42), res, torch.zeros(C, d, device="cuda"), {})
        assert last.shape == (C, d) and torch.isfinite(last).all()
        assert torch.isfinite(res["p"].data[:, :n]).all()
    assert repr(res["NFProposal"]).startswith("NF proposal with MaskedCouplingRQSpline")


@pytest.mark.gpu
def test_train_model_strategy(cuda):
    """test/unit/test_strategies.py:224-249: TrainModel keeps the model type and fills the loss buffer."""
    from flowmc_gb300.resource.buffers import Buffer
    from flowmc_gb300.resource.model.nf_model.rqSpline import MaskedCouplingRQSpline
    from flowmc_gb300.resource.optimizer import Optimizer
    from flowmc_gb300.strategy.train_model import TrainModel
    C, S, d = 5, 25, 2
    model = MaskedCouplingRQSpline(d, 3, [16, 16], 8, PRNGKey(10), device="cuda")
    data = Buffer("test_data", (C, S, d), 1, device="cuda")
    data.update_buffer(torch.randn(C, S, d, device="cuda"))
    loss = Buffer("loss", (10,), 0, device="cuda")
    res = {"test_data": data, "optimizer": Optimizer(model), "model": model, "loss": loss}
    st = TrainModel("model", "test_data", "optimizer", loss_buffer_name="loss", n_epochs=10, batch_size=C * S,
                    n_max_examples=10000, history_window=1, verbose=False)
    _, res, _ = st(PRNGKey(42), res, torch.zeros(C, d, device="cuda"), {})
    assert isinstance(res["model"], MaskedCouplingRQSpline)
    assert torch.isfinite(res["loss"].data).all() and res["loss"].cursor == 10
    st.check_errors()


@pytest.mark.gpu
def test_train_model_uneven_rows_raise(cuda):
    """A chain that produced a NaN row leaves finite rows that do not split
    evenly over the chains: the reference's reshape raises there
    (train_model.py:66-70). Here the selection fills the training data with
    NaN (the epoch losses are NaN, never stale memory) and the strategy's
    next call, or Sampler.poll_errors, raises ValueError without a stream
    sync; a CUDA-graph replay raises on the next replay."""
    from flowmc_gb300.resource.buffers import Buffer
    from flowmc_gb300.resource.model.nf_model.rqSpline import MaskedCouplingRQSpline
    from flowmc_gb300.resource.optimizer import Optimizer
    from flowmc_gb300.strategy.lambda_function import Lambda
    from flowmc_gb300.strategy.train_model import TrainModel
    C, S, d = 4, 20, 2
    model = MaskedCouplingRQSpline(d, 2, [8, 8], 4, PRNGKey(10), device="cuda")
    data = Buffer("test_data", (C, S, d), 1, device="cuda")
    rows = torch.randn(C, S, d, device="cuda")
    rows[2, 7, 1] = float("nan")
    data.update_buffer(rows)
    loss = Buffer("loss", (6,), 0, device="cuda")
    res = {"test_data": data, "optimizer": Optimizer(model), "model": model, "loss": loss}
    st = TrainModel("model", "test_data", "optimizer", loss_buffer_name="loss", n_epochs=3, batch_size=32,
                    n_max_examples=64, history_window=5, verbose=False)
    _, res, _ = st(PRNGKey(1), res, torch.zeros(C, d, device="cuda"), {})
    assert torch.isnan(res["loss"].data[:3]).all()
    with pytest.raises(ValueError, match="do not split evenly"):
        st(PRNGKey(2), res, torch.zeros(C, d, device="cuda"), {})
    # through the Sampler: eager run, then a captured schedule
    s = Sampler(d, C, PRNGKey(0), resources=res, strategies={"train": st, "noop": Lambda(lambda *a: None)},
                strategy_order=["train"])
    with pytest.raises(ValueError, match="do not split evenly"):
        s.sample(torch.zeros(C, d), {})
    cap = s.capture(torch.zeros(C, d, device="cuda"), {})
    cap.replay(torch.zeros(C, d, device="cuda"))
    with pytest.raises(ValueError, match="do not split evenly"):
        cap.replay(torch.zeros(C, d, device="cuda"))
    # finite rows that split evenly: no error
    data.update_buffer(torch.randn(C, S, d, device="cuda"))
    _, res, _ = st(PRNGKey(3), res, torch.zeros(C, d, device="cuda"), {})
    s.poll_errors()
    st.check_errors()


def test_nvtx_ranges_around_strategies_cpu():
    """With NVTX on, the sampler still runs its strategies in order (the
    ranges are no-ops without a timeline profiler attached)."""
    from flowmc_gb300 import profiling
    from flowmc_gb300.strategy.lambda_function import Lambda
    seen = []
    s = Sampler(3, 2, PRNGKey(0), resources={},
                strategies={"a": Lambda(lambda *a: seen.append("a")), "b": Lambda(lambda *a: seen.append("b"))},
                strategy_order=["a", "b", "a"])
    profiling.set_nvtx(True)
    try:
        with profiling.region("outer"):
            s.sample(torch.zeros(2, 3), {})
    finally:
        profiling.set_nvtx(False)
    assert seen == ["a", "b", "a"]


def test_sequential_monte_carlo_is_declared_but_not_constructible():
    from flowmc_gb300.strategy.sequential_monte_carlo import SequentialMonteCarlo
    with pytest.raises(TypeError):
        SequentialMonteCarlo()


def test_take_steps_checks_its_resources_cpu():
    """take_steps.py:74-97: the State and Buffer checks and their messages."""
    from flowmc_gb300.resource.buffers import Buffer
    from flowmc_gb300.resource.kernel.MALA import MALA
    from flowmc_gb300.resource.states import State
    from flowmc_gb300.strategy.take_steps import TakeSerialSteps
    st = TakeSerialSteps("logpdf", "MALA", "state", ["p", "l", "a"], n_steps=2)
    res = {"MALA": MALA(0.1), "state": {"p": "p"}}
    with pytest.raises(AssertionError, match="State resource must be a State"):
        st(PRNGKey(0), res, torch.zeros(2, 3), {})
    res["state"] = State({"p": "p", "l": 3, "a": "a"}, name="state")
    with pytest.raises(AssertionError, match="Log probability buffer resource name must be a string"):
        st(PRNGKey(0), res, torch.zeros(2, 3), {})
    res["state"] = State({"p": "p", "l": "l", "a": "a"}, name="state")
    res.update({"p": Buffer("p", (2, 4, 3), 1, device="cpu"), "l": Buffer("l", (2, 4), 1, device="cpu"),
                "a": "not a buffer"})
    with pytest.raises(AssertionError, match="Acceptance buffer resource must be a Buffer"):
        st(PRNGKey(0), res, torch.zeros(2, 3), {})
