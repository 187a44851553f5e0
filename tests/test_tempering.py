"""Parallel tempering (strategy/parallel_tempering.py, resource/logPDF.py's
TemperedPDF and resource_strategy_bundle/RQSpline_MALA_PT.py of the reference).

CPU: the oracle reproduces the golden vectors made by running the
reference's own ParallelTempering methods (tests/golden/make_golden.py) in
float64; TemperedPDF's prior handling; the PT bundle's resources and
schedule. GPU: the fused tempered local steps, the exchange sweep and the
adaptation against the golden vectors and the oracle on the same draws
(float32 trajectory tolerance 1e-5 relative, identical accept and swap
decisions away from near-ties), then statistical checks of the in-kernel
random streams and an end-to-end PT bundle run."""
import json
import os

import numpy as np
import pytest
import torch

from flowmc_gb300 import targets as TG
from flowmc_gb300.random import PRNGKey, split
from flowmc_gb300.resource.logPDF import LogPDF, TemperedPDF
from flowmc_gb300.resource_strategy_bundle.RQSpline_MALA_PT import RQSpline_MALA_PT_Bundle
from oracle import kernels as K
from oracle import tempering as PT

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz")


def _load():
    z = np.load(GOLD)
    return z, json.loads(str(z["cases"]))


def _pt_cases():
    _, cases = _load()
    return [c for c in cases if c["kind"] == "pt"]


def _M(case, d):
    return np.eye(d) if case["local"] == "hmc" else None


@pytest.mark.parametrize("case", _pt_cases(), ids=lambda c: c["name"])
def test_oracle_parallel_tempering_matches_reference_source(case):
    z, _ = _load()
    n, t = case["name"], case["target"]
    x0, noise, unif, u_ex, temps = (z[f"{n}/{k}"] for k in ("x0", "noise", "unif", "u_exchange", "temps"))
    C, Tn, S, d = noise.shape
    x, lp, acc = PT.ensemble_step(case["local"], t, x0, temps, S, noise, unif, step_size=case["step_size"],
                                  n_leapfrog=case["n_leapfrog"], M=_M(case, d), prior=case.get("prior"))
    np.testing.assert_array_equal(acc, z[f"{n}/ens_acc"])
    np.testing.assert_allclose(x, z[f"{n}/ens_x"], rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(lp, z[f"{n}/ens_lp"], rtol=1e-9, atol=1e-10)
    x2, lp2, acc2 = PT.exchange(t, x, temps, u_ex)
    np.testing.assert_array_equal(acc2, z[f"{n}/ex_acc"])
    np.testing.assert_allclose(x2, z[f"{n}/ex_x"], rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(lp2, z[f"{n}/ex_lp"], rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(PT.adapt_temperature(temps, acc2), z[f"{n}/new_temps"], rtol=1e-12)
    # the fixture exercises both outcomes of the swap test
    assert 0 < z[f"{n}/ex_acc"].mean() < 1


def test_oracle_adapt_temperature_matches_reference_source():
    z, _ = _load()
    new = PT.adapt_temperature(z["pt_adapt/temps"], z["pt_adapt/flags"])
    np.testing.assert_allclose(new, z["pt_adapt/new_temps"], rtol=1e-12)
    assert new[0] == z["pt_adapt/temps"][0] and new[-1] == z["pt_adapt/temps"][-1]


def test_oracle_exchange_edge_cases():
    t = {"kind": "diag_gaussian", "mean": np.zeros(3), "inv_var": np.ones(3), "const": 0.0}
    rng = np.random.default_rng(1)
    x = rng.normal(size=(4, 3, 3))
    # one temperature: nothing to exchange
    x1, lp1, acc1 = PT.exchange(t, x[:, :1], [1.0], np.zeros((4, 0)))
    np.testing.assert_array_equal(x1, x[:, :1])
    assert acc1.shape == (4, 0)
    # equal temperatures: the ratio is 0 and every swap with u < 1 is taken,
    # so the sequential sweep carries row 0 to the end
    x3, _, acc3 = PT.exchange(t, x, [1.0, 1.0, 1.0], np.full((4, 2), 0.5))
    assert acc3.all()
    np.testing.assert_array_equal(x3, x[:, [1, 2, 0]])


def test_tempered_pdf_prior_handling():
    like = TG.DiagGaussian(3, device="cpu")
    assert TemperedPDF(like, None, n_dims=3).prior_arrays("cpu") is None
    assert TemperedPDF(LogPDF(like, n_dims=3), lambda x, _: 0.0, n_dims=3).prior_arrays("cpu") is None
    assert TemperedPDF(like, lambda x, _: np.array(0.0), n_dims=3).prior_arrays("cpu") is None
    assert TemperedPDF(like, lambda x, _: torch.zeros(()), n_dims=3).prior_arrays("cpu") is None
    m, iv, c = TemperedPDF(like, TG.DiagGaussian(3, mean=[1, 2, 3], inv_var=[1, 2, 4], const=-0.5, device="cpu"),
                           n_dims=3).prior_arrays("cpu")
    assert m.tolist() == [1, 2, 3] and iv.tolist() == [1, 2, 4] and c == -0.5
    with pytest.raises(NotImplementedError):
        TemperedPDF(like, lambda x, _: float(np.sum(x)), n_dims=3)
    with pytest.raises(NotImplementedError):
        TemperedPDF(like, lambda x, _: 0.0 if np.all(np.abs(x) < 10) else -np.inf, n_dims=3)
    with pytest.raises(ValueError):
        TemperedPDF(like, TG.DiagGaussian(2, device="cpu"), n_dims=3)


def test_pt_bundle_initialization_cpu():
    """test/unit/test_bundle.py's construction checks, for the PT bundle."""
    b = RQSpline_MALA_PT_Bundle(PRNGKey(0), 2, 3, TG.DiagGaussian(3, device="cpu"), 10, 5, 2, 1, 3,
                                n_temperatures=4, max_temperature=7.0, device="cpu")
    assert repr(b) == "RQSpline MALA PT Bundle"
    assert b.resources["tempered_positions"].shape == (2, 3, 3)
    np.testing.assert_allclose(b.resources["temperatures"].data.numpy(), [1.0, 3.0, 5.0, 7.0])
    assert isinstance(b.resources["tempered_logpdf"], TemperedPDF)
    assert b.strategy_order[0] == "initialize_tempered_positions"
    assert b.strategy_order[1:8] == ["parallel_tempering", "local_stepper", "update_global_step", "model_trainer",
                                     "update_model", "global_stepper", "update_local_step"]
    assert b.strategy_order[15:17] == ["reset_steppers", "update_state"]
    assert b.strategy_order[17:] == ["parallel_tempering", "local_stepper", "update_global_step",
                                     "global_stepper", "update_local_step"]
    assert b.strategies["parallel_tempering"].n_steps == 10   # n_tempered_steps <= 0 -> n_local_steps


# ---------------------------------------------------------------------- GPU
def _target(t, device="cuda"):
    if t["kind"] == "dual_moon":
        return TG.DualMoon(t["n_dim"], r0=t["r0"], sr=t["sr"], mu=t["mu"], s0=t["s0"], device=device)
    if t["kind"] == "rosenbrock":
        return TG.Rosenbrock(t["n_dim"], a=t["a"], b=t["b"], c=t["c"], device=device)
    return TG.DiagGaussian(len(t["mean"]), mean=t["mean"], inv_var=t["inv_var"], const=t.get("const", 0.0),
                           device=device)


def _kernel(kind, step, nlf):
    from flowmc_gb300.resource.kernel.Gaussian_random_walk import GaussianRandomWalk
    from flowmc_gb300.resource.kernel.HMC import HMC
    from flowmc_gb300.resource.kernel.MALA import MALA
    if kind == "mala":
        return MALA(step)
    if kind == "hmc":
        return HMC(step_size=step, n_leapfrog=nlf)
    return GaussianRandomWalk(step)


def _tempered(t, prior, tgt=None):
    pr = None
    if prior is not None:
        pr = TG.DiagGaussian(len(prior["mean"]), mean=prior["mean"], inv_var=prior["inv_var"], const=prior["const"])
    tgt = _target(t) if tgt is None else tgt
    return TemperedPDF(tgt, pr, n_dims=tgt.n_dim)


def _f32(a):
    return torch.tensor(np.asarray(a), dtype=torch.float32, device="cuda")


def _check_pt(case_kind, t, x0, noise, unif, u_ex, temps, step, nlf, prior, ref, tgt=None):
    """CUDA tempered steps + exchange + adaptation vs `ref` = dict of expected
    arrays, with accept decisions compared on the rows free of near-ties."""
    from flowmc_gb300.strategy.parallel_tempering import pt_adapt_temperatures, pt_exchange, pt_local_steps
    C, Tn, S, d = noise.shape
    tlp = _tempered(t, prior, tgt)
    kern = _kernel(case_kind, step, nlf)
    acc_count = torch.empty(C, Tn, device="cuda")
    x, lp, _ = pt_local_steps(kern, tlp, _f32(x0), _f32(temps), S, 1, noise=_f32(noise), uniform=_f32(unif),
                              acc_count=acc_count)
    first = torch.empty(C, d, device="cuda")
    rest = torch.empty(C, Tn - 1, d, device="cuda")
    lp2 = torch.empty(C, Tn, device="cuda")
    acc2 = torch.empty(C, Tn - 1, device="cuda")
    _, _, _, pairs = pt_exchange(tlp.target, x, _f32(temps), 2, uniform=_f32(u_ex), out_first=first, out_rest=rest,
                                 out_logp=lp2, out_acc=acc2)
    new_t = pt_adapt_temperatures(_f32(temps), pairs, C)
    torch.cuda.synchronize()
    x, lp, first, rest = x.cpu().numpy(), lp.cpu().numpy(), first.cpu().numpy(), rest.cpu().numpy()
    lp2, acc2, pairs, new_t = lp2.cpu().numpy(), acc2.cpu().numpy(), pairs.cpu().numpy(), new_t.cpu().numpy()
    # near-ties of the tempered steps, from the float64 oracle's margins
    tt = PT.tempered(t, temps, C, prior)
    margins = K.accept_margins(case_kind, tt, x0.reshape(C * Tn, d), noise.reshape(C * Tn, S, d),
                               unif.reshape(C * Tn, S), step_size=step, n_leapfrog=nlf,
                               M=np.eye(d) if case_kind == "hmc" else None).reshape(C, Tn, S)
    clean = ~(margins < 1e-4).any(axis=2)                     # rows with no near-tie
    np.testing.assert_allclose(x[clean], ref["ens_x"][clean], rtol=1e-5, atol=1e-5)
    np.testing.assert_allclose(lp[clean], ref["ens_lp"][clean], rtol=1e-5,
                               atol=1e-5 * max(1.0, np.abs(ref["ens_lp"]).max()))
    np.testing.assert_array_equal(acc_count.cpu().numpy()[clean], ref["ens_acc"].sum(axis=2)[clean])
    chains = clean.all(axis=1)
    # the exchange of the chains whose steps agree, from the oracle on the CUDA positions
    xo, lpo, acco = PT.exchange(t, x.astype(np.float64), temps, u_ex)
    np.testing.assert_array_equal(acc2[chains], acco[chains])
    np.testing.assert_allclose(first[chains], xo[chains, 0], rtol=0, atol=0)
    np.testing.assert_allclose(rest[chains], xo[chains, 1:], rtol=0, atol=0)
    np.testing.assert_allclose(lp2[chains], lpo[chains], rtol=1e-5, atol=1e-5 * max(1.0, np.abs(lpo).max()))
    np.testing.assert_array_equal(pairs[: Tn - 1], acc2.sum(axis=0))
    np.testing.assert_allclose(new_t, PT.adapt_temperature(temps, acc2), rtol=2e-6)
    return chains, acc2


@pytest.mark.gpu
@pytest.mark.parametrize("case", _pt_cases(), ids=lambda c: c["name"])
def test_cuda_parallel_tempering_matches_reference_source(cuda, case):
    z, _ = _load()
    n = case["name"]
    ref = {k: z[f"{n}/{k}"] for k in ("ens_x", "ens_lp", "ens_acc", "ex_x", "ex_lp", "ex_acc", "new_temps")}
    chains, acc2 = _check_pt(case["local"], case["target"], z[f"{n}/x0"], z[f"{n}/noise"], z[f"{n}/unif"],
                             z[f"{n}/u_exchange"], z[f"{n}/temps"], case["step_size"], case["n_leapfrog"],
                             case.get("prior"), ref)
    assert chains.all()
    np.testing.assert_array_equal(acc2, ref["ex_acc"])


@pytest.mark.gpu
@pytest.mark.parametrize("kind,tname,step,nlf", [("mala", "mixture", 0.3, 0), ("grw", "mixture", 0.5, 0),
                                                  ("hmc", "diag", 0.1, 3), ("mala", "rosen", 0.05, 0)])
def test_cuda_parallel_tempering_matches_oracle(cuda, kind, tname, step, nlf):
    rng = np.random.default_rng(11)
    C, Tn, S = 40, 5, 12
    if tname == "mixture":
        d = 6
        tgt = TG.GaussianMixture(rng.normal(size=(3, d)) * 3, np.full((3, d), 1 / 1.5), [0.2, 0.3, 0.5])
    elif tname == "diag":
        d = 20
        tgt = TG.DiagGaussian(d, mean=rng.normal(size=d), inv_var=rng.uniform(0.5, 2, size=d))
    else:
        d = 9
        tgt = TG.Rosenbrock(d)
    t = tgt.describe()
    temps = np.geomspace(1.0, 12.0, Tn)
    x0 = rng.normal(size=(C, Tn, d)) * (0.3 if tname == "rosen" else 1.0)
    noise = rng.normal(size=(C, Tn, S, d))
    unif = rng.uniform(1e-6, 1.0, size=(C, Tn, S))
    u_ex = rng.uniform(1e-6, 1.0, size=(C, Tn - 1))
    M = np.eye(d) if kind == "hmc" else None
    ex, elp, eacc = PT.ensemble_step(kind, t, x0, temps, S, noise, unif, step_size=step, n_leapfrog=nlf, M=M)
    ref = {"ens_x": ex, "ens_lp": elp, "ens_acc": eacc}
    chains, _ = _check_pt(kind, t, x0, noise, unif, u_ex, temps, step, nlf, None, ref, tgt=tgt)
    assert chains.mean() > 0.8


@pytest.mark.gpu
def test_cuda_tempered_gaussian_variances(cuda):
    """In-kernel Philox: MALA on a diagonal Gaussian at temperature T samples
    N(m, T / inv_var) (tempered_log_pdf = log L / T)."""
    from flowmc_gb300.resource.kernel.MALA import MALA
    from flowmc_gb300.strategy.parallel_tempering import pt_local_steps
    d, C, temps = 4, 8192, [1.0, 2.0, 4.0, 9.0]
    iv = np.array([1.0, 2.0, 0.5, 4.0])
    tlp = TemperedPDF(TG.DiagGaussian(d, mean=np.zeros(d), inv_var=iv), None, n_dims=d)
    x = torch.zeros(C, len(temps), d, device="cuda")
    x, _, _ = pt_local_steps(MALA(0.35), tlp, x, _f32(temps), 600, 123)
    var = x.var(dim=0).cpu().numpy()                      # [T, d]
    expect = np.outer(temps, 1.0 / iv)
    # MALA at a finite step has O(dt^2) bias; 8192 chains give about 2-3 % noise
    np.testing.assert_allclose(var, expect, rtol=0.12)


@pytest.mark.gpu
def test_cuda_exchange_equal_temperatures_rotates(cuda):
    """Equal temperatures give a zero log ratio, so (with in-kernel uniforms
    in (0, 1)) every swap is taken and the sweep moves row 0 to the end."""
    from flowmc_gb300.strategy.parallel_tempering import pt_exchange
    C, Tn, d = 1000, 5, 7
    tgt = TG.DiagGaussian(d)
    x = torch.randn(C, Tn, d, device="cuda")
    first = torch.empty(C, d, device="cuda")
    rest = torch.empty(C, Tn - 1, d, device="cuda")
    acc = torch.empty(C, Tn - 1, device="cuda")
    _, _, _, pairs = pt_exchange(tgt, x, torch.ones(Tn, device="cuda"), 5, out_first=first, out_rest=rest,
                                 out_acc=acc)
    torch.cuda.synchronize()
    # u = 1 has probability 2^-24 per draw: allow none here
    assert int(pairs.sum()) == C * (Tn - 1) and bool((acc == 1).all())
    torch.testing.assert_close(first, x[:, 1])
    torch.testing.assert_close(rest, torch.cat([x[:, 2:], x[:, :1]], dim=1))


@pytest.mark.gpu
def test_cuda_exchange_swap_rate(cuda):
    """Two temperatures on a Gaussian with positions drawn from the tempered
    marginals: the Philox swap rate equals E[min(1, exp(ratio))] computed
    from the same positions."""
    from flowmc_gb300.strategy.parallel_tempering import pt_exchange
    C, d = 200000, 3
    temps = np.array([1.0, 3.0])
    g = torch.Generator(device="cuda").manual_seed(3)
    x = torch.randn(C, 2, d, device="cuda", generator=g) * _f32(np.sqrt(temps))[None, :, None]
    tgt = TG.DiagGaussian(d)
    _, lp, _, pairs = pt_exchange(tgt, x, _f32(temps), 9, out_logp=torch.empty(C, 2, device="cuda"))
    xs = x.double().cpu().numpy()
    l0, l1 = -0.5 * (xs[:, 0] ** 2).sum(1), -0.5 * (xs[:, 1] ** 2).sum(1)
    p = np.minimum(1.0, np.exp((1 / temps[1] - 1 / temps[0]) * (l0 - l1))).mean()
    rate = int(pairs[0]) / C
    assert abs(rate - p) < 4 * np.sqrt(p * (1 - p) / C) + 1e-4


@pytest.mark.gpu
def test_cuda_adapt_in_place_and_counts(cuda):
    from flowmc_gb300.strategy.parallel_tempering import pt_adapt_temperatures
    z, _ = _load()
    temps, flags = z["pt_adapt/temps"], z["pt_adapt/flags"]
    t = _f32(temps)
    pairs = torch.tensor(flags.sum(axis=0).astype(np.int32), device="cuda")
    pt_adapt_temperatures(t, pairs, flags.shape[0], out=t)
    torch.testing.assert_close(t.cpu().double(), torch.tensor(z["pt_adapt/new_temps"]), rtol=2e-6, atol=0)


@pytest.mark.gpu
def test_pt_bundle_runs_end_to_end(cuda):
    """The PT bundle on the 5-D dual moon (the reference's PT example target),
    shortened: buffers filled and finite, tempered chains moved off their
    start, temperatures adapted with the end points fixed."""
    from flowmc_gb300.Sampler import Sampler
    d, C = 5, 64
    key, sub = split(PRNGKey(1))
    b = RQSpline_MALA_PT_Bundle(sub, C, d, TG.DualMoon(d), 20, 20, 3, 2, 3, mala_step_size=0.1,
                                rq_spline_hidden_units=[16, 16], rq_spline_n_bins=8, rq_spline_n_layers=2,
                                n_temperatures=4, max_temperature=5.0, device="cuda")
    s = Sampler(d, C, key, resource_strategy_bundles=b)
    x0 = torch.randn(C, d, device="cuda")
    t0 = b.resources["temperatures"].data.clone()
    out = s.sample(x0, {})
    torch.cuda.synchronize()
    for name in ("positions_training", "positions_production", "log_prob_production"):
        assert torch.isfinite(b.resources[name].data).all(), name
    tp = b.resources["tempered_positions"].data
    assert torch.isfinite(tp).all() and not torch.equal(tp, x0[:, None].expand_as(tp))
    t1 = b.resources["temperatures"].data
    assert torch.isfinite(t1).all() and float(t1[0]) == 1.0 and float(t1[-1]) == 5.0
    assert not torch.equal(t0, t1)
    assert out.shape == (C, d) and torch.isfinite(out).all()


@pytest.mark.gpu
def test_pt_strategy_keeps_buffers_outside_training(cuda):
    """parallel_tempering.py:123-132: with the state's training flag off the
    tempered positions and temperatures stay as they were."""
    from flowmc_gb300.resource.buffers import Buffer
    from flowmc_gb300.resource.kernel.MALA import MALA
    from flowmc_gb300.resource.states import State
    from flowmc_gb300.strategy.parallel_tempering import ParallelTempering
    d, C, Tn = 3, 16, 3
    tp = Buffer("tempered_positions", (C, Tn - 1, d), 2)
    tp.data.normal_()
    temps = Buffer("temperature", (Tn,), 0)
    temps.update_buffer(torch.tensor([1.0, 2.0, 4.0]))
    res = {"tempered_logpdf": TemperedPDF(TG.DiagGaussian(d), None, n_dims=d), "local_sampler": MALA(0.3),
           "tempered_positions": tp, "temperatures": temps, "sampler_state": State({"training": False})}
    strat = ParallelTempering(5, "tempered_logpdf", "local_sampler", ["tempered_positions", "temperatures"],
                              "sampler_state")
    tp0, t0 = tp.data.clone(), temps.data.clone()
    _, _, out = strat(PRNGKey(0), res, torch.zeros(C, d, device="cuda"), {})
    torch.cuda.synchronize()
    assert torch.equal(tp.data, tp0) and torch.equal(temps.data, t0)
    assert out.shape == (C, d) and torch.isfinite(out).all()
    res["sampler_state"] = State({"training": True})
    strat(PRNGKey(1), res, out, {})
    torch.cuda.synchronize()
    assert not torch.equal(tp.data, tp0)


@pytest.mark.gpu
def test_pt_edge_cases(cuda):
    """One temperature (nothing to exchange, the adaptation is the identity),
    two temperatures (the adaptation keeps both ends), zero chains, and
    argument checks that the library reports instead of faulting."""
    from flowmc_gb300 import _lib
    from flowmc_gb300.resource.kernel.MALA import MALA
    from flowmc_gb300.strategy.parallel_tempering import pt_adapt_temperatures, pt_exchange, pt_local_steps
    d = 3
    tgt = TG.DiagGaussian(d)
    tlp = TemperedPDF(tgt, None, n_dims=d)
    x = torch.randn(16, 1, d, device="cuda")
    xl, lp, _ = pt_local_steps(MALA(0.3), tlp, x, torch.ones(1, device="cuda"), 5, 1)
    first = torch.empty(16, d, device="cuda")
    _, _, _, pairs = pt_exchange(tgt, xl, torch.ones(1, device="cuda"), 2, out_first=first)
    torch.cuda.synchronize()
    torch.testing.assert_close(first, xl[:, 0])
    t2 = torch.tensor([1.0, 4.0], device="cuda")
    out = pt_adapt_temperatures(t2, torch.tensor([7], dtype=torch.int32, device="cuda"), 16)
    torch.testing.assert_close(out, t2)
    # zero chains: a no-op that still zeroes the swap counts
    z = torch.empty(0, 3, d, device="cuda")
    _, _, _, pz = pt_exchange(tgt, z, torch.ones(3, device="cuda"), 2, out_first=torch.empty(0, d, device="cuda"),
                              acc_pairs=torch.full((2,), 5, dtype=torch.int32, device="cuda"))
    assert pz.tolist() == [0, 0]
    with pytest.raises(_lib.FlowMCError, match="n_temps"):
        pt_local_steps(MALA(0.3), tlp, torch.randn(4, 65, d, device="cuda"), torch.ones(65, device="cuda"), 2, 1)
    with pytest.raises(ValueError):
        pt_local_steps(MALA(0.3), tlp, torch.randn(4, 2, d + 1, device="cuda"), torch.ones(2, device="cuda"), 2, 1)
