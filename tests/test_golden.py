"""Golden vectors produced by the reference's own source (tests/golden/make_golden.py:
flowMC's MALA, HMC and GaussianRandomWalk kernels and its RQSpline, run on
scripted normals and uniforms). The oracle must reproduce them in float64;
the CUDA kernels, fed the same draws, must reproduce them within the float32
trajectory tolerance (1e-5 relative) with identical accept decisions up to
the first near-tie."""
import json
import os

import numpy as np
import pytest

from oracle import flow as F
from oracle import kernels as K

GOLD = os.path.join(os.path.dirname(__file__), "golden", "reference_vectors.npz")


def _load():
    z = np.load(GOLD)
    return z, json.loads(str(z["cases"]))


def _kernel_cases():
    _, cases = _load()
    return [c for c in cases if c["kind"] in ("mala", "hmc", "grw")]


def _spline_cases():
    _, cases = _load()
    return [c for c in cases if c["kind"] == "rqspline"]


@pytest.mark.parametrize("case", _kernel_cases(), ids=lambda c: c["name"])
def test_oracle_kernels_match_reference_source(case):
    z, _ = _load()
    n = case["name"]
    x0, noise, unif = z[f"{n}/x0"], z[f"{n}/noise"], z[f"{n}/unif"]
    M = z[f"{n}/M"] if f"{n}/M" in z else None
    pos, lps, accs, _ = K.take_serial_steps(case["kind"], case["target"], x0, noise.shape[1], noise, unif,
                                            step_size=case["step_size"], n_leapfrog=case["n_leapfrog"], M=M)
    np.testing.assert_array_equal(accs, z[f"{n}/acc"])
    np.testing.assert_allclose(pos, z[f"{n}/pos"], rtol=1e-9, atol=1e-10)
    np.testing.assert_allclose(lps, z[f"{n}/logp"], rtol=1e-9, atol=1e-10)
    assert 0 < z[f"{n}/acc"].mean() < 1 or case["kind"] == "hmc"


@pytest.mark.parametrize("case", _spline_cases(), ids=lambda c: c["name"])
def test_oracle_spline_matches_reference_source(case):
    z, _ = _load()
    n = case["name"]
    raw, x = z[f"{n}/raw"], z[f"{n}/x"]
    xp, yp, sl = F.spline_params(raw, case["n_bins"])
    y, ld = F.rqs_forward(x, xp, yp, sl)
    np.testing.assert_allclose(y, z[f"{n}/fwd_y"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(ld, z[f"{n}/fwd_logdet"], rtol=1e-12, atol=1e-12)
    xi, ldi = F.rqs_inverse(x, xp, yp, sl)
    np.testing.assert_allclose(xi, z[f"{n}/inv_x"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(ldi, z[f"{n}/inv_logdet"], rtol=1e-12, atol=1e-12)
    # the fixture covers both linear tails and the interior
    assert (x < -10).any() and (x > 10).any() and (np.abs(x) < 10).any()


@pytest.mark.gpu
@pytest.mark.parametrize("case", _kernel_cases(), ids=lambda c: c["name"])
def test_cuda_kernels_match_reference_source(cuda, case):
    import torch
    from flowmc_gb300 import targets as TG
    from flowmc_gb300.resource.kernel.Gaussian_random_walk import GaussianRandomWalk
    from flowmc_gb300.resource.kernel.HMC import HMC
    from flowmc_gb300.resource.kernel.MALA import MALA
    from flowmc_gb300.resource.kernel.base import run_local_steps
    z, _ = _load()
    n, t = case["name"], case["target"]
    x0, noise, unif = z[f"{n}/x0"], z[f"{n}/noise"], z[f"{n}/unif"]
    if t["kind"] == "dual_moon":
        tgt = TG.DualMoon(t["n_dim"], r0=t["r0"], sr=t["sr"], mu=t["mu"], s0=t["s0"])
    elif t["kind"] == "rosenbrock":
        tgt = TG.Rosenbrock(t["n_dim"], a=t["a"], b=t["b"], c=t["c"])
    else:
        tgt = TG.DiagGaussian(t["n_dim"], mean=t["mean"], inv_var=t["inv_var"], const=t["const"])
    if case["kind"] == "mala":
        kern = MALA(case["step_size"])
    elif case["kind"] == "hmc":
        kern = HMC(condition_matrix=z[f"{n}/M"], step_size=case["step_size"], n_leapfrog=case["n_leapfrog"])
    else:
        kern = GaussianRandomWalk(case["step_size"])
    C, S, d = noise.shape
    dev = torch.device("cuda")
    pos = torch.full((C, S, d), -np.inf, device=dev)
    lp = torch.full((C, S), -np.inf, device=dev)
    acc = torch.full((C, S), -np.inf, device=dev)
    f32 = lambda a: torch.tensor(a, dtype=torch.float32, device=dev)
    run_local_steps(kern, tgt, f32(x0), S, 1, 1, 0, pos, lp, acc, 0, noise=f32(noise), uniform=f32(unif))
    torch.cuda.synchronize()
    pos, lp, acc = pos.cpu().numpy(), lp.cpu().numpy(), acc.cpu().numpy()
    # near-ties: where the float64 reference's |log u - log ratio| is tiny, float32 may decide either way
    margins = K.accept_margins(case["kind"], t, x0, noise, unif, step_size=case["step_size"],
                               n_leapfrog=case["n_leapfrog"], M=z[f"{n}/M"] if f"{n}/M" in z else None)
    for c in range(C):
        ties = np.nonzero(margins[c] < 1e-4)[0]
        upto = ties[0] if len(ties) else S
        np.testing.assert_array_equal(acc[c, :upto], z[f"{n}/acc"][c, :upto], err_msg=f"chain {c}")
        np.testing.assert_allclose(pos[c, :upto], z[f"{n}/pos"][c, :upto], rtol=1e-5, atol=1e-5, err_msg=f"chain {c}")
        np.testing.assert_allclose(lp[c, :upto], z[f"{n}/logp"][c, :upto], rtol=1e-5,
                                   atol=1e-5 * max(1.0, np.abs(z[f"{n}/logp"][c]).max()), err_msg=f"chain {c}")


def _flow_cases():
    _, cases = _load()
    return [c for c in cases if c["kind"] == "rqsflow"]


def _flow_layers(z, case):
    """The fixture's weights as the oracle's reference-layout layer list."""
    n, d = case["name"], case["n_dim"]
    nlin = len(case["hidden"]) + 1
    return [{"W": [z[f"{n}/W{l}_{i}"] for i in range(nlin)], "b": [z[f"{n}/b{l}_{i}"] for i in range(nlin)],
             "scale": float(z[f"{n}/scale"][l]), "shift": float(z[f"{n}/shift"][l]),
             "mask": ((np.arange(d) + l) % 2).astype(bool)} for l in range(case["n_layers"])]


@pytest.mark.parametrize("case", _flow_cases(), ids=lambda c: c["name"])
def test_oracle_flow_matches_reference_source(case):
    """The whole MaskedCouplingRQSpline (rqSpline.py:450-504) run by the
    reference's own forward / inverse / log_prob: ScalarAffine with non-zero
    scale and shift, tanh conditioners, masks, standardisation, base Gaussian."""
    z, _ = _load()
    n = case["name"]
    fl = F.Flow(_flow_layers(z, case), case["n_bins"], z[f"{n}/mean"], np.diag(z[f"{n}/var"]))
    x = z[f"{n}/x"]
    y, ld = fl.forward(x)
    np.testing.assert_allclose(y, z[f"{n}/fwd_y"], rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(ld, z[f"{n}/fwd_logdet"], rtol=1e-10, atol=1e-10)
    xi, ldi = fl.inverse(x)
    np.testing.assert_allclose(xi, z[f"{n}/inv_x"], rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(ldi, z[f"{n}/inv_logdet"], rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(fl.log_prob(x), z[f"{n}/log_prob"], rtol=1e-10, atol=1e-10)


@pytest.mark.gpu
@pytest.mark.parametrize("case", _flow_cases(), ids=lambda c: c["name"])
def test_cuda_flow_matches_reference_source(cuda, case):
    """The FP32 flow kernels on the reference's own MaskedCouplingRQSpline
    outputs: forward, inverse and log_prob within 1e-4 (relative to
    max(1, |value|))."""
    import torch
    from flowmc_gb300.random import PRNGKey
    from flowmc_gb300.resource.model.nf_model.rqSpline import MaskedCouplingRQSpline
    z, _ = _load()
    n, d = case["name"], case["n_dim"]
    m = MaskedCouplingRQSpline(d, case["n_layers"], case["hidden"], case["n_bins"], PRNGKey(0), device="cuda")
    m.load_full(_flow_layers(z, case))
    m.aux[:d] = torch.tensor(z[f"{n}/mean"], dtype=torch.float32)
    m.aux[d:2 * d] = torch.tensor(z[f"{n}/var"], dtype=torch.float32)
    m.check_layout()
    xt = torch.tensor(z[f"{n}/x"], dtype=torch.float32, device="cuda")

    def close(got, ref):
        np.testing.assert_allclose(got.cpu().numpy(), ref, rtol=1e-4, atol=1e-4 * max(1.0, float(np.abs(ref).max())))

    y, ld = m.forward(xt)
    close(y, z[f"{n}/fwd_y"])
    close(ld, z[f"{n}/fwd_logdet"])
    xi, ldi = m.inverse(xt)
    close(xi, z[f"{n}/inv_x"])
    close(ldi, z[f"{n}/inv_logdet"])
    close(m.log_prob(xt), z[f"{n}/log_prob"])


def _loss_cases():
    _, cases = _load()
    return [c for c in cases if c["kind"] == "nfloss"]


@pytest.mark.parametrize("case", _loss_cases(), ids=lambda c: c["name"])
def test_oracle_loss_gradient_matches_reference_source(case):
    """NFModel.loss_fn (nf_model/base.py:98-100) run by the reference's own
    code, differentiated with respect to every trainable leaf: the oracle's
    loss and gradient (float64 autograd of the restated log_prob) agree to
    1e-10."""
    from oracle import flow_torch as FT
    z, _ = _load()
    n = case["name"]
    fl = F.Flow(_flow_layers(z, case), case["n_bins"], z[f"{n}/mean"], np.diag(z[f"{n}/var"]))
    loss, grad = FT.loss_and_grad(fl, z[f"{n}/x"])
    assert abs(loss - float(z[f"{n}/loss"])) <= 1e-10 * max(1.0, abs(loss))
    np.testing.assert_allclose(grad, z[f"{n}/grad"], rtol=1e-9, atol=1e-10 * np.abs(z[f"{n}/grad"]).max())


@pytest.mark.gpu
@pytest.mark.parametrize("case", _loss_cases(), ids=lambda c: c["name"])
def test_cuda_loss_gradient_matches_reference_source(cuda, case):
    """The hand-written FP32 backward (fmc_flow_loss_grad) against the
    reference's own loss_fn gradient: loss within 1e-4 relative, every
    gradient entry within 1e-4 of the largest."""
    import torch
    from flowmc_gb300.random import PRNGKey
    from flowmc_gb300.resource.model.nf_model.rqSpline import MaskedCouplingRQSpline
    from test_flow_gpu import gpu_grad_to_full
    z, _ = _load()
    n, d = case["name"], case["n_dim"]
    m = MaskedCouplingRQSpline(d, case["n_layers"], case["hidden"], case["n_bins"], PRNGKey(0), device="cuda")
    m.load_full(_flow_layers(z, case))
    m.aux[:d] = torch.tensor(z[f"{n}/mean"], dtype=torch.float32)
    m.aux[d:2 * d] = torch.tensor(z[f"{n}/var"], dtype=torch.float32)
    m.check_layout()
    loss, grad = m.loss_and_grad(torch.tensor(z[f"{n}/x"], dtype=torch.float32, device="cuda"))
    ref = float(z[f"{n}/loss"])
    assert abs(loss.item() - ref) <= 1e-4 * max(1.0, abs(ref))
    g = gpu_grad_to_full(m, grad)
    gref = z[f"{n}/grad"]
    np.testing.assert_allclose(g, gref, rtol=0, atol=1e-4 * np.abs(gref).max())


def _nfprop_cases():
    _, cases = _load()
    return [c for c in cases if c["kind"] == "nfproposal"]


@pytest.mark.parametrize("case", _nfprop_cases(), ids=lambda c: c["name"])
def test_oracle_nf_proposal_matches_reference_source(case):
    """The reference's NFProposal.kernel (NF_proposal.py:27-172) per chain,
    including sample_flow's batched scan and the chunked target evaluation:
    fed the same base normals (the rows the proposals use) and uniforms, the
    oracle's whole-batch global step gives the same accepts, positions and
    log-densities."""
    z, _ = _load()
    n = case["name"]
    fl = F.Flow(_flow_layers(z, case), case["n_bins"], z[f"{n}/mean"], np.diag(z[f"{n}/var"]))
    pos, lp, acc = K.nf_proposal_kernel(fl, case["target"], z[f"{n}/x0"], z[f"{n}/z"], z[f"{n}/unif"])
    np.testing.assert_array_equal(acc, z[f"{n}/acc"])
    np.testing.assert_allclose(pos, z[f"{n}/pos"], rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(lp, z[f"{n}/logp"], rtol=1e-10, atol=1e-10)
    assert 0 < z[f"{n}/acc"].mean() < 1


def _takesteps_cases():
    _, cases = _load()
    return [c for c in cases if c["kind"] == "takesteps"]


@pytest.mark.parametrize("case", _takesteps_cases(), ids=lambda c: c["name"])
def test_oracle_take_steps_buffers_match_reference_source(case):
    """The reference's TakeSerialSteps.__call__ and Buffer.update_buffer over
    several calls with thinning: rows written per call (ceil(S / thinning)),
    the cursor advanced by S // thinning, the clamped start of the last call,
    and the returned last positions."""
    z, _ = _load()
    n = case["name"]
    S, thin, R = case["n_steps"], case["thinning"], case["buf_rows"]
    x = z[f"{n}/x0"]
    C, d = x.shape
    pos_buf, lp_buf, acc_buf = np.full((C, R, d), -np.inf), np.full((C, R), -np.inf), np.full((C, R), -np.inf)
    cursor = 0
    for k in range(case["n_calls"]):
        pos, lps, accs, x = K.take_serial_steps(case["local"], case["target"], x, S, z[f"{n}/noise"][k],
                                                z[f"{n}/unif"][k], step_size=case["step_size"], thinning=thin)
        pos_buf = K.buffer_update(pos_buf, pos, cursor, 1)
        lp_buf = K.buffer_update(lp_buf, lps, cursor, 1)
        acc_buf = K.buffer_update(acc_buf, accs, cursor, 1)
        cursor += S // thin
        assert cursor == z[f"{n}/cursor"][k]
        np.testing.assert_allclose(x, z[f"{n}/last"][k], rtol=1e-10, atol=1e-10)
    np.testing.assert_array_equal(acc_buf, z[f"{n}/acc_buf"])
    np.testing.assert_allclose(pos_buf, z[f"{n}/pos_buf"], rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(lp_buf, z[f"{n}/logp_buf"], rtol=1e-10, atol=1e-10)


def test_oracle_training_selection_matches_reference_source():
    """TrainModel.__call__'s selection (train_model.py:66-80) run by the
    reference on a buffer with unfilled rows: finite rows per chain, the last
    history_window of them, then the scripted choice indices."""
    from oracle import flow as OF
    z, cases = _load()
    case = next(c for c in cases if c["kind"] == "train_select")
    n = case["name"]
    got = OF.select_training_data(z[f"{n}/buf"], case["history_window"], z[f"{n}/choice"])
    np.testing.assert_array_equal(got, z[f"{n}/selected"])
