"""BF16 conditioner flows at the depth and width the sampler runs them, on the
GPU against the float64 oracle, through the C ABI.

Two flow shapes:
  * 128 features, 12 coupling layers, hidden [512, 512], 12 bins (the 128-D
    Rosenbrock workload's flow);
  * 64 features, 8 layers, hidden [256, 256], 8 bins (the 64-D 4-mode
    mixture workload's flow).

Tolerances (BF16 GEMM inputs, FP32 accumulation, FP32 spline):
  * flow log-probs within 2e-2 relative to max(1, |log q|), per row;
  * forward / inverse / sample outputs and log-determinants: per value, the error against
    the float64 oracle stays within 3x the error that BF16 operands alone
    cause (the oracle run with its conditioner inputs, weights and hidden
    activations rounded to bfloat16), in the maximum and in the median.
    At 12 random layers that error exceeds 2e-2 of the output scale in the
    worst coordinates, so the per-coordinate bar is BF16's own, not 2e-2;
  * NFProposal global step (fmc_nf_global_steps, scripted normals and
    uniforms): accept decisions identical to the oracle's at every step of a
    chain up to its first near-tie, where a near-tie is a step whose oracle
    margin |log u - ratio| is below twice the measured error of that step's
    ratio ingredients (flow and target log-densities of its BF16 proposal and
    of the chain's current state against the oracle's); the proposals and their flow
    log-densities within the BF16-operand bar above; accepted positions and
    target log-densities on the compared steps within the proposals' own
    measured error.

Reference: resource/kernel/NF_proposal.py:27-128 (the global step),
resource/model/nf_model/rqSpline.py:450-504 (forward, inverse, sample,
log_prob).
"""
import numpy as np
import pytest
import torch

from oracle import flow as F
from oracle import kernels as K
from oracle import targets as OT
from test_flow_gpu import gpu_model, rand_flow, to_f32

pytestmark = pytest.mark.gpu

BF16_TOL = 2e-2

DEEP = [(128, 12, (512, 512), 12), (64, 8, (256, 256), 8)]

_FLOWS = {}


def deep_flow(d, L, hidden, nb):
    """The oracle flow (float32-rounded parameters), built once per shape."""
    key = (d, L, hidden, nb)
    if key not in _FLOWS:
        _FLOWS[key] = to_f32(rand_flow(d, L, hidden, nb, seed=1000 + d + L, wscale=0.3))
    return _FLOWS[key]


def rel_err(a, ref):
    return np.abs(a - ref) / np.maximum(1.0, np.abs(ref))


def bf16_flow(fl):
    """The same flow with BF16 conditioner operands (oracle.flow.mlp)."""
    return F.Flow(fl.layers, fl.n_bins, fl.data_mean, fl.data_cov, fl.base_cov_scale, bf16=True)


def assert_within_bf16(got, ref, emul, what):
    """|got - ref| within 3x |emul - ref| (BF16 operands alone) in the maximum
    and the median over coordinates."""
    e, b = np.abs(got - ref), np.abs(emul - ref)
    assert e.max() <= 3.0 * b.max() + 1e-4, (what, "max", e.max(), b.max())
    assert np.median(e) <= 3.0 * np.median(b) + 1e-5, (what, "median", np.median(e), np.median(b))


@pytest.mark.parametrize("d,L,hidden,nb", DEEP, ids=[f"d{c[0]}L{c[1]}H{c[2][0]}K{c[3]}" for c in DEEP])
def test_flow_bf16_full_depth_passes(cuda, d, L, hidden, nb):
    """log_prob, forward, inverse and sample of the full-depth BF16 flow."""
    from flowmc_gb300 import _lib
    from flowmc_gb300.random import PRNGKey
    fl = deep_flow(d, L, hidden, nb)
    fb = bf16_flow(fl)
    m = gpu_model(fl, hidden, precision="bf16")
    rng = np.random.default_rng(7)
    x = (rng.normal(size=(400, d)) * 1.5).astype(np.float32)
    x64 = x.astype(np.float64)
    xt = torch.tensor(x, device="cuda")

    lp = m.log_prob(xt).cpu().numpy()
    olp = fl.log_prob(x64)
    assert _lib.device_error() == 0
    assert rel_err(lp, olp).max() <= BF16_TOL, rel_err(lp, olp).max()

    y, ld = m.forward(xt)
    oy, old = fl.forward(x64)
    by, bld = fb.forward(x64)
    assert_within_bf16(y.cpu().numpy(), oy, by, "forward")
    assert_within_bf16(ld.cpu().numpy(), old, bld, "forward log-det")

    xi, ldi = m.inverse(xt)
    oxi, oldi = fl.inverse(x64)
    bxi, bldi = fb.inverse(x64)
    assert_within_bf16(xi.cpu().numpy(), oxi, bxi, "inverse")
    assert_within_bf16(ldi.cpu().numpy(), oldi, bldi, "inverse log-det")

    z = rng.normal(size=(400, d)).astype(np.float32)
    s = m.sample(PRNGKey(1), 400, z=torch.tensor(z, device="cuda")).cpu().numpy()
    z64 = z.astype(np.float64)
    assert_within_bf16(s, fl.sample(z64), fb.sample(z64), "sample")


def _target(kind, d, fl, fit):
    """diag: a diagonal Gaussian fitted to flow samples `fit` (so the flow is a
    fair independent proposal, acceptance about 0.2); mixture: the 64-D
    4-mode mixture's shape (modes +-4 along two orthonormal directions,
    variance 0.5); rosenbrock: the 128-D Rosenbrock chain."""
    from flowmc_gb300 import targets as TG
    if kind == "diag":
        return TG.DiagGaussian(d, fit.mean(0), 1.0 / fit.var(0))
    if kind == "mixture":
        rng = np.random.default_rng(3)
        q, _ = np.linalg.qr(rng.normal(size=(d, d)))
        u1, u2 = q[:, 0], q[:, 1]
        means = np.stack([4 * u1, -4 * u1, 4 * u2, -4 * u2])
        return TG.GaussianMixture(means, np.full((4, d), 0.5))
    return TG.Rosenbrock(d)


GLOBAL = [(128, 12, (512, 512), 12, "diag"), (64, 8, (256, 256), 8, "diag"),
          (128, 12, (512, 512), 12, "rosenbrock"), (64, 8, (256, 256), 8, "mixture")]


@pytest.mark.parametrize("d,L,hidden,nb,kind", GLOBAL, ids=[f"d{c[0]}L{c[1]}-{c[4]}" for c in GLOBAL])
def test_nf_global_step_bf16_full_depth(cuda, d, L, hidden, nb, kind):
    from flowmc_gb300 import _lib
    from flowmc_gb300.random import PRNGKey
    from flowmc_gb300.resource.kernel.NF_proposal import NFProposal
    fl = deep_flow(d, L, hidden, nb)
    m = gpu_model(fl, hidden, precision="bf16")
    C, S = 32, 12
    rng = np.random.default_rng(11)
    # current positions: flow samples (oracle), so that the chains start from
    # typical states of the proposal
    smp = fl.sample(rng.normal(size=(C + 512, d)))
    x0 = smp[:C].astype(np.float32)
    tgt = _target(kind, d, fl, smp[C:])
    t = tgt.describe()
    z = rng.normal(size=(C, S, d)).astype(np.float32)
    u = rng.uniform(1e-6, 1, size=(C, S)).astype(np.float32)
    dev = "cuda"
    pos = torch.full((C, S, d), -np.inf, device=dev)
    lp = torch.full((C, S), -np.inf, device=dev)
    acc = torch.full((C, S), -np.inf, device=dev)
    NFProposal(m).group_steps(5, torch.tensor(x0, device=dev), tgt, S, 1, pos, lp, acc, 0,
                              noise=torch.tensor(z, device=dev), uniform=torch.tensor(u, device=dev))
    torch.cuda.synchronize()
    assert _lib.device_error() == 0
    x064, z64, u64 = x0.astype(np.float64), z.astype(np.float64), u.astype(np.float64)
    ox, olp, oacc, oratio = K.nf_proposal_kernel(fl, t, x064, z64, u64, return_ratio=True)

    # measured error of the ratio's ingredients: the BF16 flow's proposals and
    # their flow / target log-densities against the oracle's
    gs = m.sample(PRNGKey(0), C * S, z=torch.tensor(z.reshape(C * S, d), device=dev))
    glq = m.log_prob(gs).double().cpu().numpy()
    glq0 = m.log_prob(torch.tensor(x0, device=dev)).double().cpu().numpy()
    gs64 = gs.double().cpu().numpy()
    os_ = fl.sample(z64.reshape(C * S, d))
    olq, olq0 = fl.log_prob(os_), fl.log_prob(x064)
    lpt_g, lpt_o = OT.value_grad(t, gs64)[0], OT.value_grad(t, os_)[0]
    # the proposals and their flow log-densities (each at its own proposal)
    # within the error of the same quantities with BF16 operands
    fb = bf16_flow(fl)
    bs_ = fb.sample(z64.reshape(C * S, d))
    assert_within_bf16(gs64, os_, bs_, "proposals")
    assert_within_bf16(glq, olq, fb.log_prob(bs_), "proposal flow log-densities")
    # per step, the error of the ratio's ingredients: the proposal's flow and
    # target log-densities (each at its own BF16 / float64 point) plus those
    # of the current state -- the start, then the last proposal the oracle
    # accepted -- with float32 rounding of the target on top
    err_p = (np.abs(glq - olq) + np.abs(lpt_g - lpt_o) + 1e-5 * np.abs(lpt_o)).reshape(C, S)
    lpt0 = OT.value_grad(t, x064)[0]
    cur = np.abs(glq0 - olq0) + 1e-5 * np.abs(lpt0)
    eps = np.empty((C, S))
    for s_ in range(S):
        eps[:, s_] = err_p[:, s_] + cur
        cur = np.where(oacc[:, s_] > 0.5, err_p[:, s_], cur)
    margin = np.abs(np.log(u64) - oratio)
    near = margin <= 2.0 * eps
    first_tie = np.where(near.any(1), near.argmax(1), S)    # per chain: steps compared = [0, first_tie)
    cmp_mask = np.arange(S)[None, :] < first_tie[:, None]
    g_acc = acc.cpu().numpy()
    np.testing.assert_array_equal(g_acc[cmp_mask], oacc[cmp_mask])
    gx, glp = pos.cpu().numpy(), lp.cpu().numpy()
    # accepted rows are proposals (or the starting rows): within the BF16
    # error of the proposals themselves, and their target log-densities
    # within the target's measured spread over those proposals
    assert np.abs(gx[cmp_mask] - ox[cmp_mask]).max() <= 3.0 * np.abs(bs_ - os_).max() + 1e-4
    lp_tol = 1.5 * np.abs(lpt_g - lpt_o).max() + 1e-5 * np.abs(lpt_o).max() + 1e-4
    assert np.abs(glp[cmp_mask] - olp[cmp_mask]).max() <= lp_tol
    # the comparison is not vacuous: most steps are away from ties, and (for
    # the fitted target, where the flow is a fair proposal) both decisions occur
    assert cmp_mask.mean() >= 0.5, (cmp_mask.mean(), float(np.median(eps)))
    if kind == "diag":
        assert 0.05 <= oacc[cmp_mask].mean() <= 0.95, oacc[cmp_mask].mean()
