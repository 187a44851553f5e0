"""Resource persistence in the reference's formats: Buffer / State .npz
(resource/buffers.py:52-64, resource/states.py:53-63) and the flow's
equinox-serialised .eqx checkpoint (resource/model/nf_model/base.py:92-96)."""
import io

import numpy as np
import pytest
import torch

from flowmc_gb300.random import PRNGKey
from flowmc_gb300.resource.buffers import Buffer
from flowmc_gb300.resource.model.nf_model import eqx_format
from flowmc_gb300.resource.model.nf_model.rqSpline import MaskedCouplingRQSpline
from flowmc_gb300.resource.states import State


def test_buffer_npz_round_trip(tmp_path):
    b = Buffer("positions_training", (3, 4, 2), 1, device="cpu")
    b.update_buffer(torch.arange(12.0).reshape(3, 2, 2), 1)
    b.save_resource(str(tmp_path) + "/")
    path = tmp_path / "positions_training.npz"
    z = np.load(path)
    assert str(z["name"]) == "positions_training"          # the reference's keys
    np.testing.assert_array_equal(z["data"], b.data.numpy())
    r = b.load_resource(str(path))
    assert r.name == "positions_training" and r.shape == (3, 4, 2)
    np.testing.assert_array_equal(r.data.numpy(), b.data.numpy())
    assert np.isinf(r.data.numpy()[:, 0]).all()


def test_state_npz_round_trip(tmp_path):
    s = State({"target_positions": "positions_training", "training": True}, name="sampler_state")
    s.save_resource(str(tmp_path) + "/")
    r = s.load_resource(str(tmp_path / "sampler_state.npz"))
    assert r.name == "sampler_state" and r.data == s.data


def _model(seed, d=5, L=3, H=(16, 8), K=6, **kw):
    return MaskedCouplingRQSpline(d, L, list(H), K, PRNGKey(seed), device="cpu", **kw)


def _full_equal(a, b):
    for la, lb in zip(a.to_full(), b.to_full()):
        assert la["scale"] == lb["scale"] and la["shift"] == lb["shift"]
        for x, y in zip(la["W"] + la["b"], lb["W"] + lb["b"]):
            np.testing.assert_array_equal(x, y)


def test_eqx_record_layout(tmp_path):
    d, L, H, K = 5, 3, (16, 8), 6
    m = _model(0, d, L, H, K, data_mean=torch.arange(5.0), data_cov=torch.diag(torch.arange(1.0, 6.0)))
    m.save_model(str(tmp_path / "flow"))
    recs = eqx_format._records(str(tmp_path / "flow.eqx"))
    P = 3 * K + 1
    shapes = [(), (d,), (d, d), (d,), (d, d), (), (L, d), (L,), (L,), (L, d), (), (), (), (), (),
              (L, H[0], d), (L, H[0]), (L, H[1], H[0]), (L, H[1]), (L, d * P, H[1]), (L, d * P)]
    assert [r.shape for r in recs] == shapes
    assert recs[0].item() == d and recs[5].item() is False and recs[12].item() == K
    assert recs[10].item() == -10.0 and recs[11].item() == 10.0 and recs[13].item() == 1e-4
    np.testing.assert_array_equal(recs[1], np.arange(5.0))
    np.testing.assert_array_equal(recs[2], np.diag(np.arange(1.0, 6.0)))
    np.testing.assert_array_equal(recs[4], np.eye(d))
    assert recs[6].dtype == bool and not recs[6].any()
    np.testing.assert_array_equal(recs[9], (np.arange(d)[None] + np.arange(L)[:, None]) % 2 == 1)
    assert all(r.dtype == np.float32 for i, r in enumerate(recs) if r.ndim and i not in (6, 9))


def test_eqx_round_trip(tmp_path):
    a = _model(0, data_mean=torch.arange(5.0))
    a.theta.add_(torch.randn_like(a.theta) * 0.1)     # scale / shift away from zero
    b = _model(1)
    a.save_model(str(tmp_path / "flow"))
    b.load_model(str(tmp_path / "flow"))
    _full_equal(a, b)
    torch.testing.assert_close(b.aux[: 2 * 5 + 1], a.aux[: 2 * 5 + 1])


def test_eqx_reader_from_documented_layout(tmp_path):
    """A checkpoint assembled record by record from the documented leaf order
    (not by the writer), without the scalar records, loads into the model."""
    d, L, H, K = 4, 2, (8,), 5
    P = 3 * K + 1
    rng = np.random.default_rng(0)
    W0, b0 = rng.normal(size=(L, H[0], d)), rng.normal(size=(L, H[0]))
    W1, b1 = rng.normal(size=(L, d * P, H[0])), rng.normal(size=(L, d * P))
    scale, shift = rng.normal(size=L), rng.normal(size=L)
    masks = ((np.arange(d)[None] + np.arange(L)[:, None]) % 2).astype(bool)
    arrays = [rng.normal(size=d), np.diag(rng.uniform(1, 2, size=d)), np.zeros(d), np.eye(d),
              np.zeros((L, d), bool), scale, shift, masks, W0, b0, W1, b1]
    f = io.BytesIO()
    for a in arrays:
        np.save(f, a.astype(np.float32) if a.dtype != bool else a)
    (tmp_path / "ref.eqx").write_bytes(f.getvalue())
    m = _model(3, d, L, H, K)
    m.load_model(str(tmp_path / "ref"))
    full = m.to_full()
    for l in range(L):
        np.testing.assert_allclose(full[l]["W"][0], W0[l], rtol=1e-7)
        np.testing.assert_allclose(full[l]["W"][1], W1[l], rtol=1e-7)
        np.testing.assert_allclose(full[l]["b"][1], b1[l], rtol=1e-7)
        assert full[l]["scale"] == np.float32(scale[l]) and full[l]["shift"] == np.float32(shift[l])
    np.testing.assert_allclose(m.data_mean.numpy(), arrays[0].astype(np.float32))
    np.testing.assert_allclose(torch.diagonal(m.data_cov).numpy(), np.diag(arrays[1]).astype(np.float32))


def test_eqx_rejects_other_architectures(tmp_path):
    _model(0).save_model(str(tmp_path / "flow"))
    with pytest.raises(ValueError, match="shape"):
        _model(0, H=(16, 16)).load_model(str(tmp_path / "flow"))
    with pytest.raises(ValueError):
        _model(0, L=4).load_model(str(tmp_path / "flow"))
    with pytest.raises(ValueError, match="num_bins|shape"):
        _model(0, K=7).load_model(str(tmp_path / "flow"))


@pytest.mark.gpu
def test_eqx_round_trip_log_prob_on_gpu(cuda, tmp_path):
    d = 6
    a = MaskedCouplingRQSpline(d, 4, [32, 32], 8, PRNGKey(0), device="cuda")
    a.theta.add_(torch.randn_like(a.theta) * 0.05)
    a.sync_bf16()
    b = MaskedCouplingRQSpline(d, 4, [32, 32], 8, PRNGKey(9), device="cuda")
    x = torch.randn(1000, d, device="cuda") * 2
    a.save_model(str(tmp_path / "flow"))
    b.load_model(str(tmp_path / "flow"))
    torch.testing.assert_close(b.log_prob(x), a.log_prob(x), rtol=0, atol=0)
