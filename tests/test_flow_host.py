"""Host-side flow logic without a GPU: the packed parameter layout agrees
with libflowmc's fmc_flow_layout, and reference-layout parameters round-trip
through the packing."""
import numpy as np
import pytest
import torch

from flowmc_gb300 import _lib
from flowmc_gb300.random import PRNGKey
from flowmc_gb300.resource.model.nf_model.rqSpline import MaskedCouplingRQSpline

needs_lib = pytest.mark.skipif(not _lib.LIB_PATH.exists(), reason="libflowmc.so not built")


@needs_lib
@pytest.mark.parametrize("d,L,hidden,nb", [(2, 3, [16, 16], 8), (5, 4, [32, 32], 8), (7, 2, [9], 4),
                                           (128, 12, [512, 512], 12), (33, 5, [8, 8, 8], 3)])
def test_layout_matches_library(d, L, hidden, nb):
    m = MaskedCouplingRQSpline(d, L, hidden, nb, PRNGKey(0), device="cpu")
    m.check_layout()


def test_full_roundtrip_and_masks():
    m = MaskedCouplingRQSpline(5, 3, [6, 7], 4, PRNGKey(3), device="cpu")
    full = m.to_full()
    assert full[0]["W"][0].shape == (6, 5) and full[0]["W"][-1].shape == (5 * 13, 7)
    assert list(full[0]["mask"]) == [False, True, False, True, False]
    assert list(full[1]["mask"]) == [True, False, True, False, True]
    rng = np.random.default_rng(0)
    for Lr in full:
        Lr["W"] = [rng.normal(size=w.shape).astype(np.float32) for w in Lr["W"]]
        Lr["b"] = [rng.normal(size=b.shape).astype(np.float32) for b in Lr["b"]]
        Lr["scale"], Lr["shift"] = 0.25, -0.5
    m.load_full(full)
    back = m.to_full()
    for a, b in zip(full, back):
        for w1, w2 in zip(a["W"] + a["b"], b["W"] + b["b"]):
            np.testing.assert_array_equal(w1, w2)
        assert b["scale"] == 0.25 and b["shift"] == -0.5


def test_reference_initialisation_statistics():
    m = MaskedCouplingRQSpline(64, 2, [256, 256], 8, PRNGKey(1), device="cpu")
    full = m.to_full()
    W0 = full[0]["W"][0]
    assert abs(W0.std() - np.sqrt(1e-2 / 64)) < 0.1 * np.sqrt(1e-2 / 64)   # N(0, scale/in), scale 1e-2
    Wl = full[0]["W"][-1]
    assert np.abs(Wl).max() <= 1 / np.sqrt(256) + 1e-7                     # Equinox U(-1/sqrt(in), ..)
    assert float(m.aux[2 * 64]) == 1.0
    assert torch.equal(m.data_mean, torch.zeros(64))


@pytest.mark.parametrize("d", [0, 1, 4097])
def test_feature_count_outside_the_supported_range(d):
    with pytest.raises(ValueError, match="2 to 4096 features"):
        MaskedCouplingRQSpline(d, 2, [8, 8], 4, PRNGKey(0), device="cpu")


def _infer_ws_bytes(d, L, hidden, nb, precision, n):
    """fmc_flow_workspace_size (inference) of a flow description; host
    arithmetic only, no device memory is touched."""
    import ctypes
    s = _lib.FmcFlow()
    s.n_dim, s.n_layers, s.n_hidden, s.n_bins = d, L, len(hidden), nb
    for i, h in enumerate(hidden):
        s.hidden[i] = h
    s.range_min, s.range_max, s.min_bin_size, s.min_knot_slope = -10.0, 10.0, 1e-3, 1e-3
    s.precision = precision
    nbytes = ctypes.c_size_t()
    _lib.check(_lib.lib().fmc_flow_workspace_size(ctypes.byref(s), n, 0, ctypes.byref(nbytes)))
    return nbytes.value


@needs_lib
def test_bf16_workspace_keeps_every_layers_logdet_partials():
    """BF16 passes keep each layer's log-det partials (three per 6-coordinate
    group and row for 12 bins: 3 * 11 = 33 for 64 transformed coordinates) in
    the workspace and reduce them once per pass; a flow past 16 layers reduces
    after every layer, so only one layer's partials differ between the two.
    Chunks are 77,824 rows."""
    rows, per_layer = 77824, 3 * ((64 + 5) // 6)
    a = _infer_ws_bytes(128, 12, [512, 512], 12, _lib.PREC_BF16, 200000)
    b = _infer_ws_bytes(128, 17, [512, 512], 12, _lib.PREC_BF16, 200000)
    assert a - b == 4 * rows * per_layer * (12 - 1)
    # a wide flow (1,026 partials per row and layer) never keeps more than one layer's
    assert _infer_ws_bytes(4096, 12, [64, 64], 12, _lib.PREC_BF16, 1000) == \
        _infer_ws_bytes(4096, 2, [64, 64], 12, _lib.PREC_BF16, 1000)
    # the FP32 path reduces inside its spline kernels: no partials at all
    assert _infer_ws_bytes(128, 12, [512, 512], 12, _lib.PREC_FP32, 200000) == \
        _infer_ws_bytes(128, 17, [512, 512], 12, _lib.PREC_FP32, 200000)
