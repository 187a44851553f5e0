"""The allocation-free training-data selection (fmc_select_training_data_noalloc).

It exists for callers that cannot allocate device memory -- code running
inside another framework's allocator or memory pool, or under a
no-allocation policy -- and keeps its scratch in a static device array
instead of a caller workspace. Here it is called through the C ABI and must
reproduce the workspace entry point (fmc_select_training_data) exactly, on
two calls in a row (the second call reuses the static scratch the first left
behind), and, on a third call with scripted choice indices, the rows the
reference's own TrainModel selected (the golden train_select case, made by
tests/golden/make_golden.py from the reference's source). Selection is index
work, so the tolerance is bit-exact. Sizes past its stated maximum
(n_chains * n_steps > 2**20 rows) are refused on the host.
"""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def _select(lib, fn_name, buf, hw, n_out, seed, idx=None):
    from flowmc_gb300 import _lib
    C, S, d = buf.shape
    out = torch.full((n_out, d), float("nan"), device=buf.device)
    err = torch.zeros((), dtype=torch.int32, device=buf.device)
    stream = _lib.stream_handle(buf.device)
    if fn_name == "fmc_select_training_data":
        nb = ctypes.c_size_t()
        _lib.check(lib.fmc_select_workspace_size(C, S, ctypes.byref(nb)))
        ws = torch.empty(nb.value + 256, dtype=torch.uint8, device=buf.device)
        base = ws.data_ptr() + (-ws.data_ptr()) % 256
        _lib.check(lib.fmc_select_training_data(buf.data_ptr(), C, S, d, hw, n_out, seed, 0, _lib.ptr(idx),
                                                out.data_ptr(), err.data_ptr(), base, nb.value, stream))
    else:
        _lib.check(lib.fmc_select_training_data_noalloc(buf.data_ptr(), C, S, d, hw, n_out, seed, 0, _lib.ptr(idx),
                                                        out.data_ptr(), err.data_ptr(), stream))
    torch.cuda.synchronize()
    assert int(err.item()) == 0
    return out.cpu().numpy()


def test_noalloc_selection_matches_workspace_entry_point(cuda):
    from flowmc_gb300 import _lib
    lib = _lib.lib()
    rng = np.random.default_rng(0)
    # two calls in a row on different inputs; the second one is larger, so the
    # static scratch holds the first call's words where the second reads
    cases = [((9, 120, 4), 60, 30, 1000, 11), ((31, 700, 3), 650, 100, 5000, 12)]
    for (C, S, d), filled, hw, n_out, seed in cases:
        buf = np.full((C, S, d), -np.inf, np.float32)
        buf[:, :filled] = rng.normal(size=(C, filled, d))
        tb = torch.tensor(buf, device="cuda")
        ref = _select(lib, "fmc_select_training_data", tb, hw, n_out, seed)
        got = _select(lib, "fmc_select_training_data_noalloc", tb, hw, n_out, seed)
        assert np.isfinite(got).all()
        np.testing.assert_array_equal(got, ref)
    # third call: the reference's own selection (golden vectors)
    from test_golden import _load
    z, gcases = _load()
    case = next(c for c in gcases if c["kind"] == "train_select")
    n = case["name"]
    gbuf = torch.tensor(z[f"{n}/buf"].astype(np.float32), device="cuda")
    choice = torch.tensor(z[f"{n}/choice"].astype(np.int64), device="cuda")
    got = _select(lib, "fmc_select_training_data_noalloc", gbuf, case["history_window"], choice.numel(), 0,
                  idx=choice)
    np.testing.assert_array_equal(got, z[f"{n}/selected"].astype(np.float32))


def test_noalloc_selection_rejects_oversized_buffers(cuda):
    from flowmc_gb300 import _lib
    lib = _lib.lib()
    # 1025 chains x 1024 steps > 2**20 rows: refused before any launch (no memory is touched)
    err = torch.zeros((), dtype=torch.int32, device="cuda")
    out = torch.empty(4, 2, device="cuda")
    rc = lib.fmc_select_training_data_noalloc(out.data_ptr(), 1025, 1024, 2, 10, 4, 0, 0, None, out.data_ptr(),
                                              err.data_ptr(), _lib.stream_handle())
    assert rc == _lib.FMC_ERR_INVALID_ARG
    assert b"exceeds" in lib.fmc_last_error()
