"""tcgen05 BF16 GEMM (fmc_tc_gemm_bf16) against a plain PyTorch FP32
reference of the same op: C = epi(A B^T + bias) on bf16-rounded A and B.
Tolerance: 2e-3 relative to the largest |C| (FP32 accumulation order) for the
fp32 epilogue; bf16 output rounding (2^-8) for the tanh epilogue."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def run(M, K, N, epi, seed=0):
    from flowmc_gb300 import _lib
    g = torch.Generator(device="cpu").manual_seed(seed)
    rows_a = -(-M // 128) * 128
    rows_b = -(-N // 256) * 256
    A = torch.zeros(rows_a, K, dtype=torch.bfloat16)
    B = torch.zeros(rows_b, K, dtype=torch.bfloat16)
    A[:M] = (torch.randn(M, K, generator=g) * 0.5).to(torch.bfloat16)
    B[:N] = (torch.randn(N, K, generator=g) / np.sqrt(K)).to(torch.bfloat16)
    bias = torch.randn(N, generator=g) * 0.1
    A, B, bias = A.cuda(), B.cuda(), bias.cuda()
    if epi == 0:
        ldc = -(-N // 64) * 64
        C = torch.full((M, ldc), float("nan"), dtype=torch.bfloat16, device="cuda")
        n_store = ldc
    else:
        ldc = N
        C = torch.full((M, ldc), float("nan"), dtype=torch.float32, device="cuda")
        n_store = N
    _lib.check(_lib.lib().fmc_tc_gemm_bf16(A.data_ptr(), M, rows_a, K, B.data_ptr(), N, rows_b, bias.data_ptr(),
                                           C.data_ptr(), ldc, n_store, epi, _lib.stream_handle()))
    torch.cuda.synchronize()
    assert _lib.device_error() == 0
    ref = A[:M].float() @ B[:N].float().T + bias
    if epi == 0:
        ref = torch.tanh(ref)
        got = C.float()
        assert torch.isfinite(got).all()
        assert (got[:, N:] == 0).all()                      # padding columns are zero
        err = (got[:, :N] - ref).abs().max().item()
        assert err <= 2 ** -7, err
    else:
        err = (C - ref).abs().max().item()
        assert err <= 2e-3 * ref.abs().max().item() + 1e-5, err


@pytest.mark.parametrize("M,K,N", [(128, 64, 128), (300, 64, 256), (1000, 128, 512), (257, 512, 512),
                                   (129, 64, 100), (4096, 512, 4736), (640, 192, 384)])
@pytest.mark.parametrize("epi", [0, 1])
def test_tc_gemm_matches_torch(cuda, M, K, N, epi):
    run(M, K, N, epi, seed=M + K + N)


def test_bounded_wait_expires_and_context_survives(cuda):
    """Failure path of the tcgen05 kernels' mbarrier waits, without a fault:
    a wait on a barrier that nothing completes gives up after about a second
    and reports it; the next GEMM on the same context is still correct."""
    import ctypes
    import time
    from flowmc_gb300 import _lib
    flag = ctypes.c_int32(-1)
    t0 = time.perf_counter()
    _lib.check(_lib.lib().fmc_selftest_bounded_wait(ctypes.byref(flag), _lib.stream_handle()))
    dt = time.perf_counter() - t0
    assert flag.value == 1
    assert 0.5 < dt < 10.0          # one second of wall time, plus launch and copy
    M, K, N = 256, 128, 256
    A = torch.randn(M, K, device="cuda").to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda").to(torch.bfloat16)
    C = torch.empty(M, N, device="cuda")
    bias = torch.zeros(N, device="cuda")
    _lib.check(_lib.lib().fmc_tc_gemm_bf16(A.data_ptr(), M, M, K, B.data_ptr(), N, N, bias.data_ptr(), C.data_ptr(),
                                           N, N, 1, _lib.stream_handle()))
    torch.cuda.synchronize()
    ref = A.float() @ B.float().T
    torch.testing.assert_close(C, ref, rtol=1e-2, atol=1e-2)
    assert _lib.device_error() == 0


def test_raised_error_word_skips_tensor_core_work(cuda):
    """While the device error word is raised (a bounded wait expired earlier
    and nobody cleared it), a tensor-core launch returns at once without
    touching its output; once the word is cleared the same GEMM is correct."""
    import time
    from flowmc_gb300 import _lib
    M, K, N = 512, 256, 256
    A = torch.randn(M, K, device="cuda").to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda").to(torch.bfloat16)
    bias = torch.zeros(N, device="cuda")
    C = torch.full((M, N), float("nan"), device="cuda")
    _lib.check(_lib.lib().fmc_device_error_set(1))
    t0 = time.perf_counter()
    for _ in range(20):
        _lib.check(_lib.lib().fmc_tc_gemm_bf16(A.data_ptr(), M, M, K, B.data_ptr(), N, N, bias.data_ptr(),
                                               C.data_ptr(), N, N, 1, _lib.stream_handle()))
    torch.cuda.synchronize()
    assert time.perf_counter() - t0 < 0.5          # no wait ran out: nothing waited at all
    assert torch.isnan(C).all()
    assert _lib.device_error() == 1                 # read and cleared
    _lib.check(_lib.lib().fmc_tc_gemm_bf16(A.data_ptr(), M, M, K, B.data_ptr(), N, N, bias.data_ptr(),
                                           C.data_ptr(), N, N, 1, _lib.stream_handle()))
    torch.cuda.synchronize()
    torch.testing.assert_close(C, A.float() @ B.float().T, rtol=1e-2, atol=1e-2)
    assert _lib.device_error() == 0


def test_kernel_timing_eager_and_captured(cuda):
    """fmc_kernel_timing_*: an eager launch and a launch captured into a CUDA
    graph (timed on replay) are each counted once, with positive time and
    the GEMM's 2 M N K FLOPs."""
    from flowmc_gb300 import _lib
    M, K, N = 4096, 512, 512
    A = torch.randn(M, K, device="cuda").to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda").to(torch.bfloat16)
    bias = torch.zeros(N, device="cuda")
    C = torch.empty(M, N, device="cuda")

    def gemm():
        _lib.check(_lib.lib().fmc_tc_gemm_bf16(A.data_ptr(), M, M, K, B.data_ptr(), N, N, bias.data_ptr(),
                                               C.data_ptr(), N, N, 1, _lib.stream_handle()))

    gemm()
    torch.cuda.synchronize()
    _lib.kernel_timing(True)
    gemm()
    got = _lib.kernel_timing_read()
    assert got["k_tc_gemm_f32"]["launches"] == 1 and got["k_tc_gemm_f32"]["ms"] > 0
    assert got["k_tc_gemm_f32"]["flops"] == 2.0 * M * N * K
    _lib.kernel_timing(True)
    s = torch.cuda.Stream()
    s.wait_stream(torch.cuda.current_stream())
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        gemm()
    _lib.kernel_timing(False)
    g.replay()
    torch.cuda.synchronize()
    got = _lib.kernel_timing_read()
    assert got["k_tc_gemm_f32"]["launches"] == 1 and got["k_tc_gemm_f32"]["ms"] > 0
    torch.testing.assert_close(C, A.float() @ B.float().T, rtol=1e-2, atol=1e-2)
    _lib.kernel_timing(False)
