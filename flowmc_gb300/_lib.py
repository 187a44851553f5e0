"""ctypes binding of libflowmc.so (the C ABI declared in include/flowmc.h).

The library is loaded lazily from this package directory. There is no
fallback: if the library is missing or the tensors are not on a CUDA device,
the call raises.
"""
from __future__ import annotations

import ctypes
import threading
from pathlib import Path

import torch

LIB_PATH = Path(__file__).resolve().parent / "libflowmc.so"

FMC_OK = 0
FMC_ERR_INVALID_ARG = 1
FMC_ERR_UNSUPPORTED = 2
FMC_ERR_CUDA = 3
FMC_ERR_TIMEOUT = 4
FMC_ERR_NONFINITE = 5
_STATUS = {1: "INVALID_ARG", 2: "UNSUPPORTED", 3: "CUDA_ERROR", 4: "TIMEOUT", 5: "NONFINITE"}

TARGET_DIAG_GAUSSIAN = 0
TARGET_DUAL_MOON = 1
TARGET_GAUSS_MIXTURE = 2
TARGET_ROSENBROCK = 3
TARGET_DENSE_GAUSSIAN = 4

KERNEL_MALA = 0
KERNEL_HMC = 1
KERNEL_GRW = 2

c_float_p = ctypes.POINTER(ctypes.c_float)


class FmcTarget(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("n_dim", ctypes.c_int32),
        ("n_comp", ctypes.c_int32),
        ("reserved", ctypes.c_int32),
        ("mean", ctypes.c_void_p),
        ("inv_var", ctypes.c_void_p),
        ("log_w", ctypes.c_void_p),
        ("precision", ctypes.c_void_p),
        ("scalars", ctypes.c_float * 8),
    ]


class FmcLocalParams(ctypes.Structure):
    _fields_ = [
        ("kind", ctypes.c_int32),
        ("n_leapfrog", ctypes.c_int32),
        ("step_size", ctypes.c_float),
        ("lanes_per_chain", ctypes.c_int32),
        ("momentum_scale", ctypes.c_void_p),
        ("metric_colsum", ctypes.c_void_p),
        ("momentum_chol", ctypes.c_void_p),
        ("philox_rounds", ctypes.c_int32),
    ]


FMC_MAX_HIDDEN = 4
PREC_FP32 = 0
PREC_BF16 = 1


class FmcFlow(ctypes.Structure):
    _fields_ = [
        ("n_dim", ctypes.c_int32),
        ("n_layers", ctypes.c_int32),
        ("n_hidden", ctypes.c_int32),
        ("n_bins", ctypes.c_int32),
        ("hidden", ctypes.c_int32 * FMC_MAX_HIDDEN),
        ("range_min", ctypes.c_float),
        ("range_max", ctypes.c_float),
        ("min_bin_size", ctypes.c_float),
        ("min_knot_slope", ctypes.c_float),
        ("precision", ctypes.c_int32),
        ("gemm_bn", ctypes.c_int32),
        ("tile_rows", ctypes.c_int32),
        ("gemm_stages", ctypes.c_int32),
        ("wgrad_splits", ctypes.c_int32),
        ("theta", ctypes.c_void_p),
        ("theta_bf16", ctypes.c_void_p),
        ("aux", ctypes.c_void_p),
    ]


class FmcAdamParams(ctypes.Structure):
    _fields_ = [(n, ctypes.c_float) for n in ("lr", "b1", "b2", "eps", "weight_decay", "max_norm")]


class FlowMCError(RuntimeError):
    """A libflowmc entry point returned a non-zero status."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"libflowmc {_STATUS.get(status, status)}: {msg}")
        self.status = status


_lock = threading.Lock()
_lib = None

_SIGNATURES = {
    "fmc_local_steps": (ctypes.c_int, [
        ctypes.POINTER(FmcTarget), ctypes.POINTER(FmcLocalParams), ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64, ctypes.c_uint64,
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fmc_pt_local_steps": (ctypes.c_int, [
        ctypes.POINTER(FmcTarget), ctypes.POINTER(FmcLocalParams), ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_float, ctypes.c_int32, ctypes.c_uint64,
        ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_void_p]),
    "fmc_pt_exchange": (ctypes.c_int, [
        ctypes.POINTER(FmcTarget), ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_uint64,
        ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_void_p]),
    "fmc_pt_adapt_temperatures": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]),
    "fmc_adam_optimize": (ctypes.c_int, [
        ctypes.POINTER(FmcTarget), ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_float, ctypes.c_float,
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_void_p]),
    "fmc_target_value_grad": (ctypes.c_int, [
        ctypes.POINTER(FmcTarget), ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_void_p]),
    "fmc_flow_layout": (ctypes.c_int, [ctypes.POINTER(FmcFlow), ctypes.POINTER(ctypes.c_int64),
                                       ctypes.POINTER(ctypes.c_int64)]),
    "fmc_flow_workspace_size": (ctypes.c_int, [ctypes.POINTER(FmcFlow), ctypes.c_int64, ctypes.c_int32,
                                               ctypes.POINTER(ctypes.c_size_t)]),
    "fmc_flow_sync_bf16": (ctypes.c_int, [ctypes.POINTER(FmcFlow), ctypes.c_void_p]),
    "fmc_flow_bf16_size": (ctypes.c_int, [ctypes.POINTER(FmcFlow), ctypes.POINTER(ctypes.c_int64)]),
    "fmc_tc_gemm_bf16": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
        ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32,
        ctypes.c_void_p]),
    "fmc_device_error": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int32), ctypes.c_int32]),
    "fmc_device_error_set": (ctypes.c_int, [ctypes.c_int32]),
    "fmc_kernel_timing_enable": (ctypes.c_int, [ctypes.c_int32]),
    "fmc_welford_state_size": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(ctypes.c_size_t)]),
    "fmc_welford_reset": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32,
                                         ctypes.c_void_p]),
    "fmc_welford_ess_update": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32,
                                              ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p, ctypes.c_void_p]),
    "fmc_welford_ess_finalize": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                                ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_void_p]),
    "fmc_kernel_grid": (ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(ctypes.c_int32), ctypes.POINTER(ctypes.c_int32)]),
    "fmc_kernel_timing_reset": (ctypes.c_int, []),
    "fmc_kernel_timing_read": (ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(ctypes.c_int64),
                                              ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_double),
                                              ctypes.POINTER(ctypes.c_double)]),
    "fmc_selftest_bounded_wait": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p]),
    "fmc_flow_forward": (ctypes.c_int, [ctypes.POINTER(FmcFlow), ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "fmc_flow_inverse": (ctypes.c_int, [ctypes.POINTER(FmcFlow), ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "fmc_flow_log_prob": (ctypes.c_int, [ctypes.POINTER(FmcFlow), ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                         ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "fmc_flow_sample": (ctypes.c_int, [ctypes.POINTER(FmcFlow), ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p,
                                       ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                       ctypes.c_void_p]),
    "fmc_flow_loss_grad": (ctypes.c_int, [ctypes.POINTER(FmcFlow), ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "fmc_nf_workspace_size": (ctypes.c_int, [ctypes.POINTER(FmcFlow), ctypes.c_int32, ctypes.c_int32,
                                             ctypes.POINTER(ctypes.c_size_t)]),
    "fmc_nf_global_steps": (ctypes.c_int, [
        ctypes.POINTER(FmcFlow), ctypes.POINTER(FmcTarget), ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32,
        ctypes.c_int32, ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "fmc_nf_accept": (ctypes.c_int, [
        ctypes.POINTER(FmcTarget), ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint64,
        ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fmc_adamw_workspace_size": (ctypes.c_int, [ctypes.POINTER(ctypes.c_size_t)]),
    "fmc_adamw_step": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64,
        ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.POINTER(FmcAdamParams), ctypes.c_void_p,
        ctypes.c_size_t, ctypes.c_void_p]),
    "fmc_flag_less": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fmc_copy_if": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t,
                                   ctypes.c_void_p]),
    "fmc_column_stats_workspace_size": (ctypes.c_int, [ctypes.c_int64, ctypes.c_int32,
                                                       ctypes.POINTER(ctypes.c_size_t)]),
    "fmc_column_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]),
    "fmc_permute_rows": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_int32, ctypes.c_uint64,
                                        ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64, ctypes.c_void_p,
                                        ctypes.c_void_p]),
    "fmc_select_workspace_size": (ctypes.c_int, [ctypes.c_int32, ctypes.c_int64, ctypes.POINTER(ctypes.c_size_t)]),
    "fmc_select_training_data": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int64,
        ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
        ctypes.c_size_t, ctypes.c_void_p]),
    "fmc_select_training_data_noalloc": (ctypes.c_int, [
        ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, ctypes.c_int32, ctypes.c_int64,
        ctypes.c_uint64, ctypes.c_uint64, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "fmc_rng_epoch_attach": (ctypes.c_int, [ctypes.c_void_p]),
    "fmc_rng_epoch_advance": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "fmc_last_error": (ctypes.c_char_p, []),
    "fmc_version": (ctypes.c_int, []),
    "fmc_device_sm_count": (ctypes.c_int, [ctypes.POINTER(ctypes.c_int32)]),
    "fmc_launch_count": (ctypes.c_int, [ctypes.POINTER(ctypes.c_uint64)]),
}

EXPORTED = tuple(_SIGNATURES)


def _register(lib, name, restype, argtypes):
    fn = getattr(lib, name)
    fn.restype = restype
    fn.argtypes = argtypes


def lib():
    """The loaded library (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    with _lock:
        if _lib is None:
            if not LIB_PATH.exists():
                raise RuntimeError(
                    f"{LIB_PATH} is missing: build it with `python -m flowmc_gb300.build` "
                    "(there is no CPU fallback)")
            h = ctypes.CDLL(str(LIB_PATH))
            for name, (rt, at) in _SIGNATURES.items():
                _register(h, name, rt, at)
            _lib = h
    return _lib


def register_extra(name: str, restype, argtypes) -> None:
    """Declare another exported entry point (used by sibling modules)."""
    _SIGNATURES[name] = (restype, argtypes)
    global EXPORTED
    EXPORTED = tuple(_SIGNATURES)
    if _lib is not None:
        _register(_lib, name, restype, argtypes)


def check(status: int) -> None:
    if status != FMC_OK:
        msg = lib().fmc_last_error()
        raise FlowMCError(status, msg.decode() if msg else "")


def stream_handle(device: torch.device | None = None) -> int:
    """cudaStream_t of torch's current stream on `device`."""
    return torch.cuda.current_stream(device).cuda_stream


def ptr(t: torch.Tensor | None) -> int | None:
    """Device pointer of a CUDA tensor (None -> NULL); raises for CPU tensors."""
    if t is None:
        return None
    if not t.is_cuda:
        raise RuntimeError("libflowmc takes CUDA tensors only (there is no CPU path)")
    return t.data_ptr()


def require_cuda_f32(t: torch.Tensor, name: str, shape: tuple | None = None) -> torch.Tensor:
    if not isinstance(t, torch.Tensor) or not t.is_cuda:
        raise RuntimeError(f"{name} must be a CUDA tensor (there is no CPU path)")
    if t.dtype != torch.float32:
        raise TypeError(f"{name} must be float32, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if shape is not None and tuple(t.shape) != tuple(shape):
        raise ValueError(f"{name} has shape {tuple(t.shape)}, expected {tuple(shape)}")
    return t


class Workspace:
    """A growable, 256-byte aligned device scratch buffer owned by the caller
    (the library never allocates)."""

    def __init__(self):
        self._buf = None

    def get(self, nbytes: int, device) -> tuple[int, int]:
        nbytes = max(int(nbytes), 256)
        if self._buf is None or self._buf.numel() < nbytes or self._buf.device != torch.device(device):
            self._buf = torch.empty(nbytes + 256, dtype=torch.uint8, device=device)
        base = self._buf.data_ptr()
        off = (-base) % 256
        return base + off, self._buf.numel() - off


def column_stats(x: torch.Tensor, mean: torch.Tensor, var: torch.Tensor, ws: "Workspace") -> None:
    """fmc_column_stats of x [n, d] into mean [d] and var [d], partials in ws."""
    n, d = x.shape
    nb = ctypes.c_size_t()
    check(lib().fmc_column_stats_workspace_size(n, d, ctypes.byref(nb)))
    ptr, size = ws.get(nb.value, x.device)
    check(lib().fmc_column_stats(x.data_ptr(), n, d, mean.data_ptr(), var.data_ptr(), ptr, size,
                                 stream_handle(x.device)))


KERNEL_IDS = {"k_tc_spline_fwd": 0, "k_tc_spline_inv": 1, "k_tc_spline_bwd": 2, "k_tc_gemm_tanh": 3,
              "k_tc_gemm_dtanh": 4, "k_tc_gemm_f32": 5, "k_local_steps": 6, "k_nf_accept": 7}


def kernel_timing(on: bool) -> None:
    """Start (and reset) or stop the library's per-kernel event timing.
    Launches captured into a CUDA graph while it is on are timed when the
    graph is replayed (replay it before kernel_timing_read)."""
    if on:
        check(lib().fmc_kernel_timing_enable(0))
        check(lib().fmc_kernel_timing_reset())
    check(lib().fmc_kernel_timing_enable(1 if on else 0))


def kernel_timing_read() -> dict:
    """{kernel: {launches, ms, flops, bytes}} since the last reset (synchronises)."""
    out = {}
    for name, kid in KERNEL_IDS.items():
        n, ms, fl, by = ctypes.c_int64(), ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        check(lib().fmc_kernel_timing_read(kid, ctypes.byref(n), ctypes.byref(ms), ctypes.byref(fl),
                                           ctypes.byref(by)))
        if n.value:
            out[name] = {"launches": int(n.value), "ms": ms.value, "flops": fl.value, "bytes": by.value}
    return out


def kernel_grid(name: str) -> tuple[int, int]:
    """(CTAs, CTAs per cluster) of the last launch of a timed kernel."""
    a, b = ctypes.c_int32(), ctypes.c_int32()
    check(lib().fmc_kernel_grid(KERNEL_IDS[name], ctypes.byref(a), ctypes.byref(b)))
    return int(a.value), int(b.value)


def launch_count() -> int:
    """Kernels launched by libflowmc so far in this process."""
    v = ctypes.c_uint64()
    check(lib().fmc_launch_count(ctypes.byref(v)))
    return int(v.value)


def device_error(clear: bool = True) -> int:
    """Error word of the tensor-core kernels (1 = a bounded wait expired); synchronous."""
    v = ctypes.c_int32()
    check(lib().fmc_device_error(ctypes.byref(v), 1 if clear else 0))
    return int(v.value)


_epoch_words: dict = {}


def rng_epoch(device=None) -> torch.Tensor:
    """The device word (int64 [1]) every random stream of the library folds
    into its key, created at zero and attached on first use. A CUDA graph
    that runs ``rng_epoch_advance`` draws fresh numbers on every replay."""
    dev = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
    if dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    w = _epoch_words.get(dev)
    if w is None:
        w = torch.zeros(1, dtype=torch.int64, device=dev)
        _epoch_words[dev] = w
    check(lib().fmc_rng_epoch_attach(w.data_ptr()))
    return w


def rng_epoch_advance(word: torch.Tensor) -> None:
    check(lib().fmc_rng_epoch_advance(word.data_ptr(), stream_handle(word.device)))
