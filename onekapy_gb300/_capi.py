"""ctypes binding of liboneka_gb300.so (include/oneka_gb300.h).

The library is the only compute path: importing this module on a machine
without the built library, or calling it without a CUDA device, raises.
There is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import threading

import torch

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "_lib", "liboneka_gb300.so")

ONEKA_OK, ONEKA_ERR_INVALID, ONEKA_ERR_CUDA, ONEKA_ERR_SCRATCH = 0, -1, -2, -3
REAL_OK, REAL_RANGE, REAL_NOT_SPD, REAL_NOT_FINITE = 0, 1, 2, 3
TRACE_OK, TRACE_DRY, TRACE_STEP_LIMIT, TRACE_SKIPPED = 0, 1, 2, 3
DIST_CONST, DIST_UNIFORM, DIST_TRIANGULAR, DIST_LOGNORMAL = 0, 1, 2, 3
MODE_STOCHASTIC, MODE_MEAN, MODE_GIVEN, MODE_GIVEN_EV = 0, 1, 2, 3
FP64, FP32 = 0, 1

EXPORTS = ["oneka_abi_version", "oneka_last_error", "oneka_site_logr2", "oneka_realize",
           "oneka_track_scratch_bytes", "oneka_track", "oneka_evaluate", "oneka_rasterize",
           "oneka_register_weighted", "oneka_distancesquared", "oneka_fma_peak",
           "oneka_track_noalloc", "oneka_track_batched", "oneka_track_batched_scratch_bytes",
           "oneka_gaussian_filter", "oneka_count_histogram", "oneka_gemm_bf16", "oneka_bce_bitmask",
           "oneka_gelu_backward", "oneka_colsum_bf16", "oneka_adamw", "oneka_features",
           "oneka_sigmoid_colsum", "oneka_gemm_bf16_sigmoid_colsum", "oneka_gemm_bf16_path",
           "oneka_gemm_tc_status", "oneka_fit_rows", "oneka_fit_solve", "oneka_transpose_bf16",
           "oneka_adamw_scheduled", "oneka_bce_bitmask_t", "oneka_adamw_scheduled_t"]
NOALLOC_SCRATCH_BYTES = 32 << 20

_P = ctypes.c_void_p
_D = ctypes.c_double
_I = ctypes.c_int32


class OnekaDist(ctypes.Structure):
    _fields_ = [("kind", _I), ("pad", _I), ("p0", _D), ("p1", _D), ("p2", _D)]


class OnekaSite(ctypes.Structure):
    _fields_ = [("nwells", _I), ("nobs", _I), ("target", _I), ("pad", _I), ("base", _D),
                ("xo", _D), ("yo", _D), ("wells", _P), ("obs", _P)]


class OnekaRealizations(ctypes.Structure):
    _fields_ = [("coef", _P), ("coef_ev", _P), ("coef_cov", _P), ("q", _P), ("aquifer", _P),
                ("status", _P)]


class OnekaGrid(ctypes.Structure):
    _fields_ = [("xmin", _D), ("ymin", _D), ("dx", _D), ("dy", _D), ("nrows", _I), ("ncols", _I)]


class OnekaFrame(ctypes.Structure):
    _fields_ = [("xmin", _D), ("ymin", _D), ("coff", _I), ("roff", _I), ("ncols", _I),
                ("nrows", _I)]


class OnekaTrackOpts(ctypes.Structure):
    _fields_ = [("duration", _D), ("tol", _D), ("maxstep", _D), ("umbra", _D), ("confined", _I),
                ("precision", _I), ("max_attempts", _I), ("block", _I), ("window_kb", _I),
                ("occupancy", _I), ("head64", _I)]


class OnekaTrackOut(ctypes.Structure):
    _fields_ = [("endpoint", _P), ("bbox", _P), ("naccept", _P), ("nattempt", _P), ("status", _P),
                ("vertices", _P), ("nvertices", _P), ("max_vertices", _I), ("pad", _I),
                ("counters", _P)]


class OnekaTrackJob(ctypes.Structure):
    _fields_ = [("site", ctypes.POINTER(OnekaSite)), ("real", ctypes.POINTER(OnekaRealizations)),
                ("nreal", _I), ("npaths", _I), ("release", _P), ("opts", ctypes.POINTER(OnekaTrackOpts)),
                ("grid", ctypes.POINTER(OnekaGrid)), ("counts", _P), ("registered", _P),
                ("out", ctypes.POINTER(OnekaTrackOut))]


_lib = None
_lock = threading.Lock()


class OnekaError(RuntimeError):
    pass


def load() -> ctypes.CDLL:
    """Load the library (built by ``onekapy_gb300.build``); raise if absent."""
    global _lib
    with _lock:
        if _lib is not None:
            return _lib
        if not os.path.exists(LIB_PATH):
            raise OnekaError(
                f"{LIB_PATH} is missing: build it with `python -m onekapy_gb300.build` "
                "(there is no CPU fallback)")
        L = ctypes.CDLL(LIB_PATH)
        L.oneka_abi_version.restype = ctypes.c_int
        L.oneka_abi_version.argtypes = []
        L.oneka_last_error.restype = ctypes.c_char_p
        L.oneka_last_error.argtypes = []
        L.oneka_site_logr2.restype = ctypes.c_int
        L.oneka_site_logr2.argtypes = [ctypes.POINTER(OnekaSite), _P, _P]
        L.oneka_realize.restype = ctypes.c_int
        L.oneka_realize.argtypes = [ctypes.POINTER(OnekaSite), _P, ctypes.POINTER(OnekaDist), _P,
                                    ctypes.c_uint64, ctypes.c_uint64, _I, _I,
                                    ctypes.POINTER(OnekaRealizations), _P]
        L.oneka_adamw_scheduled.restype = ctypes.c_int
        L.oneka_adamw_scheduled.argtypes = [_P, _P, _P, _P, _P, ctypes.c_int64, _P, ctypes.c_float, ctypes.c_float,
                                            ctypes.c_float, ctypes.c_float, _P]
        L.oneka_bce_bitmask_t.restype = ctypes.c_int
        L.oneka_bce_bitmask_t.argtypes = [_P, _P, ctypes.c_int64, _I, _I, _I, _I, ctypes.c_float, _P, _P,
                                          ctypes.c_int64, _P, _P]
        L.oneka_adamw_scheduled_t.restype = ctypes.c_int
        L.oneka_adamw_scheduled_t.argtypes = [_P, _P, _P, _P, _P, _P, ctypes.c_int64, _I, _I, _P, ctypes.c_float,
                                              ctypes.c_float, ctypes.c_float, ctypes.c_float, _P]
        L.oneka_transpose_bf16.restype = ctypes.c_int
        L.oneka_transpose_bf16.argtypes = [_P, _I, _I, ctypes.c_int64, _P, ctypes.c_int64, _P]
        L.oneka_fit_rows.restype = ctypes.c_int
        L.oneka_fit_rows.argtypes = [ctypes.POINTER(OnekaSite), _P, _D, _D, _P, _P, _P, _P]
        L.oneka_fit_solve.restype = ctypes.c_int
        L.oneka_fit_solve.argtypes = [_P, _P, _I, _I, _P, _P, _P, _P]
        L.oneka_track_scratch_bytes.restype = ctypes.c_size_t
        L.oneka_track_scratch_bytes.argtypes = [ctypes.POINTER(OnekaGrid), _I]
        L.oneka_track.restype = ctypes.c_int
        L.oneka_track.argtypes = [ctypes.POINTER(OnekaSite), ctypes.POINTER(OnekaRealizations), _I,
                                  _P, _I, ctypes.POINTER(OnekaTrackOpts), ctypes.POINTER(OnekaGrid),
                                  _P, _P, _P, ctypes.POINTER(OnekaTrackOut), _P, ctypes.c_size_t, _P]
        L.oneka_track_noalloc.restype = ctypes.c_int
        L.oneka_track_noalloc.argtypes = [ctypes.POINTER(OnekaSite), ctypes.POINTER(OnekaRealizations), _I,
                                          _P, _I, ctypes.POINTER(OnekaTrackOpts),
                                          ctypes.POINTER(OnekaGrid), _P, _P, _P,
                                          ctypes.POINTER(OnekaTrackOut), _P]
        L.oneka_track_batched_scratch_bytes.restype = ctypes.c_size_t
        L.oneka_track_batched_scratch_bytes.argtypes = [ctypes.POINTER(OnekaTrackJob), _I]
        L.oneka_track_batched.restype = ctypes.c_int
        L.oneka_track_batched.argtypes = [ctypes.POINTER(OnekaTrackJob), _I, _P, ctypes.c_size_t, _P]
        L.oneka_gaussian_filter.restype = ctypes.c_int
        L.oneka_gaussian_filter.argtypes = [_P, _P, _P, _I, _I, _P, _I, _P]
        L.oneka_count_histogram.restype = ctypes.c_int
        L.oneka_count_histogram.argtypes = [_P, ctypes.c_int64, _I, _P, _P]
        L.oneka_gemm_bf16.restype = ctypes.c_int
        L.oneka_gemm_bf16.argtypes = [_P, _I, _I, _P, _I, _I, _P, _I, _I, _P, _I, _P, _I, _I, _I, _I, _I, _P]
        L.oneka_gemm_bf16_path.restype = ctypes.c_int
        L.oneka_gemm_bf16_path.argtypes = [_I] * 9
        L.oneka_gemm_tc_status.restype = ctypes.c_int
        L.oneka_gemm_tc_status.argtypes = [ctypes.POINTER(ctypes.c_int32)]
        L.oneka_bce_bitmask.restype = ctypes.c_int
        L.oneka_bce_bitmask.argtypes = [_P, _P, ctypes.c_int64, _I, _I, _I, _I, ctypes.c_float, _P, _P, _P]
        L.oneka_gelu_backward.restype = ctypes.c_int
        L.oneka_gelu_backward.argtypes = [_P, _P, _P, ctypes.c_int64, _P]
        L.oneka_colsum_bf16.restype = ctypes.c_int
        L.oneka_colsum_bf16.argtypes = [_P, _I, _I, _P, _P]
        L.oneka_adamw.restype = ctypes.c_int
        L.oneka_adamw.argtypes = [_P, _P, _P, _P, _P, ctypes.c_int64, ctypes.c_float, ctypes.c_float,
                                  ctypes.c_float, ctypes.c_float, ctypes.c_float, _I, _P]
        L.oneka_features.restype = ctypes.c_int
        L.oneka_features.argtypes = [_P, _P, _P, _I, _I, _P, _P, _I, _I, _P, _P]
        L.oneka_sigmoid_colsum.restype = ctypes.c_int
        L.oneka_sigmoid_colsum.argtypes = [_P, _I, _I, _P, _P]
        L.oneka_gemm_bf16_sigmoid_colsum.restype = ctypes.c_int
        L.oneka_gemm_bf16_sigmoid_colsum.argtypes = [_P, _I, _P, _I, _P, _P, _I, _I, _I, _I, _P]
        L.oneka_evaluate.restype = ctypes.c_int
        L.oneka_evaluate.argtypes = [ctypes.POINTER(OnekaSite), _P, _D, _D, _D,
                                     ctypes.POINTER(ctypes.c_double), _P, ctypes.c_int64, _I, _P, _P,
                                     _P, _P, _P, _P]
        L.oneka_rasterize.restype = ctypes.c_int
        L.oneka_rasterize.argtypes = [ctypes.POINTER(OnekaGrid), ctypes.POINTER(OnekaFrame), _P,
                                      ctypes.c_int64, _D, _P, _P]
        L.oneka_register_weighted.restype = ctypes.c_int
        L.oneka_register_weighted.argtypes = [ctypes.POINTER(OnekaGrid), _P, _D, _P, _P]
        L.oneka_fma_peak.restype = ctypes.c_int
        L.oneka_fma_peak.argtypes = [_I, ctypes.POINTER(ctypes.c_double), _P]
        L.oneka_distancesquared.restype = ctypes.c_int
        L.oneka_distancesquared.argtypes = [_P, _P, ctypes.c_int64, _P]
        if L.oneka_abi_version() != 1:
            raise OnekaError("liboneka_gb300.so ABI version mismatch")
        _lib = L
        return L


def check(rc: int) -> None:
    if rc != ONEKA_OK:
        msg = load().oneka_last_error().decode(errors="replace")
        raise OnekaError(f"liboneka_gb300 error {rc}: {msg}")


def device() -> torch.device:
    if not torch.cuda.is_available():
        raise OnekaError("onekapy_gb300 needs a CUDA device (GB300, sm_103a); none is visible")
    return torch.device("cuda", torch.cuda.current_device())


def stream_ptr(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def ptr(t) -> int | None:
    if t is None:
        return None
    if not t.is_cuda:
        raise OnekaError("expected a CUDA tensor")
    if not t.is_contiguous():
        raise OnekaError("expected a contiguous tensor")
    return int(t.data_ptr())
