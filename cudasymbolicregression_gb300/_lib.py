"""ctypes binding of ``libsr_gb300.so`` (declared in ``include/sr_gb300.h``).

The library is built in-tree by ``cudasymbolicregression_gb300/build.py``.  There
is no fallback: when the library is missing or CUDA is unavailable every entry
point of the package raises.
"""
from __future__ import annotations

import ctypes
import os

import torch

from . import build as _build

_LIB = None

i64 = ctypes.c_int64
i32 = ctypes.c_int32
vp = ctypes.c_void_p
dbl = ctypes.c_double


class FitOptions(ctypes.Structure):
    """Mirror of ``sr_fit_options``."""
    _fields_ = [
        ("max_iter", i32),
        ("history_size", i32),
        ("tolerance_grad", dbl),
        ("line_search", i32),
        ("line_search_max_iter", i32),
        ("eps", dbl),
        ("objective", i32),
        ("warps_per_block", i32),
        ("points_per_lane", i32),
        ("grid_blocks", i32),
        ("max_operators", i32),
        ("max_live", i32),
    ]


class MlpEpilogue(ctypes.Structure):
    """Mirror of ``sr_mlp_epilogue``."""
    _fields_ = [
        ("epilogue", i32),
        ("splits", i32),
        ("bias", vp),
        ("gate", vp),
        ("ld_gate", i64),
        ("out", vp),
        ("ld_out", i64),
        ("out_col0", i64),
        ("out_t", vp),
        ("ld_out_t", i64),
        ("out_t_row0", i64),
        ("out_f32", vp),
        ("ld_out_f32", i64),
        ("split_stride", i64),
    ]


MLP_EPI_RELU, MLP_EPI_LINEAR, MLP_EPI_F32, MLP_EPI_RELU_GRAD, MLP_EPI_SPLIT_F32 = 0, 1, 2, 3, 4
MLP_VOCAB, MLP_EMB, MLP_FEATS, MLP_PROJ, MLP_IN = 64, 64, 32, 28, 128
MLP_TIMEOUT = 601
TAPE_EXCEEDS_LAUNCH = 602

_SIGS = {
    "sr_last_error": ([], ctypes.c_char_p),
    "sr_version": ([], ctypes.c_char_p),
    "sr_validate": ([vp, vp, i64, i64, i64, i64, i64, i64, i64, vp, vp], ctypes.c_int),
    "sr_tape_compile": ([vp, vp, i64, i64, i64, i64, i64, i64, i64, i32, vp, vp, vp, vp], ctypes.c_int),
    "sr_eval_forward_f32": ([vp, i64, i64, vp, vp, vp, i64, i64, i32, vp, i64, i64, vp, vp], ctypes.c_int),
    "sr_eval_forward_f64": ([vp, i64, i64, vp, vp, vp, i64, i64, i32, vp, i64, i64, vp, vp], ctypes.c_int),
    "sr_eval_backward_f32": ([vp, i64, i64, vp, vp, vp, i64, i64, i32, vp, i64, i64, vp, vp, vp, vp, vp, vp],
                             ctypes.c_int),
    "sr_eval_backward_f64": ([vp, i64, i64, vp, vp, vp, i64, i64, i32, vp, i64, i64, vp, vp, vp, vp, vp, vp],
                             ctypes.c_int),
    "sr_eval_forward_multi_f32": ([vp, i64, i64, vp, vp, vp, i64, i64, i32, vp, i64, i64, i64, i64, vp, vp],
                                  ctypes.c_int),
    "sr_eval_forward_multi_f64": ([vp, i64, i64, vp, vp, vp, i64, i64, i32, vp, i64, i64, i64, i64, vp, vp],
                                  ctypes.c_int),
    "sr_eval_backward_multi_f32": ([vp, i64, i64, vp, vp, vp, i64, i64, i32, vp, i64, i64, i64, i64, vp, vp, vp, vp,
                                    vp, vp], ctypes.c_int),
    "sr_eval_backward_multi_f64": ([vp, i64, i64, vp, vp, vp, i64, i64, i32, vp, i64, i64, i64, i64, vp, vp, vp, vp,
                                    vp, vp], ctypes.c_int),
    "sr_fit_workspace_bytes": ([i64, i64, i64, i32, i32, ctypes.POINTER(FitOptions)], i64),
    "sr_tape_live_rows": ([vp, vp, i64, i64, vp, vp], ctypes.c_int),
    "sr_fit_launch_shape": ([i64, i64, i64, i64, i32, i32, ctypes.POINTER(FitOptions), vp], ctypes.c_int),
    "sr_fit_screen": ([vp, i64, i64, vp, vp, vp, i64, i64, vp, i64, i64, i64, i64, vp, i32, i32,
                       ctypes.POINTER(FitOptions), vp, vp], ctypes.c_int),
    "sr_fit_lbfgs": ([vp, i64, i64, vp, vp, vp, i64, i64, vp, vp, i64, i64, vp, vp, vp, vp, vp, i32, i32,
                      ctypes.POINTER(FitOptions), vp, i64, vp, vp], ctypes.c_int),
    "sr_fit_lbfgs_static_scratch": ([vp, i64, i64, vp, vp, vp, i64, i64, vp, vp, i64, i64, vp, vp, vp, vp, vp,
                                     i32, i32, ctypes.POINTER(FitOptions), vp, vp], ctypes.c_int),
    "sr_postfix_children": ([vp, i64, i64, i32, vp, vp, vp], ctypes.c_int),
    "sr_postfix_to_infix": ([vp, i64, i64, i32, vp, i64, vp, vp], ctypes.c_int),
    "sr_pcfg_sample_infix": ([vp, vp, vp, vp, i32, i32, i64, i32, i32, ctypes.c_uint64, vp, vp, vp], ctypes.c_int),
    "sr_infix_to_postfix": ([vp, i64, i64, i32, vp, vp, vp], ctypes.c_int),
    "sr_infix_to_prefix": ([vp, i64, i64, i32, vp, vp, vp], ctypes.c_int),
    "sr_prefix_to_postfix": ([vp, i64, i64, i32, vp, vp, vp], ctypes.c_int),
    "sr_postfix_to_prefix": ([vp, i64, i64, i32, vp, vp, vp], ctypes.c_int),
    "sr_prefix_parent": ([vp, i64, i64, i32, vp, vp, vp], ctypes.c_int),
    "sr_prefix_to_infix": ([vp, i64, i64, i32, vp, i64, vp, vp], ctypes.c_int),
    "sr_const_offsets": ([vp, i64, i64, i64, i64, vp, vp], ctypes.c_int),
    "sr_const_scatter": ([vp, i64, i64, i64, i64, vp, vp, vp, vp], ctypes.c_int),
    "sr_mlp_gemm": ([vp, i64, i64, i64, vp, i64, i64, ctypes.POINTER(MlpEpilogue), vp, vp], ctypes.c_int),
    "sr_mlp_gemm_splits_used": ([i64, i32], ctypes.c_int),
    "sr_mlp_random_features": ([vp, i64, i64, vp, vp, vp, vp], ctypes.c_int),
    "sr_mlp_features": ([vp, i64, i64, i64, i64, vp, i64, vp, vp, vp, i64, vp, vp, vp, vp], ctypes.c_int),
    "sr_mlp_loss": ([vp, i64, i64, vp, vp, i32, ctypes.c_float, vp, vp, i64, vp, i64, vp], ctypes.c_int),
    "sr_mlp_colsum": ([vp, i64, i64, i64, vp, vp], ctypes.c_int),
    "sr_mlp_output_grad": ([vp, i64, i32, i64, ctypes.c_float, vp, i64, vp, i64, vp], ctypes.c_int),
    "sr_mlp_reduce_splits": ([vp, i32, i64, i64, vp, vp], ctypes.c_int),
    "sr_mlp_adam": ([vp, vp, vp, vp, i64, i64, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                     ctypes.c_float, i32, vp, vp, vp], ctypes.c_int),
}


def exported_symbols():
    """Names every ``include/sr_gb300.h`` entry point must export."""
    return list(_SIGS)


def load(build_if_missing: bool = True) -> ctypes.CDLL:
    """Load the library (building it first when it is missing or stale)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB
    if not os.path.exists(path) or (build_if_missing and not _build.up_to_date()):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing; build it with cudasymbolicregression_gb300.build.build()")
        _build.build()
    lib = ctypes.CDLL(path)
    for name, (args, res) in _SIGS.items():
        fn = getattr(lib, name)
        fn.argtypes = args
        fn.restype = res
    _LIB = lib
    return lib


def lib() -> ctypes.CDLL:
    return load()


def check(rc: int, what: str) -> None:
    """Raise for an API-level failure (negative return code)."""
    if rc != 0:
        msg = lib().sr_last_error().decode(errors="replace")
        raise RuntimeError(f"{what} failed ({rc}): {msg}")


def ptr(t: torch.Tensor | None):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


def stream_ptr(device: torch.device):
    return ctypes.c_void_p(torch.cuda.current_stream(device).cuda_stream)


def require_cuda(*tensors: torch.Tensor) -> torch.device:
    """All tensors on one CUDA device; returns it.  There is no CPU path."""
    dev = tensors[0].device
    for t in tensors:
        if t.device != dev:
            raise RuntimeError("All input tensors must be on the same device.")
    if dev.type != "cuda":
        raise RuntimeError(
            f"cudasymbolicregression_gb300 runs on CUDA tensors only (got device '{dev}'); "
            "move the inputs to a GPU")
    return dev
