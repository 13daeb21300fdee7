"""Batched postfix-tape evaluation with its adjoint, behind torch autograd.

Drop-in for ``symbolic_torch.evaluation`` (reference symbolic_torch/evaluation.py:4-34
and the C++ entry src/symbolic_evaluation.cpp:306-355):

* ``evaluate(X, Ops, Ch, C)`` with batch-first inputs returns the (B, M, N) value
  cache; it is differentiable w.r.t. X and C and accepts any dense gradient on
  every node.
* ``evaluate_backend(X, Ops, Ch, C)`` takes the M-first layout and returns a
  (M, N, B) view, as the reference's backend does.
* ``evaluate_multiple(X, Ops, Ch, C)`` with C (B, M, K) evaluates K constant sets
  per tape into a (B, M, N, K) cache (reference symbolic_torch/evaluation.py:36-65);
  ``evaluate_multiple_constant_backend`` is its M-first entry point.

The cache is written directly in (B, M, N) order by one kernel launch (the
reference launches one kernel per tape position); the adjoint recomputes node
values and never reads the cache.  Shape, dtype and validation errors carry the
reference's messages.
"""
from __future__ import annotations

import torch

from . import _lib
from .operators import error_message, scalar_type_name
from .tape import CompiledTapes, compile_tapes


def _check_dispatch(X, C):
    """The reference's evaluation reads X through a two-dimensional accessor and C as
    X's scalar type (its type dispatch): torch's messages for either mismatch."""
    if X.dim() != 2:
        raise RuntimeError(f"TensorAccessor expected 2 dims but tensor has {X.dim()}")
    if C.dtype != X.dtype:
        raise RuntimeError(f"expected scalar type {scalar_type_name(X.dtype)} but found {scalar_type_name(C.dtype)}")


def _check_backend_inputs(X, Ops, Ch, C):
    """The reference's argument checks, in its order and with its messages
    (src/symbolic_evaluation.cpp:312-334).  Ops/Ch/C are M-first here."""
    dev = X.device
    if Ops.device != dev or Ch.device != dev or C.device != dev:
        raise RuntimeError("All input tensors must be on the same device.")
    X.size(1)  # the reference reads n_x and M here: torch's IndexError below their ranks
    Ops.size(0)
    if Ops.dim() != 2:
        raise RuntimeError("Ops must be a 2D tensor")
    if Ch.dim() != 3:
        raise RuntimeError("Ch must be a 3D tensor")
    if C.dim() != 2:
        raise RuntimeError("C must be a 2D tensor")
    if Ops.size(0) != Ch.size(0):
        raise RuntimeError("Ops and Ch must have the same max length (dim 0)")
    if Ops.size(1) != Ch.size(1):
        raise RuntimeError("Ops and Ch must have the same batch size (dim 1)")
    if Ops.shape != C.shape:
        raise RuntimeError("Ops and C must have the same shape")
    if Ch.size(2) != 2:
        raise RuntimeError("Ch must have MaxArity as its last dimension")
    if X.dtype not in (torch.float32, torch.float64):
        raise RuntimeError("X must be a floating-point tensor (float or double)")
    if C.dtype not in (torch.float32, torch.float64):
        raise RuntimeError("C must be a floating-point tensor (float or double)")
    if Ops.dtype != torch.int64:
        raise RuntimeError("Ops must be a Long tensor")
    if Ch.dtype != torch.int64:
        raise RuntimeError("Ch must be a Long tensor")
    _check_dispatch(X, C)
    _lib.require_cuda(X, Ops, Ch, C)


class _Evaluate(torch.autograd.Function):
    """Forward: sr_eval_forward_*; backward: sr_eval_backward_* (dense grad)."""

    @staticmethod
    def forward(ctx, X: torch.Tensor, C_bm: torch.Tensor, tapes: CompiledTapes):
        Xc = X.contiguous()
        B, M = tapes.B, tapes.M
        N, nx = Xc.shape
        cache = torch.empty((B, M, N), dtype=Xc.dtype, device=Xc.device)
        L = _lib.lib()
        fn = L.sr_eval_forward_f32 if Xc.dtype == torch.float32 else L.sr_eval_forward_f64
        cb, cm = C_bm.stride()
        rc = fn(_lib.ptr(Xc), N, nx, _lib.ptr(tapes.desc), _lib.ptr(tapes.meta), _lib.ptr(tapes.order), B, M,
                tapes.max_len, _lib.ptr(C_bm), cb, cm, _lib.ptr(cache), _lib.stream_ptr(Xc.device))
        _lib.check(rc, "sr_eval_forward")
        ctx.tapes = tapes
        # the adjoint reads the node values from the cache, as the reference's backward does
        ctx.save_for_backward(Xc, C_bm, cache)
        return cache

    @staticmethod
    def backward(ctx, grad):
        Xc, C_bm, cache = ctx.saved_tensors
        tapes: CompiledTapes = ctx.tapes
        B, M = tapes.B, tapes.M
        N, nx = Xc.shape
        grad = grad.contiguous()
        gC = torch.empty((B, M), dtype=Xc.dtype, device=Xc.device)
        gX = torch.zeros_like(Xc) if ctx.needs_input_grad[0] else None
        status = torch.empty(1, dtype=torch.int32, device=Xc.device)
        L = _lib.lib()
        fn = L.sr_eval_backward_f32 if Xc.dtype == torch.float32 else L.sr_eval_backward_f64
        cb, cm = C_bm.stride()
        rc = fn(_lib.ptr(Xc), N, nx, _lib.ptr(tapes.desc), _lib.ptr(tapes.meta), _lib.ptr(tapes.order), B, M,
                tapes.max_len, _lib.ptr(C_bm), cb, cm, _lib.ptr(cache), _lib.ptr(grad), _lib.ptr(gC), _lib.ptr(gX),
                _lib.ptr(status), _lib.stream_ptr(Xc.device))
        _lib.check(rc, "sr_eval_backward")
        code = int(status.item())
        if code:
            raise RuntimeError(error_message(code, "symbolic evaluation backward pass"))
        return gX, gC, None


def _evaluate_bmn(X, ops_bm, ch_bm, C_bm):
    tapes = compile_tapes(ops_bm, ch_bm, X.shape[1])
    return _Evaluate.apply(X, C_bm, tapes)


def evaluate_backend(X: torch.Tensor, Ops: torch.Tensor, Ch: torch.Tensor, C: torch.Tensor) -> torch.Tensor:
    """M-first entry point: X (N, n_x), Ops (M, B), Ch (M, B, 2), C (M, B) -> (M, N, B).

    The result is a view of the (B, M, N) cache."""
    _check_backend_inputs(X, Ops, Ch, C)
    out = _evaluate_bmn(X, Ops.permute(1, 0), Ch.permute(1, 0, 2), C.permute(1, 0))
    return out.permute(1, 2, 0)


def evaluate(X: torch.Tensor, Ops: torch.Tensor, Ch: torch.Tensor, C: torch.Tensor) -> torch.Tensor:
    """Evaluate B postfix tapes at N points.

    Args:
        X: (N, n_x) float32/float64 inputs.
        Ops: (B, M) int64 operator codes (postfix, child indices below parents).
        Ch: (B, M, 2) int64 child indices, -1 where absent.
        C: (B, M) learnable constants (read where Ops is LEARNABLE_CONSTANT).

    Returns:
        (B, M, N) values of every node at every point; NO_OP nodes are NaN.
    """
    # the reference permutes to M-first (torch's own error for a wrong rank), then checks
    _check_backend_inputs(X, Ops.permute(1, 0), Ch.permute(1, 0, 2), C.permute(1, 0))
    return _evaluate_bmn(X, Ops, Ch, C)


# ---- multiple constant sets -----------------------------------------------------------

def _check_multiple_inputs(X, Ops, Ch, C):
    """The reference's argument checks for the multiple-constant entry point, in its
    order and with its messages (src/symbolic_evaluation.cpp:171-200).  M-first."""
    dev = X.device
    if Ops.device != dev or Ch.device != dev or C.device != dev:
        raise RuntimeError("All input tensors must be on the same device.")
    X.size(1)  # the reference reads n_x here: torch's IndexError below two dimensions
    if Ops.dim() != 2:
        raise RuntimeError("Ops must be a 2D tensor")
    if Ch.dim() != 3:
        raise RuntimeError("Ch must be a 3D tensor")
    if C.dim() != 3:
        raise RuntimeError("C must be a 3D tensor for multiple constant evaluation")
    if not (Ops.size(0) == Ch.size(0) == C.size(0)):
        raise RuntimeError("Ops, Ch, and C must have the same max length (dim 0)")
    if not (Ops.size(1) == Ch.size(1) == C.size(1)):
        raise RuntimeError("Ops, Ch, and C must have the same batch size (dim 1)")
    if Ch.size(2) != 2:
        raise RuntimeError("Ch must have MaxArity as its last dimension")
    if X.dtype not in (torch.float32, torch.float64):
        raise RuntimeError("X must be a floating-point tensor (float or double)")
    if C.dtype not in (torch.float32, torch.float64):
        raise RuntimeError("C must be a floating-point tensor (float or double)")
    if Ops.dtype != torch.int64:
        raise RuntimeError("Ops must be a Long tensor")
    if Ch.dtype != torch.int64:
        raise RuntimeError("Ch must be a Long tensor")
    _check_dispatch(X, C)
    _lib.require_cuda(X, Ops, Ch, C)


class _EvaluateMultiple(torch.autograd.Function):
    """Forward: sr_eval_forward_multi_*; backward: sr_eval_backward_multi_*."""

    @staticmethod
    def forward(ctx, X: torch.Tensor, C_bmk: torch.Tensor, tapes: CompiledTapes):
        Xc = X.contiguous()
        B, M = tapes.B, tapes.M
        K = C_bmk.shape[2]
        N, nx = Xc.shape
        cache = torch.empty((B, M, N, K), dtype=Xc.dtype, device=Xc.device)
        L = _lib.lib()
        fn = L.sr_eval_forward_multi_f32 if Xc.dtype == torch.float32 else L.sr_eval_forward_multi_f64
        cb, cm, ck = C_bmk.stride()
        rc = fn(_lib.ptr(Xc), N, nx, _lib.ptr(tapes.desc), _lib.ptr(tapes.meta), _lib.ptr(tapes.order), B, M,
                tapes.max_len, _lib.ptr(C_bmk), cb, cm, ck, K, _lib.ptr(cache), _lib.stream_ptr(Xc.device))
        _lib.check(rc, "sr_eval_forward_multi")
        ctx.tapes = tapes
        ctx.save_for_backward(Xc, C_bmk, cache)
        return cache

    @staticmethod
    def backward(ctx, grad):
        Xc, C_bmk, cache = ctx.saved_tensors
        tapes: CompiledTapes = ctx.tapes
        B, M = tapes.B, tapes.M
        K = C_bmk.shape[2]
        N, nx = Xc.shape
        grad = grad.contiguous()
        gC = torch.empty((B, M, K), dtype=Xc.dtype, device=Xc.device)
        gX = torch.zeros_like(Xc) if ctx.needs_input_grad[0] else None
        status = torch.empty(1, dtype=torch.int32, device=Xc.device)
        L = _lib.lib()
        fn = L.sr_eval_backward_multi_f32 if Xc.dtype == torch.float32 else L.sr_eval_backward_multi_f64
        cb, cm, ck = C_bmk.stride()
        rc = fn(_lib.ptr(Xc), N, nx, _lib.ptr(tapes.desc), _lib.ptr(tapes.meta), _lib.ptr(tapes.order), B, M,
                tapes.max_len, _lib.ptr(C_bmk), cb, cm, ck, K, _lib.ptr(cache), _lib.ptr(grad), _lib.ptr(gC),
                _lib.ptr(gX),
                _lib.ptr(status), _lib.stream_ptr(Xc.device))
        _lib.check(rc, "sr_eval_backward_multi")
        code = int(status.item())
        if code:
            raise RuntimeError(error_message(code, "symbolic evaluation (multiple constants) backward pass"))
        return gX, gC, None


def evaluate_multiple_constant_backend(X: torch.Tensor, Ops: torch.Tensor, Ch: torch.Tensor,
                                       C: torch.Tensor) -> torch.Tensor:
    """M-first entry point: X (N, n_x), Ops (M, B), Ch (M, B, 2), C (M, B, K) ->
    (M, N, B, K) (reference src/symbolic_evaluation.cpp:171-202).  The result is a
    view of the (B, M, N, K) cache."""
    _check_multiple_inputs(X, Ops, Ch, C)
    tapes = compile_tapes(Ops.permute(1, 0), Ch.permute(1, 0, 2), X.shape[1])
    out = _EvaluateMultiple.apply(X, C.permute(1, 0, 2), tapes)
    return out.permute(1, 2, 0, 3)


def evaluate_multiple(X: torch.Tensor, Ops: torch.Tensor, Ch: torch.Tensor, C: torch.Tensor) -> torch.Tensor:
    """Evaluate B postfix tapes at N points for K constant sets each
    (reference symbolic_torch/evaluation.py:36-65).

    Args:
        X: (N, n_x) float32/float64 inputs.  Ops: (B, M) int64.  Ch: (B, M, 2) int64.
        C: (B, M, K) constant sets.

    Returns:
        (B, M, N, K) values of every node at every point for every set; NO_OP nodes
        are NaN.  Differentiable w.r.t. X (summed over the sets) and C.
    """
    _check_multiple_inputs(X, Ops.permute(1, 0), Ch.permute(1, 0, 2), C.permute(1, 0, 2))
    tapes = compile_tapes(Ops, Ch, X.shape[1])
    return _EvaluateMultiple.apply(X, C, tapes)
