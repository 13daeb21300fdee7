"""Batched constant fitting: drop-in for ``symbolic_torch.optimize``
(reference symbolic_torch/optimization.py:9-112 with symbolic_torch/lbfgs_batch.py).

The whole L-BFGS run of every expression happens inside one persistent CUDA kernel
(``sr_fit_lbfgs``): no per-iteration host round trips, no (M, N, B) cache.
``optimize`` returns what the reference returns; ``optimize_ex`` also returns the
per-expression iteration counts, final losses and closure counts.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Literal, Optional, Tuple

import ctypes

import torch

from . import _lib
from .evaluation import _check_backend_inputs
from .operators import error_message
from .tape import compile_tapes


@dataclass
class FitResult:
    C: torch.Tensor        # (B, M) fitted constants
    Y: torch.Tensor        # (B, N) root values at the fitted constants
    iters: torch.Tensor    # (B,) int32 L-BFGS iterations run (-code for a problem that hit an error)
    loss: torch.Tensor     # (B,) float32 final mean squared error
    evals: torch.Tensor    # (B,) int32 closures (forward + adjoint passes) evaluated
    # per kernel launch: (problems, points per lane, warps per problem); the launch
    # shape fixes the order of the sums over the points, so a host restatement of a
    # fit needs it to reproduce the bits
    shapes: Optional[list] = None


# Launch shapes (points per lane V, warps per CTA W) the autotuner tries, and its
# decisions per problem class: (N, n_x, longest tape, most constants, line search).
_TUNE_CANDIDATES = ((1, 2), (1, 4), (1, 8), (2, 2), (2, 4), (2, 8))
_TUNED: dict = {}


def _autotune(X, Y, Ops, Ch, C_init, max_iter, history_size, tolerance_grad, line_search_fn, key, sample=2048,
              tune_iter=20, **kw):
    """Time every candidate launch shape on a seeded random sample of the problems
    (at most `tune_iter` iterations each) and return the fastest (V, W)."""
    if key in _TUNED:
        return _TUNED[key]
    B = Ops.shape[0]
    g = torch.Generator().manual_seed(1234)
    idx = torch.randperm(B, generator=g)[:min(B, sample)].to(Ops.device)
    Xs, Ys, Os, Cs, C0 = X, Y[idx] if Y is not None else None, Ops[idx], Ch[idx], C_init[idx]
    N = X.shape[0]
    best, best_t = None, float("inf")
    for V, W in _TUNE_CANDIDATES:
        if W * 32 * V > 2 * max(N, 32):
            continue  # more points per CTA than the data has
        try:
            times = []
            for rep in range(2):  # the first run also builds the program caches
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                _fit(Xs, Ys, Os, Cs, C0, min(max_iter, tune_iter), history_size, tolerance_grad, line_search_fn,
                     points_per_lane=V, warps_per_block=W, raise_errors=False, want_y=False, **kw)
                e1.record()
                e1.synchronize()
                times.append(e0.elapsed_time(e1))
            t = times[-1]
        except RuntimeError:
            continue  # the shape does not fit (shared memory)
        if t < best_t:
            best, best_t = (V, W), t
    _TUNED[key] = best if best is not None else (0, 0)
    return _TUNED[key]


def _targets(Y: torch.Tensor, B: int, N: int, dev: torch.device) -> torch.Tensor:
    """(B, N) float32 contiguous targets.  The reference's loss broadcasts Y against
    the (B, N) predictions (nn.MSELoss(reduction='none'), symbolic_torch/optimization.py:
    69, 87), so one target row of shape (N,) or (1, N), a column (B, 1) or a scalar
    serves every expression; a Y that does not broadcast to (B, N) is an error."""
    if Y.device != dev:
        raise RuntimeError("All input tensors must be on the same device.")
    try:
        shape = tuple(torch.broadcast_shapes(tuple(Y.shape), (B, N)))
    except RuntimeError:
        shape = None
    if shape != (B, N):
        raise RuntimeError(f"Y must broadcast to (B, N) = ({B}, {N}), got {tuple(Y.shape)}")
    return Y.to(torch.float32).expand(B, N).contiguous()


def _fit(X, Y, Ops, Ch, C_init, max_iter, history_size, tolerance_grad, line_search_fn, *,
         objective: int = 0, line_search_max_iter: int = 10, eps: float = 1e-10,
         warps_per_block: int = 0, points_per_lane: int = 0, grid_blocks: int = 0,
         order: Optional[torch.Tensor] = None, want_y: bool = True, raise_errors: bool = True,
         class_width: int = 0, kernel_events=None, autotune: bool = False, consts_floor: int = 0) -> FitResult:
    # the reference's order: unpack Ops' shape (ValueError for another rank), permute C_init
    # and Ops (torch's error for a wrong rank), build the optimizer (line search name),
    # then the evaluation's own checks
    B, M = Ops.shape
    C_init.permute(1, 0)
    if line_search_fn not in ("strong_wolfe", "backtracking"):
        raise ValueError(f"Invalid line_search_fn: {line_search_fn}. Choose 'strong_wolfe' or 'backtracking'.")
    _check_backend_inputs(X, Ops.permute(1, 0), Ch.permute(1, 0, 2), C_init.permute(1, 0))
    if X.dtype != torch.float32:
        raise RuntimeError("optimize runs in float32: X and C_init must be float32")
    dev = X.device
    N, nx = X.shape
    if Y is not None:
        Y = _targets(Y, B, N, dev)
    tapes = compile_tapes(Ops, Ch, nx, live=True)
    # the constant slots are laid out for the most constants of any tape (at least
    # consts_floor): 1, 2 or 4 slot registers per lane, which fixes the order of the
    # direction's sums
    kmax = max(int(tapes.max_consts), int(consts_floor))
    Xc = X.contiguous()
    if autotune and warps_per_block == 0 and points_per_lane == 0:
        key = (N, nx, tapes.max_root, tapes.max_consts, line_search_fn, objective)
        points_per_lane, warps_per_block = _autotune(
            X, Y, Ops, Ch, C_init, max_iter, history_size, tolerance_grad, line_search_fn, key, objective=objective,
            line_search_max_iter=line_search_max_iter, eps=eps)
    opts = _lib.FitOptions(max_iter=int(max_iter), history_size=int(history_size),
                           tolerance_grad=float(tolerance_grad),
                           line_search=0 if line_search_fn == "strong_wolfe" else 1,
                           line_search_max_iter=int(line_search_max_iter), eps=float(eps),
                           objective=int(objective), warps_per_block=int(warps_per_block),
                           points_per_lane=int(points_per_lane), grid_blocks=int(grid_blocks),
                           max_operators=int(max(tapes.max_operators, 1)),
                           max_live=int(tapes.max_live))
    L = _lib.lib()
    C_out = torch.empty((B, M), dtype=torch.float32, device=dev)
    Y_out = torch.empty((B, N), dtype=torch.float32, device=dev) if want_y else None
    iters = torch.empty(B, dtype=torch.int32, device=dev)
    loss = torch.empty(B, dtype=torch.float32, device=dev)
    evals = torch.empty(B, dtype=torch.int32, device=dev)
    Cin = C_init.to(torch.float32).contiguous()
    lens = tapes.meta[:, 1] + 1
    if order is None:
        # longest tapes first: the persistent warps then finish at about the same time
        order = torch.argsort(lens, descending=True, stable=True).to(torch.int32)
        classes = _length_classes(lens, order, class_width) if class_width > 0 else [(0, B, max(tapes.max_root, 1))]
    else:
        order = order.to(device=dev, dtype=torch.int32).contiguous()
        classes = [(0, B, max(tapes.max_root, 1))]
    status = torch.zeros(max(len(classes), 1), dtype=torch.int32, device=dev)
    shapes = []
    if kernel_events is not None:
        kernel_events[0].record()
    for ci, (start, count, max_len) in enumerate(classes):
        if count == 0:
            continue
        # one launch per class of tape lengths: the per-warp shared memory is sized
        # for the class, so short tapes run with more resident warps
        max_len = min(max_len, M)
        wsb = L.sr_fit_workspace_bytes(count, N, M, max_len, kmax, opts)
        if wsb < 0:
            _lib.check(-1, "sr_fit_workspace_bytes")
        ws = torch.empty(int(wsb), dtype=torch.uint8, device=dev)
        shapes.append((order[start:start + count], *_launch_shape(L, count, N, nx, M, max_len, kmax, opts)))
        optr = ctypes.c_void_p(order.data_ptr() + 4 * start)
        rc = L.sr_fit_lbfgs(_lib.ptr(Xc), N, nx, _lib.ptr(Y), _lib.ptr(tapes.desc), _lib.ptr(tapes.meta), count, M,
                            _lib.ptr(Cin), _lib.ptr(C_out), M, 1, _lib.ptr(Y_out), _lib.ptr(iters), _lib.ptr(loss),
                            _lib.ptr(evals), optr, max_len, kmax, opts, _lib.ptr(ws), ws.numel(),
                            ctypes.c_void_p(status.data_ptr() + 4 * ci), _lib.stream_ptr(dev))
        _lib.check(rc, "sr_fit_lbfgs")
    if kernel_events is not None:
        kernel_events[1].record()
    codes = [c for c in status.tolist() if c]
    code = codes[0] if codes else 0
    if code == _lib.TAPE_EXCEEDS_LAUNCH:  # the sizes above come from compile_tapes: cannot happen here
        raise RuntimeError("a tape exceeds the table sizes the fit kernel was launched with")
    if code and raise_errors:
        ctx = "input validation" if code in (101, 102) else "symbolic evaluation backward pass"
        raise RuntimeError(error_message(code, ctx))
    return FitResult(C=C_out, Y=Y_out, iters=iters, loss=loss, evals=evals, shapes=shapes)


def screen_starts(X, Y, Ops, Ch, C_sets, *, objective: int = 0, tapes=None) -> torch.Tensor:
    """Multi-start screening: the loss of each of K candidate starting constant sets
    for every problem, as the fit's first closure measures it, in one kernel launch
    (``sr_fit_screen``; forward passes only).  C_sets is (K, B, M) float32; returns
    (B, K) float32 (NaN where a candidate's loss is not finite).  No counterpart in
    the reference, whose optimize starts from one C."""
    B, M = Ops.shape
    K = C_sets.shape[0]
    if C_sets.dim() != 3 or tuple(C_sets.shape[1:]) != (B, M):
        raise RuntimeError(f"C_sets must be (K, B, M) = (K, {B}, {M}), got {tuple(C_sets.shape)}")
    _check_backend_inputs(X, Ops.permute(1, 0), Ch.permute(1, 0, 2), C_sets[0].permute(1, 0))
    if X.dtype != torch.float32:
        raise RuntimeError("optimize runs in float32: X and C_init must be float32")
    dev = X.device
    N, nx = X.shape
    if Y is not None:
        Y = _targets(Y, B, N, dev)
    if tapes is None:
        tapes = compile_tapes(Ops, Ch, nx, live=True)
    opts = _lib.FitOptions(max_iter=0, history_size=1, tolerance_grad=0.0, line_search=0, line_search_max_iter=0,
                           eps=0.0, objective=int(objective), max_operators=int(max(tapes.max_operators, 1)),
                           max_live=int(tapes.max_live))
    Cs = C_sets.to(torch.float32).contiguous()
    out = torch.empty((B, K), dtype=torch.float32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    L = _lib.lib()
    rc = L.sr_fit_screen(_lib.ptr(X.contiguous()), N, nx, _lib.ptr(Y), _lib.ptr(tapes.desc), _lib.ptr(tapes.meta), B,
                         M, _lib.ptr(Cs), B * M, M, 1, K, _lib.ptr(out), min(max(tapes.max_root, 1), M),
                         tapes.max_consts, opts, _lib.ptr(status), _lib.stream_ptr(dev))
    _lib.check(rc, "sr_fit_screen")
    return out


def _launch_shape(L, B, N, nx, M, max_len, max_consts, opts):
    """(points per lane, warps per problem) that sr_fit_lbfgs picks for a launch."""
    shape = (ctypes.c_int32 * 3)()
    _lib.check(L.sr_fit_launch_shape(B, N, nx, M, max_len, max_consts, opts, ctypes.cast(shape, ctypes.c_void_p)),
               "sr_fit_launch_shape")
    return int(shape[0]), int(shape[1])


def batch_launch_shape(X: torch.Tensor, Ops: torch.Tensor, Ch: torch.Tensor) -> dict:
    """What fixes the arithmetic of a fit of this whole batch in one launch, as
    optimize_ex keywords: the launch shape the library picks for it (points per lane,
    warps per problem: the order of the sums over the points) and its most constants
    of any tape (the slot registers per lane: the order of the direction's sums).  A
    slice of the batch fitted with these keywords gives every problem the bits the
    whole fit gives it; left to itself, a slice can get another shape (the shape
    depends on the problem count, the longest tape and the most constants)."""
    B, M = Ops.shape
    N, nx = X.shape
    tapes = compile_tapes(Ops, Ch, nx, live=True)
    opts = _lib.FitOptions(max_iter=1, history_size=1, tolerance_grad=0.0, line_search=0, line_search_max_iter=0,
                           eps=0.0, objective=0, max_operators=int(max(tapes.max_operators, 1)),
                           max_live=int(tapes.max_live))
    V, W = _launch_shape(_lib.lib(), B, N, nx, M, min(max(tapes.max_root, 1), M), tapes.max_consts, opts)
    return {"points_per_lane": V, "warps_per_block": W, "consts_floor": int(tapes.max_consts)}


def _length_classes(lens: torch.Tensor, order: torch.Tensor, width: int):
    """(start, count, max_len) of each class of tape lengths along ``order``
    (longest first); class c holds lengths in ((c-1)*width, c*width].  One host sync."""
    cls = (lens[order.long()] + width - 1) // width
    counts = torch.bincount(cls).tolist()
    classes, start = [], 0
    for c in range(len(counts) - 1, 0, -1):
        if counts[c]:
            classes.append((start, counts[c], c * width))
            start += counts[c]
    return classes


def optimize(
    X: torch.Tensor,
    Y: torch.Tensor,
    Ops: torch.Tensor,
    Ch: torch.Tensor,
    C_init: torch.Tensor,
    max_iter: int = 100,
    history_size: int = 10,
    tolerance_grad: float = 1e-7,
    line_search_fn: Literal["strong_wolfe", "backtracking"] = "strong_wolfe",
) -> Tuple[torch.Tensor, torch.Tensor]:
    """Fit the learnable constants of every expression to its target row.

    Args:
        X: (N, n_x) float32 inputs.  Y: (B, N) float32 targets.
        Ops: (B, M) int64 postfix tapes, left-packed (root = number of non-NO_OP
            entries - 1).  Ch: (B, M, 2) int64 children.  C_init: (B, M) float32.
        max_iter, history_size, tolerance_grad, line_search_fn: as LBFGS_batch.

    Returns:
        (C_final (B, M), Y_final (B, N)).
    """
    r = _fit(X, Y, Ops, Ch, C_init, max_iter, history_size, tolerance_grad, line_search_fn)
    return r.C, r.Y


def optimize_ex(X, Y, Ops, Ch, C_init, max_iter=100, history_size=10, tolerance_grad=1e-7,
                line_search_fn="strong_wolfe", **kw) -> FitResult:
    """``optimize`` plus per-expression iterations, final loss and closure counts.

    Extra keywords: line_search_max_iter, eps, objective (0 = MSE against Y,
    1 = mean of the root value; Y may be None), warps_per_block, points_per_lane,
    grid_blocks (kernel shape), consts_floor (lay the constant slots out for at least
    this many constants; see batch_launch_shape), order (processing order), want_y, class_width
    (tapes are fitted in launches per class of lengths this many nodes wide, 0 =
    one launch), raise_errors
    (False: problems whose closures hit error 201/204 are reported through
    ``iters < 0`` instead of aborting the whole batch as the reference does),
    kernel_events (a pair of torch.cuda.Event recorded on the current stream just
    before the first and just after the last fit-kernel launch), autotune (time the
    candidate launch shapes on a sample of the batch once per problem class and use
    the fastest; the choice is cached for the process).
    """
    return _fit(X, Y, Ops, Ch, C_init, max_iter, history_size, tolerance_grad, line_search_fn, **kw)


class FitPlan:
    """A fit of fixed tapes and data whose launches can be replayed and captured in a
    CUDA graph: validation, staging, ordering and every allocation happen once here
    (one host synchronisation); ``run`` then only enqueues the status/counter resets
    and the fused fit kernel on the current stream, so a sequence of fits of the same
    expressions from different starting constants (multi-start, warm-start rounds)
    costs one graph replay each.

    plan = FitPlan(X, Y, Ops, Ch, max_iter=100)
    plan.C_in.copy_(C0); plan.run()            # or: g = plan.capture(); ...; g.replay()
    plan.result()                              # FitResult (reads the status once)
    """

    def __init__(self, X, Y, Ops, Ch, max_iter=100, history_size=10, tolerance_grad=1e-7,
                 line_search_fn="strong_wolfe", *, objective: int = 0, line_search_max_iter: int = 10,
                 eps: float = 1e-10, warps_per_block: int = 0, points_per_lane: int = 0, grid_blocks: int = 0,
                 want_y: bool = True):
        if line_search_fn not in ("strong_wolfe", "backtracking"):
            raise ValueError(f"Invalid line_search_fn: {line_search_fn}. Choose 'strong_wolfe' or 'backtracking'.")
        B, M = Ops.shape
        _check_backend_inputs(X, Ops.permute(1, 0), Ch.permute(1, 0, 2),
                              torch.empty((M, B), dtype=X.dtype, device=X.device))
        if X.dtype != torch.float32:
            raise RuntimeError("optimize runs in float32: X and C_init must be float32")
        dev = X.device
        N, nx = X.shape
        self.B, self.M, self.N, self.nx = B, M, N, nx
        self.X = X.contiguous()
        self.Y = None if Y is None else _targets(Y, B, N, dev)
        self.tapes = compile_tapes(Ops, Ch, nx, live=True)
        self.order = torch.argsort(self.tapes.meta[:, 1] + 1, descending=True, stable=True).to(torch.int32)
        self.opts = _lib.FitOptions(max_iter=int(max_iter), history_size=int(history_size),
                                    tolerance_grad=float(tolerance_grad),
                                    line_search=0 if line_search_fn == "strong_wolfe" else 1,
                                    line_search_max_iter=int(line_search_max_iter), eps=float(eps),
                                    objective=int(objective), warps_per_block=int(warps_per_block),
                                    points_per_lane=int(points_per_lane), grid_blocks=int(grid_blocks),
                                    max_operators=int(max(self.tapes.max_operators, 1)),
                                    max_live=int(self.tapes.max_live))
        L = _lib.lib()
        self.max_len = min(max(self.tapes.max_root, 1), M)
        wsb = L.sr_fit_workspace_bytes(B, N, M, self.max_len, self.tapes.max_consts, self.opts)
        if wsb < 0:
            _lib.check(-1, "sr_fit_workspace_bytes")
        self.ws = torch.empty(int(wsb), dtype=torch.uint8, device=dev)
        self.C_in = torch.zeros((B, M), dtype=torch.float32, device=dev)
        self.C_out = torch.empty((B, M), dtype=torch.float32, device=dev)
        self.Y_out = torch.empty((B, N), dtype=torch.float32, device=dev) if want_y else None
        self.iters = torch.empty(B, dtype=torch.int32, device=dev)
        self.loss = torch.empty(B, dtype=torch.float32, device=dev)
        self.evals = torch.empty(B, dtype=torch.int32, device=dev)
        self.status = torch.zeros(1, dtype=torch.int32, device=dev)

    def run(self) -> None:
        """Enqueue one fit from self.C_in on the current stream (no synchronisation)."""
        L = _lib.lib()
        rc = L.sr_fit_lbfgs(_lib.ptr(self.X), self.N, self.nx, _lib.ptr(self.Y), _lib.ptr(self.tapes.desc),
                            _lib.ptr(self.tapes.meta), self.B, self.M, _lib.ptr(self.C_in), _lib.ptr(self.C_out),
                            self.M, 1, _lib.ptr(self.Y_out), _lib.ptr(self.iters), _lib.ptr(self.loss),
                            _lib.ptr(self.evals), _lib.ptr(self.order), self.max_len, self.tapes.max_consts, self.opts,
                            _lib.ptr(self.ws), self.ws.numel(), _lib.ptr(self.status),
                            _lib.stream_ptr(self.X.device))
        _lib.check(rc, "sr_fit_lbfgs")

    def capture(self) -> torch.cuda.CUDAGraph:
        """A CUDA graph of ``run`` (one warm-up run first, on a side stream)."""
        s = torch.cuda.Stream(device=self.X.device)
        s.wait_stream(torch.cuda.current_stream(self.X.device))
        with torch.cuda.stream(s):
            self.run()
        torch.cuda.current_stream(self.X.device).wait_stream(s)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.run()
        return g

    def result(self, raise_errors: bool = True) -> FitResult:
        """The outputs of the last run (reads the status word once)."""
        code = int(self.status.item())
        if code and raise_errors:
            ctx = "input validation" if code in (101, 102) else "symbolic evaluation backward pass"
            raise RuntimeError(error_message(code, ctx))
        return FitResult(C=self.C_out, Y=self.Y_out, iters=self.iters, loss=self.loss, evals=self.evals)
