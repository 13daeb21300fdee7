"""ctypes wrapper around ``oracle/sr_oracle.c``, the CPU restatement of the
reference's expression-fitting path.

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
bench.py's CPU-baseline leg, never by the package.  The shared library is built
by :func:`build` (gcc, OpenMP, ``-ffp-contract=off``) into ``oracle/``.

All arrays use the reference's user-facing layouts: X (N,nx), Ops (B,M),
Ch (B,M,2), C (B,M), cache (B,M,N), Y (B,N).
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sr_oracle.c")
# the kernels' own float math, compiled into the kernel-arithmetic mode
FMATH = os.path.join(os.path.dirname(HERE), "cudasymbolicregression_gb300", "csrc", "sr_fmath.h")
LIB = os.path.join(HERE, "libsr_oracle.so")

ERR_MESSAGES = {
    101: "Validation failed: A child's index is greater than or equal to its parent's.",
    102: "Validation failed: Operator arity does not match the number of children.",
    201: "Backward pass error: A non-zero gradient was passed to a NO_OP node.",
    204: "Backward pass error: Gradient for a/b where b = 0.",
}

_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle shared library (no-op when it is up to date)."""
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(SRC),
                                                                         os.path.getmtime(FMATH)):
        return LIB
    cmd = ["gcc", "-O2", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared",
           "-std=gnu11", SRC, "-o", LIB + ".tmp", "-lm"]
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        i64, vp, dbl = ctypes.c_int64, ctypes.c_void_p, ctypes.c_double
        L.sro_validate.argtypes = [vp, vp, i64, i64, i64, i64, i64, i64]
        L.sro_validate.restype = ctypes.c_int
        for suf in ("f32", "f64"):
            f = getattr(L, "sro_eval_fwd_" + suf)
            f.argtypes = [vp, i64, i64, vp, vp, vp, i64, i64, vp]
            f.restype = None
            g = getattr(L, "sro_eval_bwd_" + suf)
            g.argtypes = [vp, i64, i64, vp, vp, vp, i64, i64, vp, vp, vp]
            g.restype = ctypes.c_int
        L.sro_eval_fwd_kf32.argtypes = [vp, i64, i64, vp, vp, vp, i64, i64, vp]
        L.sro_eval_fwd_kf32.restype = None
        L.sro_eval_bwd_kf32.argtypes = [vp, i64, i64, vp, vp, vp, i64, i64, vp, vp, vp]
        L.sro_eval_bwd_kf32.restype = ctypes.c_int
        L.sro_eval_bwd_gc_kernel_order_f32.argtypes = [vp, i64, i64, vp, vp, vp, i64, i64, vp, vp, vp, vp, vp, vp]
        L.sro_eval_bwd_gc_kernel_order_f32.restype = ctypes.c_int
        L.sro_optimize_f32.argtypes = [vp, i64, i64, vp, vp, vp, vp, i64, i64, ctypes.c_int, ctypes.c_int,
                                       dbl, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp]
        L.sro_optimize_f32.restype = ctypes.c_int
        L.sro_optimize_shape_f32.argtypes = [vp, i64, i64, vp, vp, vp, vp, i64, i64, ctypes.c_int, ctypes.c_int,
                                             dbl, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                             ctypes.c_int, ctypes.c_int, vp, vp, vp, vp, vp]
        L.sro_optimize_shape_f32.restype = ctypes.c_int
        L.sro_num_threads.restype = ctypes.c_int
        L.sro_set_num_threads.argtypes = [ctypes.c_int]
        L.sro_set_num_threads.restype = ctypes.c_int
        L.sro_node_fwd_f32.argtypes = [i64, vp, vp, vp, vp, vp, vp]
        L.sro_node_fwd_f32.restype = None
        L.sro_node_fwd_kf32.argtypes = [i64, vp, vp, vp, vp, vp, vp]
        L.sro_node_fwd_kf32.restype = None
        L.sro_direction_f32.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, vp, vp,
                                        vp, dbl, vp]
        L.sro_direction_f32.restype = None
        L.sro_fmath_f32.argtypes = [ctypes.c_int, i64, vp, vp]
        L.sro_fmath_f32.restype = None
        L.sro_fmath_error.argtypes = [ctypes.c_int, ctypes.c_uint32, ctypes.c_uint32, ctypes.c_uint32, vp]
        L.sro_fmath_error.restype = None
        i32 = ctypes.c_int32
        L.sro_pcfg_sample.argtypes = [vp, vp, vp, vp, i32, i32, i64, i32, i32, ctypes.c_uint64, vp, vp]
        L.sro_pcfg_sample.restype = None
        L.sro_infix_parse.argtypes = [vp, i64, i64, i32, i32, vp, vp]
        L.sro_infix_parse.restype = None
        L.sro_postfix_children.argtypes = [vp, i64, i64, vp, vp]
        L.sro_postfix_children.restype = None
        for name in ("sro_postfix_to_infix", "sro_prefix_to_infix"):
            getattr(L, name).argtypes = [vp, i64, i64, i32, vp, i64, vp]
            getattr(L, name).restype = None
        L.sro_prefix_reorder.argtypes = [vp, i64, i64, i32, i32, vp, vp]
        L.sro_prefix_reorder.restype = None
        L.sro_prefix_parent.argtypes = [vp, i64, i64, i32, vp, vp]
        L.sro_prefix_parent.restype = None
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _c(a, dt):
    return np.ascontiguousarray(a, dtype=dt)


def validate(ops, ch) -> int:
    ops = _c(ops, np.int64)
    ch = _c(ch, np.int64)
    B, M = ops.shape
    return lib().sro_validate(_p(ops), _p(ch), B, M, M, 1, 2 * M, 2)


def eval_fwd(X, ops, ch, C, dtype=np.float32, kernel_math=False):
    """Node values (B,M,N) of every tape at every point; kernel_math (float32) takes
    sin, cos, exp and log from the kernels' own functions (sr_fmath.h)."""
    X = _c(X, dtype)
    ops = _c(ops, np.int64)
    ch = _c(ch, np.int64)
    C = _c(C, dtype)
    N, nx = X.shape
    B, M = ops.shape
    out = np.empty((B, M, N), dtype=dtype)
    fn = lib().sro_eval_fwd_f32 if dtype == np.float32 else lib().sro_eval_fwd_f64
    if kernel_math:
        assert dtype == np.float32
        fn = lib().sro_eval_fwd_kf32
    fn(_p(X), N, nx, _p(ops), _p(ch), _p(C), B, M, _p(out))
    return out


def eval_gc_kernel_order(X, ops, ch, C, gout, gx_terms=False):
    """grad_C (B, M) of the evaluation adjoint for a dense output gradient, with the
    kernels' own sin/cos/exp/log and in the device kernel's summation order (per lane
    over the points l, l + 32, ..., then a 32-lane xor butterfly); returns (gC, err).

    With gx_terms, returns (gC, err, terms): terms describes, per (point, variable), the
    nonzero variable-node adjoints that the device adds atomically into grad_X (in no
    fixed order): "sum" (float64 sum of the finite ones), "abs" (sum of their
    magnitudes), "count" (all of them) and "flags" (bit 0 NaN, bit 1 +inf, bit 2 -inf
    among them).  check_gx_bound compares a grad_X against them."""
    X = _c(X, np.float32)
    ops = _c(ops, np.int64)
    ch = _c(ch, np.int64)
    C = _c(C, np.float32)
    gout = _c(gout, np.float32)
    N, nx = X.shape
    B, M = ops.shape
    gC = np.zeros((B, M), np.float32)
    if not gx_terms:
        err = lib().sro_eval_bwd_gc_kernel_order_f32(_p(X), N, nx, _p(ops), _p(ch), _p(C), B, M, _p(gout), _p(gC),
                                                     None, None, None, None)
        return gC, err
    assert B * N * nx <= 1 << 26, "gx_terms keeps per-tape partials: keep B * N * n_x small"
    t = {"sum": np.zeros((N, nx), np.float64), "abs": np.zeros((N, nx), np.float64),
         "count": np.zeros((N, nx), np.int32), "flags": np.zeros((N, nx), np.int32)}
    err = lib().sro_eval_bwd_gc_kernel_order_f32(_p(X), N, nx, _p(ops), _p(ch), _p(C), B, M, _p(gout), _p(gC),
                                                 _p(t["sum"]), _p(t["abs"]), _p(t["count"]), _p(t["flags"]))
    return gC, err, t


def check_gx_bound(gx, terms):
    """Whether a float32 grad_X (N, nx) is a float32 sum, in some order, of the terms that
    eval_gc_kernel_order(..., gx_terms=True) describes, added to a zeroed buffer.

    Non-finite entries: NaN where a term is NaN or both infinities occur, +inf / -inf
    where only that infinity occurs.  Finite entries: recursive summation of n terms in
    any order errs by at most gamma(n - 1) = (n - 1) u / (1 - (n - 1) u) times the sum of
    their magnitudes (u = 2^-24; Higham, Accuracy and Stability of Numerical Algorithms,
    2nd ed., section 4.2), plus n 2^-125 for subnormal inputs and partial sums flushed to
    zero (the device's float atomic add flushes them) and n 2^-53 of the magnitudes for
    the float64 reference sum.  Returns (ok mask, slack = error / bound)."""
    gx = np.asarray(gx, np.float32).astype(np.float64)
    s, a, n, f = terms["sum"], terms["abs"], terms["count"].astype(np.float64), terms["flags"]
    want_nan = (f & 1).astype(bool) | ((f & 6) == 6)
    want_pinf = ~want_nan & ((f & 6) == 2)
    want_ninf = ~want_nan & ((f & 6) == 4)
    fin = ~(want_nan | want_pinf | want_ninf)
    u = 2.0 ** -24
    k = np.maximum(n - 1, 0)
    bound = k * u / (1 - k * u) * a + n * 2.0 ** -125 + n * 2.0 ** -53 * a
    err = np.abs(gx - s)
    ok = np.where(want_nan, np.isnan(gx), False)
    ok |= want_pinf & (gx == np.inf)
    ok |= want_ninf & (gx == -np.inf)
    with np.errstate(invalid="ignore"):
        ok |= fin & np.isfinite(gx) & (err <= bound)
        slack = np.where(fin & (bound > 0), err / np.where(bound > 0, bound, 1.0), 0.0)
    return ok, slack


def eval_bwd(X, ops, ch, C, gout, dtype=np.float32, want_gx=True, kernel_math=False):
    """Adjoint sweep for a dense (B,M,N) output gradient -> (gC (B,M), gX (N,nx), err);
    kernel_math (float32) takes sin, cos, exp and log from the kernels' own functions."""
    X = _c(X, dtype)
    ops = _c(ops, np.int64)
    ch = _c(ch, np.int64)
    C = _c(C, dtype)
    gout = _c(gout, dtype)
    N, nx = X.shape
    B, M = ops.shape
    gC = np.zeros((B, M), dtype=dtype)
    gX = np.zeros((N, nx), dtype=dtype) if want_gx else None
    fn = lib().sro_eval_bwd_f32 if dtype == np.float32 else lib().sro_eval_bwd_f64
    if kernel_math:
        assert dtype == np.float32
        fn = lib().sro_eval_bwd_kf32
    err = fn(_p(X), N, nx, _p(ops), _p(ch), _p(C), B, M, _p(gout), _p(gC), _p(gX))
    return gC, gX, err


def eval_fwd_multi(X, ops, ch, C3, dtype=np.float32):
    """evaluate_multiple: (B,M,N,K) node values for K constant sets C3 (B,M,K).  The
    reference evaluates every set with the single-set operator policies
    (src/evaluation_kernels_cpu.cpp multiple-constant kernels), so each set is one
    single-set evaluation here."""
    C3 = np.asarray(C3)
    return np.stack([eval_fwd(X, ops, ch, C3[:, :, k], dtype) for k in range(C3.shape[2])], axis=3)


def eval_bwd_multi(X, ops, ch, C3, gout4, dtype=np.float32, want_gx=True):
    """Adjoint of evaluate_multiple for a dense (B,M,N,K) output gradient ->
    (gC (B,M,K), gX (N,nx) summed over the sets, first error code)."""
    C3 = np.asarray(C3)
    gout4 = np.asarray(gout4)
    gCs, gX, err = [], None, 0
    for k in range(C3.shape[2]):
        gC, gx, e = eval_bwd(X, ops, ch, C3[:, :, k], gout4[..., k], dtype, want_gx)
        gCs.append(gC)
        err = err or e
        if want_gx:
            gX = gx if gX is None else gX + gx
    return np.stack(gCs, axis=2), gX, err


def kernel_slot_registers(ops, M=None):
    """Slot registers per lane of the fused fit kernel for a batch: 1, 2 or 4 (one
    register holds 32 slots: the largest count of constants up to the root, plus the
    virtual slot)."""
    ops = np.asarray(ops)
    nz = (ops != 0).sum(1)
    root = np.maximum(nz - 1, 0)
    pos = np.arange(ops.shape[1])[None, :]
    kmax = int(((ops == 1) & (pos <= root[:, None])).sum(1).max()) if ops.size else 0
    return 1 if kmax + 1 <= 32 else (2 if kmax + 1 <= 64 else 4)


def optimize(X, Y, ops, ch, C_init, max_iter=100, history_size=10, tolerance_grad=1e-7,
             line_search_fn="strong_wolfe", line_search_max_iter=10, dot_mode=1, warps=1,
             points_per_lane=1, slot_registers=None):
    """Per-problem restatement of ``symbolic_torch.optimize``.

    dot_mode=0 follows the reference's float32 arithmetic; dot_mode=1 approximates
    the fused kernel's (double dots and two-loop scalars, where the kernel uses
    float pairs); dot_mode=2 is the fused kernel's arithmetic exactly for a launch
    shape of `warps` warps per problem and `points_per_lane` points per lane (its
    per-lane sums, lane and warp reduction order, float-pair dots, its direction --
    the compact representation up to 32 pairs of history, the two-loop recursion
    beyond -- slot vectors and closure count; slot_registers defaults to the batch's
    own, as the kernel derives it).
    Returns dict(C, Y, iters, evals, loss, err); iters[b] = -code for a problem
    whose closures raised an error.  Y=None selects the raw
    objective (mean of the root value) used by the Rosenbrock test.
    """
    X = _c(X, np.float32)
    ops = _c(ops, np.int64)
    ch = _c(ch, np.int64)
    C_init = _c(C_init, np.float32)
    Yc = None if Y is None else _c(np.broadcast_to(Y, (ops.shape[0], X.shape[0])), np.float32)
    N, nx = X.shape
    B, M = ops.shape
    C = np.empty((B, M), np.float32)
    Yo = np.empty((B, N), np.float32)
    iters = np.empty(B, np.int32)
    evals = np.empty(B, np.int64)
    loss = np.empty(B, np.float32)
    ls = {"strong_wolfe": 0, "backtracking": 1}[line_search_fn]
    spl = kernel_slot_registers(ops) if slot_registers is None else int(slot_registers)
    err = lib().sro_optimize_shape_f32(_p(X), N, nx, _p(Yc), _p(ops), _p(ch), _p(C_init), B, M,
                                       int(max_iter), int(history_size), float(tolerance_grad), ls,
                                       int(line_search_max_iter), int(dot_mode), int(warps), int(points_per_lane),
                                       spl, _p(C), _p(Yo), _p(iters), _p(evals), _p(loss))
    return dict(C=C, Y=Yo, iters=iters, evals=evals, loss=loss, err=err)


def direction(S, Y, g, history_size, nslots, two_loop=False, eps=1e-10):
    """The fused kernel's search direction p = -H g after the pairs S, Y (npairs, 32 spl)
    float32 rows, oldest first) pass through its history ring of history_size pairs:
    the compact representation (two lanes per pair up to 16 pairs) or, with two_loop or
    above 32 pairs, the two-loop recursion.  Returns p (32 spl,) float32."""
    S = _c(S, np.float32)
    Y = _c(Y, np.float32)
    g = _c(g, np.float32)
    n, D = S.shape
    spl = D // 32
    p = np.zeros(D, np.float32)
    lib().sro_direction_f32(int(history_size), int(bool(two_loop)), spl, int(nslots), n, _p(S), _p(Y), _p(g),
                            float(eps), _p(p))
    return p


def node_fwd(op, a, b, c, x, kernel_math=False):
    """Elementwise single-node forward (float32) of flat arrays; kernel_math takes sin,
    cos, exp and log from the kernels' own functions (sr_fmath.h) instead of libm."""
    op = _c(op, np.int64)
    a, b, c, x = (_c(v, np.float32) for v in (a, b, c, x))
    out = np.empty(op.shape, np.float32)
    fn = lib().sro_node_fwd_kf32 if kernel_math else lib().sro_node_fwd_f32
    fn(op.size, _p(op), _p(a), _p(b), _p(c), _p(x), _p(out))
    return out


FMATH_FN = {"sin": 0, "cos": 1, "exp": 2, "log": 3}


def fmath(name, x):
    """The kernels' own float32 sin, cos, exp or log (sr_fmath.h) on the host."""
    x = _c(x, np.float32)
    y = np.empty_like(x)
    lib().sro_fmath_f32(FMATH_FN[name], x.size, _p(x), _p(y))
    return y


def fmath_error(name, lo_bits, hi_bits, step=1):
    """Largest error in ulps of the kernels' float32 function over the inputs whose bit
    patterns run from lo_bits to hi_bits in steps of `step`, against the double
    function: (max ulp, input at the max, special-value mismatches, inputs checked)."""
    out = np.zeros(4)
    lib().sro_fmath_error(FMATH_FN[name], int(lo_bits), int(hi_bits), int(step), _p(out))
    return float(out[0]), float(out[1]), int(out[2]), int(out[3])


def pcfg_sample(tables, start, B, max_len, max_tries, seed):
    """Restatement of the grammar sampler (src/pcfg_cpu.cpp:10-119) with the
    library's SplitMix64 stream.  tables = (nt_rule_ptr, cum_probs, rhs_ptr,
    rhs_concat) as numpy arrays.  Returns (infix (B, max_len) int64, errors (B))."""
    nt, cum, rp, rc = (_c(tables[0], np.int32), _c(tables[1], np.float32), _c(tables[2], np.int32),
                       _c(tables[3], np.int32))
    out = np.empty((B, max_len), np.int64)
    err = np.empty(B, np.int64)
    lib().sro_pcfg_sample(_p(nt), _p(cum), _p(rp), _p(rc), int(nt.size - 1), int(start), int(B), int(max_len),
                          int(max_tries), int(seed) & 0xFFFFFFFFFFFFFFFF, _p(out), _p(err))
    return out, err


def infix_parse(infix, n_vars, prefix=False):
    """Restatement of infix_to_postfix / infix_to_prefix (src/pcfg_cpu.cpp:121-448).
    Returns (tokens (B, M) int64, errors (B))."""
    x = _c(infix, np.int64)
    B, M = x.shape
    out = np.empty((B, M), np.int64)
    err = np.empty(B, np.int64)
    lib().sro_infix_parse(_p(x), B, M, int(n_vars), int(bool(prefix)), _p(out), _p(err))
    return out, err


def postfix_children(post):
    """Restatement of get_postfix_children (src/pcfg_cpu.cpp:1066-1142).
    Returns (ch (B, M, 2) int64, errors (B))."""
    x = _c(post, np.int64)
    B, M = x.shape
    ch = np.empty((B, M, 2), np.int64)
    err = np.empty(B, np.int64)
    lib().sro_postfix_children(_p(x), B, M, _p(ch), _p(err))
    return ch, err


def to_infix(rows, n_vars, max_infix_len, prefix=False):
    """Restatement of postfix_to_infix / prefix_to_infix (src/pcfg_cpu.cpp:449-811).
    Returns (infix (B, max_infix_len) int64, errors (B))."""
    x = _c(rows, np.int64)
    B, M = x.shape
    out = np.empty((B, int(max_infix_len)), np.int64)
    err = np.empty(B, np.int64)
    fn = lib().sro_prefix_to_infix if prefix else lib().sro_postfix_to_infix
    fn(_p(x), B, M, int(n_vars), _p(out), int(max_infix_len), _p(err))
    return out, err


def reorder(rows, n_vars, from_prefix):
    """Restatement of prefix_to_postfix (from_prefix) and postfix_to_prefix
    (src/pcfg_cpu.cpp:812-993).  Returns (tokens (B, M) int64, errors (B))."""
    x = _c(rows, np.int64)
    B, M = x.shape
    out = np.empty((B, M), np.int64)
    err = np.empty(B, np.int64)
    lib().sro_prefix_reorder(_p(x), B, M, int(n_vars), int(bool(from_prefix)), _p(out), _p(err))
    return out, err


def prefix_parent(rows, n_vars):
    """Restatement of get_prefix_parent (src/pcfg_cpu.cpp:995-1064).
    Returns (parents (B, M) int64, -1 for roots and padding; errors (B))."""
    x = _c(rows, np.int64)
    B, M = x.shape
    out = np.empty((B, M), np.int64)
    err = np.empty(B, np.int64)
    lib().sro_prefix_parent(_p(x), B, M, int(n_vars), _p(out), _p(err))
    return out, err


def num_threads() -> int:
    return lib().sro_num_threads()


def set_num_threads(n: int) -> int:
    """OpenMP threads of the oracle's parallel loops; returns the count in effect."""
    return lib().sro_set_num_threads(int(n))
