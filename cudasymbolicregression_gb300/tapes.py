"""Seeded synthetic postfix tapes for the fitting and evaluation workloads.

The reference's PCFG sampler (src/pcfg_cuda.cu:10-146) caps the *infix* token
count, so it cannot produce long postfix tapes; the workloads here therefore use
this generator, which emits the reference's tensor layout directly:

* ``Ops`` (B, M) int64, left-packed postfix (root at L-1, NO_OP padding),
* ``Ch`` (B, M, 2) int64 child indices (-1 where absent), exactly the table the
  reference's ``get_postfix_children`` builds from the same Ops
  (src/pcfg_cuda.cu:1228-1300).

Shapes are drawn as random postfix arity sequences: at every position a leaf,
unary or binary symbol is chosen among those that can still close into a single
tree within the remaining length; symbols are then drawn uniformly from the
operator sets.  Tapes whose DIV denominators evaluate to exactly 0 at one of the
screening rows are redrawn (the reference raises error 204 on them).
Everything is vectorised over the batch with numpy and seeded.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from .operators import Operator

BIN_DEFAULT = (int(Operator.ADD), int(Operator.SUB), int(Operator.MUL), int(Operator.DIV))
UN_DEFAULT = (int(Operator.SIN), int(Operator.COS), int(Operator.EXP), int(Operator.LOG))


@dataclass
class TapeBatch:
    ops: np.ndarray      # (B, M) int64
    ch: np.ndarray       # (B, M, 2) int64
    lengths: np.ndarray  # (B,) int64
    n_consts: np.ndarray  # (B,) int64


def _shapes(rng: np.random.Generator, lengths: np.ndarray, M: int,
            p_leaf=0.4, p_un=0.2, p_bin=0.4) -> np.ndarray:
    """Random valid postfix arity sequences (0 leaf, 1 unary, 2 binary, -1 pad)."""
    B = lengths.shape[0]
    ar = np.full((B, M), -1, np.int8)
    depth = np.zeros(B, np.int64)
    for k in range(M):
        live = k < lengths
        r = lengths - k                      # steps left including this one
        # after a move the depth d' must satisfy 1 <= d' and d' - 1 <= r - 1
        ok_leaf = (depth + 1 - 1) <= (r - 1)
        ok_un = (depth >= 1) & ((depth - 1) <= (r - 1))
        ok_bin = (depth >= 2) & ((depth - 2) <= (r - 1))
        w = np.stack([ok_leaf * p_leaf, ok_un * p_un, ok_bin * p_bin], 1).astype(np.float64)
        s = w.sum(1)
        s[s == 0] = 1.0
        cum = np.cumsum(w / s[:, None], 1)
        u = rng.random(B)
        choice = (u[:, None] > cum).sum(1)
        choice = np.minimum(choice, 2)
        choice = np.where(live, choice, -1)
        ar[:, k] = choice
        depth = depth + np.where(choice == 0, 1, np.where(choice == 2, -1, 0)) * live
    return ar


def _children(ar: np.ndarray) -> np.ndarray:
    """Child table of left-packed postfix arity sequences (operand stack)."""
    B, M = ar.shape
    ch = np.full((B, M, 2), -1, np.int64)
    stack = np.zeros((B, M + 1), np.int64)
    sp = np.zeros(B, np.int64)
    rows = np.arange(B)
    for k in range(M):
        a = ar[:, k]
        un = a == 1
        bi = a == 2
        top = stack[rows, np.maximum(sp - 1, 0)]
        below = stack[rows, np.maximum(sp - 2, 0)]
        ch[un, k, 0] = top[un]
        ch[bi, k, 0] = below[bi]
        ch[bi, k, 1] = top[bi]
        sp = sp - un.astype(np.int64) - 2 * bi.astype(np.int64)
        push = a >= 0
        stack[rows[push], sp[push]] = k
        sp = sp + push
    return ch


def _screen_eval(ops: np.ndarray, ch: np.ndarray, X: np.ndarray, C: np.ndarray) -> np.ndarray:
    """Mask of tapes with a DIV whose denominator is exactly 0 at some row of X
    (float32, vectorised over B; the default operator sets plus SQUARE and NEG are
    modelled)."""
    B, M = ops.shape
    N = X.shape[0]
    vals = np.zeros((M, B, N), np.float32)
    bad = np.zeros(B, bool)
    rows = np.arange(B)
    with np.errstate(all="ignore"):
        for k in range(M):
            op = ops[:, k]
            a = vals[np.maximum(ch[:, k, 0], 0), rows]
            b = vals[np.maximum(ch[:, k, 1], 0), rows]
            v = np.full((B, N), np.nan, np.float32)
            var = op >= int(Operator.VAR_START_ID)
            v[var] = X[:, op[var] - int(Operator.VAR_START_ID)].T
            cst = op == int(Operator.LEARNABLE_CONSTANT)
            v[cst] = C[cst, k][:, None]
            for code, fn in ((Operator.ADD, lambda a, b: a + b), (Operator.SUB, lambda a, b: a - b),
                             (Operator.MUL, lambda a, b: a * b),
                             (Operator.DIV, lambda a, b: np.where(b == 0, np.nan, a / b)),
                             (Operator.SIN, lambda a, b: np.sin(a)), (Operator.COS, lambda a, b: np.cos(a)),
                             (Operator.EXP, lambda a, b: np.exp(a)),
                             (Operator.SQUARE, lambda a, b: a * a), (Operator.NEG, lambda a, b: -a),
                             (Operator.LOG, lambda a, b: np.where(a <= 0, np.nan, np.log(np.abs(a))))):
                m = op == int(code)
                if m.any():
                    v[m] = fn(a[m], b[m]).astype(np.float32)
            dm = op == int(Operator.DIV)
            if dm.any():
                bad[dm] |= (b[dm] == 0).any(1)
            vals[k] = v
    return bad


def _exp_under_div(ops: np.ndarray, ch: np.ndarray) -> np.ndarray:
    """Mask of tapes with an EXP node inside the denominator of a DIV.  exp of a
    fitted argument can underflow to exactly 0 (or overflow to inf, which turns an
    enclosing quotient into 0) while L-BFGS extrapolates, and the reference then
    raises error 204 for the whole batch."""
    B, M = ops.shape
    has = np.zeros((B, M), bool)
    bad = np.zeros(B, bool)
    rows = np.arange(B)
    for k in range(M):
        c0 = np.maximum(ch[:, k, 0], 0)
        c1 = np.maximum(ch[:, k, 1], 0)
        h0 = has[rows, c0] & (ch[:, k, 0] >= 0)
        h1 = has[rows, c1] & (ch[:, k, 1] >= 0)
        has[:, k] = (ops[:, k] == int(Operator.EXP)) | h0 | h1
        bad |= (ops[:, k] == int(Operator.DIV)) & h1
    return bad


def generate(B: int, M: int = 64, *, seed: int = 0, lengths=None, mean_length: float | None = None,
             n_vars: int = 4, binary=BIN_DEFAULT, unary=UN_DEFAULT, const_counts=None,
             p_const_leaf: float = 0.2, X_screen: np.ndarray | None = None,
             C_screen: np.ndarray | None = None, no_exp_in_denominator: bool = False,
             screen_fn=None) -> TapeBatch:
    """Draw B postfix tapes of padded length M.

    lengths: (B,) int array of exact tape lengths, or None to draw them from a
      geometric law with the given ``mean_length`` (clipped to [1, M]).
    const_counts: (B,) requested numbers of LEARNABLE_CONSTANT leaves (capped
      by the number of leaves); None makes every leaf a constant with
      probability ``p_const_leaf`` and otherwise a uniform variable.
    X_screen/C_screen: rows used to reject exact-zero denominators (None skips).
    no_exp_in_denominator: also redraw tapes with EXP under a DIV denominator.
    screen_fn(ops, ch, X_screen, C) -> (B,) bool: the zero-denominator test
      (default: a float32 numpy evaluation).
    """
    rng = np.random.default_rng(seed)
    if lengths is None:
        mean_length = 20.0 if mean_length is None else mean_length
        lengths = np.minimum(rng.geometric(1.0 / max(mean_length, 1.0), size=B), M)
    lengths = np.asarray(lengths, np.int64).clip(1, M)
    if const_counts is not None:
        const_counts = np.asarray(const_counts, np.int64)
    ops = np.zeros((B, M), np.int64)
    ch = np.full((B, M, 2), -1, np.int64)
    todo = np.arange(B)
    for _attempt in range(64):
        nb = todo.shape[0]
        ar = _shapes(rng, lengths[todo], M)
        o = np.zeros((nb, M), np.int64)
        leaf = ar == 0
        if const_counts is None:
            is_c = rng.random((nb, M)) < p_const_leaf
        else:
            # choose const_counts leaves uniformly among each tape's leaves
            key = np.where(leaf, rng.random((nb, M)), 2.0)
            rank = np.argsort(np.argsort(key, 1), 1)
            is_c = rank < const_counts[todo][:, None]
        varid = rng.integers(0, n_vars, size=(nb, M)) + int(Operator.VAR_START_ID)
        o[leaf] = np.where(is_c[leaf], int(Operator.LEARNABLE_CONSTANT), varid[leaf])
        un = ar == 1
        o[un] = np.asarray(unary, np.int64)[rng.integers(0, len(unary), size=int(un.sum()))]
        bi = ar == 2
        o[bi] = np.asarray(binary, np.int64)[rng.integers(0, len(binary), size=int(bi.sum()))]
        c = _children(ar)
        ops[todo] = o
        ch[todo] = c
        bad = _exp_under_div(o, c) if no_exp_in_denominator else np.zeros(nb, bool)
        if X_screen is None and not bad.any():
            break
        if X_screen is not None:
            Cs = np.zeros((nb, M), np.float32) if C_screen is None else np.asarray(C_screen, np.float32)[todo]
            bad |= (screen_fn or _screen_eval)(o, c, np.asarray(X_screen, np.float32), Cs)
        todo = todo[bad]
        if todo.size == 0:
            break
    nconst = (ops == int(Operator.LEARNABLE_CONSTANT)).sum(1)
    return TapeBatch(ops=ops, ch=ch, lengths=lengths, n_consts=nconst)
