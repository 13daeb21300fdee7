"""Seeded synthetic workloads with the shapes of the benchmark configurations.

* ``ragged_fit``: ragged batched L-BFGS -- B tapes of uniform length 3..64 with
  0..8 learnable constants, 2 variables, N points with X ~ U[-3, 3]; each target
  row is a hidden random expression from the same generator with N(0, 1)
  constants plus N(0, 0.01^2) noise.  Defaults: B=16384, N=512.  Tapes to be
  fitted have no EXP under a DIV denominator (see tapes.generate), so that the
  reference's batch-wide error 204 is not triggered by extrapolated steps.
* ``eval_batch``: forward+adjoint evaluation -- B=65536 tapes of padded length
  64 over {+,-,*,/,sin,cos,exp,log,X0..X3,C} with mean length about 20,
  X ~ U[-3, 3] (1024, 4), C ~ N(0, 1).

Hidden targets are evaluated with the library's own forward kernel; rows that
are not finite everywhere are redrawn.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np
import torch

from . import tapes
from .operators import Operator

# Floating-point operations per node and point, forward and adjoint, counted as
# FP32 add/mul = 1, FMA = 2, reciprocal/sqrt/transcendental unit op = 1, with the
# polynomial/range-reduction work of the accurate CUDA math routines counted in
# FMAs.  Used for the fit kernel's FLOP roofline.
FWD_FLOPS = {int(Operator.ADD): 1, int(Operator.SUB): 1, int(Operator.MUL): 1, int(Operator.DIV): 5,
             int(Operator.SIN): 20, int(Operator.COS): 20, int(Operator.EXP): 10, int(Operator.LOG): 16}
ADJ_FLOPS = {int(Operator.ADD): 2, int(Operator.SUB): 2, int(Operator.MUL): 4, int(Operator.DIV): 13,
             int(Operator.SIN): 22, int(Operator.COS): 22, int(Operator.EXP): 2, int(Operator.LOG): 6,
             int(Operator.LEARNABLE_CONSTANT): 1}


@dataclass
class FitWorkload:
    X: np.ndarray
    Y: np.ndarray
    ops: np.ndarray
    ch: np.ndarray
    C: np.ndarray
    name: str

    @property
    def B(self):
        return self.ops.shape[0]

    def flops_per_closure(self) -> np.ndarray:
        """(B,) algorithmic FLOPs of one closure (forward + adjoint over all N points)."""
        f = np.zeros(self.ops.shape, np.float64)
        for op, w in FWD_FLOPS.items():
            f += (self.ops == op) * w
        for op, w in ADJ_FLOPS.items():
            f += (self.ops == op) * w
        return f.sum(1) * self.X.shape[0]


def _gpu_roots(X, ops, ch, C, device="cuda"):
    """Root values (B, N) of each tape with the library's forward kernel."""
    from .evaluation import evaluate
    with torch.no_grad():
        cache = evaluate(torch.tensor(X, device=device), torch.tensor(ops, device=device),
                         torch.tensor(ch, device=device), torch.tensor(C, device=device))
        root = torch.tensor(np.maximum((ops != 0).sum(1) - 1, 0), device=device)
        return cache[torch.arange(ops.shape[0], device=device), root].cpu().numpy()


def ragged_fit(B: int = 16384, N: int = 512, M: int = 64, n_vars: int = 2, seed: int = 0,
               device: str = "cuda", root_eval=None, X: np.ndarray | None = None) -> FitWorkload:
    """root_eval(X, ops, ch, C) -> (B, N) root values of the hidden targets
    (default: the library's forward kernel on ``device``, which then also screens
    the tapes for zero denominators; with a root_eval given, everything runs on the
    host)."""
    screen = None
    if root_eval is None:
        root_eval = lambda X_, o, c, C_: _gpu_roots(X_, o, c, C_, device)  # noqa: E731
        screen = lambda o, c, Xs_, Cs_: _gpu_zero_denominators(Xs_, o, c, Cs_, device)  # noqa: E731
    rng = np.random.default_rng(seed)
    Xd = rng.uniform(-3, 3, (N, n_vars)).astype(np.float32)
    X = Xd if X is None else np.asarray(X, np.float32)
    C = rng.standard_normal((B, M)).astype(np.float32)
    lengths = rng.integers(3, M + 1, size=B)
    kc = rng.integers(0, 9, size=B)
    Xs = X[rng.choice(N, size=min(N, 32), replace=False)]
    tb = tapes.generate(B, M, seed=seed + 1, lengths=lengths, const_counts=kc, n_vars=n_vars,
                        X_screen=Xs, C_screen=C, no_exp_in_denominator=True, screen_fn=screen)
    # hidden target expressions
    Y = np.zeros((B, N), np.float32)
    todo = np.arange(B)
    for attempt in range(20):
        nb = todo.size
        hl = rng.integers(3, M + 1, size=nb)
        hk = rng.integers(0, 9, size=nb)
        Ch_ = rng.standard_normal((nb, M)).astype(np.float32)
        hid = tapes.generate(nb, M, seed=seed + 100 + attempt, lengths=hl, const_counts=hk, n_vars=n_vars,
                             X_screen=Xs, C_screen=Ch_, screen_fn=screen)
        yh = np.asarray(root_eval(X, hid.ops, hid.ch, Ch_), np.float32)
        ok = np.isfinite(yh).all(1) & (np.abs(yh).max(1) < 1e4)
        Y[todo[ok]] = yh[ok]
        todo = todo[~ok]
        if todo.size == 0:
            break
    Y[todo] = 0.0
    Y = (Y + 0.01 * rng.standard_normal((B, N))).astype(np.float32)
    return FitWorkload(X=X, Y=Y, ops=tb.ops, ch=tb.ch, C=C, name=f"ragged_fit_B{B}_N{N}_M{M}")


def ragged_fit_chunks(B: int, N: int = 512, M: int = 64, n_vars: int = 2, seed: int = 0, chunk: int = 4096,
                      n_chunks: int | None = None, device: str = "cuda", root_eval=None) -> FitWorkload:
    """The ragged workload built from chunks of `chunk` problems with seeds
    seed * 1000 + i that share one X (drawn from `seed`): the first chunks of a large
    batch are the same problems as a small batch, so a bounded CPU sample and the
    GPU batch can be compared problem by problem.  n_chunks limits how many are built."""
    X = np.random.default_rng(seed).uniform(-3, 3, (N, n_vars)).astype(np.float32)
    total = (B + chunk - 1) // chunk if n_chunks is None else n_chunks
    parts = []
    for i in range(total):
        b = min(chunk, B - i * chunk)
        parts.append(ragged_fit(B=b, N=N, M=M, n_vars=n_vars, seed=seed * 1000 + i, device=device,
                                root_eval=root_eval, X=X))
    cat = lambda k: np.concatenate([getattr(p, k) for p in parts])  # noqa: E731
    return FitWorkload(X=X, Y=cat("Y"), ops=cat("ops"), ch=cat("ch"), C=cat("C"),
                       name=f"ragged_fit_B{B}_N{N}_M{M}_chunks{chunk}")


@dataclass
class EvalWorkload:
    X: np.ndarray
    ops: np.ndarray
    ch: np.ndarray
    C: np.ndarray


def _gpu_zero_denominators(X, ops, ch, C, device="cuda", chunk=8192):
    """Tapes with a DIV whose denominator is exactly 0 at some row of X (device forward)."""
    from .evaluation import evaluate
    bad = np.zeros(ops.shape[0], bool)
    Xt = torch.tensor(X, device=device)
    for s in range(0, ops.shape[0], chunk):
        o = torch.tensor(ops[s:s + chunk], device=device)
        c = torch.tensor(ch[s:s + chunk], device=device)
        with torch.no_grad():
            cache = evaluate(Xt, o, c, torch.tensor(C[s:s + chunk], device=device))
        is_div = o == int(Operator.DIV)
        den = torch.gather(cache, 1, c[:, :, 1].clamp(min=0).unsqueeze(2).expand(-1, -1, cache.shape[2]))
        zero = ((den == 0).any(2) & is_div).any(1)
        bad[s:s + chunk] = zero.cpu().numpy()
        del cache, den
    return bad


def eval_batch(B: int = 65536, N: int = 1024, M: int = 64, n_vars: int = 4, seed: int = 0,
               device: str = "cuda") -> EvalWorkload:
    """Tapes whose DIV denominators are exactly 0 at some of the N rows are redrawn
    (the reference raises error 204 when such a node receives a gradient)."""
    rng = np.random.default_rng(seed)
    X = rng.uniform(-3, 3, (N, n_vars)).astype(np.float32)
    C = rng.standard_normal((B, M)).astype(np.float32)
    Xs = X[rng.choice(N, size=min(N, 32), replace=False)]
    tb = tapes.generate(B, M, seed=seed + 1, mean_length=20.0, n_vars=n_vars, p_const_leaf=0.2, X_screen=Xs,
                        C_screen=C)
    ops, ch = tb.ops, tb.ch
    for attempt in range(16):
        bad = np.where(_gpu_zero_denominators(X, ops, ch, C, device))[0]
        if bad.size == 0:
            break
        nb = tapes.generate(bad.size, M, seed=seed + 1000 + attempt, mean_length=20.0, n_vars=n_vars,
                            p_const_leaf=0.2, X_screen=Xs, C_screen=C[bad])
        ops[bad] = nb.ops
        ch[bad] = nb.ch
    return EvalWorkload(X=X, ops=ops, ch=ch, C=C)


def _readme_expression(rng: np.random.Generator, max_infix: int):
    """One postfix expression from the grammar
    E -> E + T (0.4) | T (0.6);  T -> F * T (0.4) | F (0.6);  F -> R(V) (0.3) | V (0.7);
    R -> sin (0.5) | cos (0.5);  V -> X_0 (0.5) | C (0.5),
    with its infix token count (parentheses included); None when the infix is longer
    than max_infix."""
    X0, C = 50, int(Operator.LEARNABLE_CONSTANT)
    SIN, COS, ADD, MUL = int(Operator.SIN), int(Operator.COS), int(Operator.ADD), int(Operator.MUL)

    def V():
        return [X0 if rng.random() < 0.5 else C], 1

    def F():
        if rng.random() < 0.3:
            r = SIN if rng.random() < 0.5 else COS
            v, n = V()
            return v + [r], n + 3
        return V()

    def T():
        post, n = F()
        rest = []
        while rng.random() < 0.4:  # T -> F * T: right-nested products
            f, m = F()
            rest.append(f)
            n += m + 1
        for f in rest:
            post = post + f
        return post + [MUL] * len(rest), n

    post, n = T()
    while rng.random() < 0.4:  # E -> E + T: left-nested sums
        t, m = T()
        post = post + t + [ADD]
        n += m + 1
    return (post, n) if n <= max_infix else None


# Candidate grammar of the sampling workload: +, -, *, /, sin, cos, exp, log over
# X_0..X_2 and learnable constants (about 12 infix tokens on average).
SEARCH_GRAMMAR = """E -> E + T [0.2]
E -> E - T [0.15]
E -> T [0.65]
T -> T * F [0.2]
T -> T / F [0.1]
T -> F [0.7]
F -> ( E ) [0.1]
F -> U ( E ) [0.2]
F -> V [0.7]
U -> sin [0.3]
U -> cos [0.3]
U -> exp [0.2]
U -> log [0.2]
V -> X_0 [0.25]
V -> X_1 [0.25]
V -> X_2 [0.2]
V -> C [0.3]
"""


def readme_fit(B: int = 1024, N: int = 100, M: int = 32, seed: int = 0) -> FitWorkload:
    """The README problem: expressions from the grammar above (infix capped at M
    tokens), X = 2 randn(N, 1), every target row 2.5 cos(X_0) - 1.5, C ~ N(0, 1)."""
    rng = np.random.default_rng(seed)
    X = (2.0 * rng.standard_normal((N, 1))).astype(np.float32)
    ops = np.zeros((B, M), np.int64)
    for b in range(B):
        e = None
        while e is None:
            e = _readme_expression(rng, M)
        ops[b, :len(e[0])] = e[0]
    arity = np.where(ops == 0, -1, np.where(ops >= 50, 0, np.where(ops == 1, 0, np.where(ops >= 40, 2, 1))))
    ch = tapes._children(arity.astype(np.int8))
    C = rng.standard_normal((B, M)).astype(np.float32)
    Y = np.tile((2.5 * np.cos(X[:, 0]) - 1.5).astype(np.float32), (B, 1))
    return FitWorkload(X=X, Y=Y, ops=ops, ch=ch, C=C, name=f"readme_fit_B{B}_N{N}_M{M}")
