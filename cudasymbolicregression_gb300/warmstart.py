"""Learned warm start for ``optimize``: a BF16 MLP that predicts starting constants.

The network reads a tape as a bag of tokens (token frequencies through a 64-wide
embedding) and its target row through 32 summary features (four moments of Y and
the projections of the standardised Y on 28 fixed seeded random features of X),
and predicts the first ``N_OUT`` learnable constants of the tape (row-major order):

    hist (64) --E--> emb (64) ; x0 = [emb | feats (32) | 0 (32)]
    x0 --W1,b1,ReLU--> h1 (256) --W2,b2,ReLU--> h2 --W3,b3,ReLU--> h3 --W4,b4--> out (8, padded to 64)

Weights and activations are bf16, every GEMM accumulates in fp32 on the tensor
cores (``sr_mlp_gemm``), master weights and Adam moments are fp32.  Training runs in
two stages: ``train`` minimises the squared error against the constants that
``optimize`` itself found, on the problems it fitted well; ``train_fit_objective``
then back-propagates the fit's own objective (the normalised MSE of each expression at
the predicted constants, through the library's forward and adjoint kernels) into the
network.  ``warm_start_constants`` puts the predictions in the first learnable slots of
C and keeps the plain ``create_constants``-style draw everywhere else;
``gated_warm_start`` (``candidate_starts`` + ``screened_start``) scores that start and
the plain one in one launch of the screening kernel and keeps, per problem, the one
with the lower initial loss (the plain start on ties), so the plain initialisation
stays the fallback and the judge.

There is no counterpart in the reference; everything here runs on the library's
own kernels (declared in include/sr_gb300.h).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib

N_OUT = 8
HIDDEN = 256
OUT_PAD = 64
VOCAB, EMB, FEATS, PROJ, IN = _lib.MLP_VOCAB, _lib.MLP_EMB, _lib.MLP_FEATS, _lib.MLP_PROJ, _lib.MLP_IN
TILE = 128

# layer name -> (out rows, in cols, has bias)
LAYERS = {
    "E": (EMB, VOCAB, False),
    "W1": (HIDDEN, IN, True),
    "W2": (HIDDEN, HIDDEN, True),
    "W3": (HIDDEN, HIDDEN, True),
    "W4": (OUT_PAD, HIDDEN, True),
}


def _pad_rows(n: int) -> int:
    return max(TILE, (n + TILE - 1) // TILE * TILE)


def _p(t):
    return None if t is None else ctypes.c_void_p(t.data_ptr())


class _Workspace:
    """Activation and gradient buffers for batches of up to R rows (R a multiple of 128).
    Zero-filled once: padding rows and columns stay zero."""

    def __init__(self, R: int, device, splits: int):
        z = lambda *s: torch.zeros(*s, dtype=torch.bfloat16, device=device)  # noqa: E731
        f = lambda *s: torch.zeros(*s, dtype=torch.float32, device=device)  # noqa: E731
        self.R = R
        self.hist, self.hist_t = z(R, VOCAB), z(VOCAB, R)
        self.x0, self.x0_t = z(R, IN), z(IN, R)
        self.feats = f(R, FEATS)
        self.h = {i: (z(R, HIDDEN), z(HIDDEN, R)) for i in (1, 2, 3)}
        self.out = f(R, OUT_PAD)
        self.target, self.mask, self.row_loss = f(R, N_OUT), f(R, N_OUT), f(R)
        self.d_out, self.d_out_t = z(R, OUT_PAD), z(TILE, R)
        self.dz = {i: (z(R, HIDDEN), z(HIDDEN, R)) for i in (1, 2, 3)}
        self.dx0_t = z(IN, R)
        self.splits = splits
        self.part = f(splits, HIDDEN, HIDDEN)
        self.status = torch.zeros(1, dtype=torch.int32, device=device)


@dataclass
class TrainStats:
    steps: int
    loss: list


class WarmStartMLP:
    """The warm-start network with its training step (all on ``sr_mlp_*`` kernels)."""

    def __init__(self, device="cuda", seed: int = 0, n_vars: int = 2):
        self.device = torch.device(device)
        self.n_vars = n_vars
        g = torch.Generator().manual_seed(seed)
        self.w, self.b = {}, {}
        for name, (o, i, has_b) in LAYERS.items():
            real_o = N_OUT if name == "W4" else o
            real_i = EMB + FEATS if name == "W1" else i
            std = 0.01 if name == "W4" else (2.0 / real_i) ** 0.5
            w = torch.zeros(o, i)
            w[:real_o, :real_i] = torch.randn(real_o, real_i, generator=g) * std
            self.w[name] = w.to(self.device)
            if has_b:
                self.b[name] = torch.zeros(o, device=self.device)
        self.w_bf = {n: torch.zeros(LAYERS[n][0], LAYERS[n][1], dtype=torch.bfloat16, device=self.device)
                     for n in LAYERS}
        self.w_bf_t = {n: torch.zeros(LAYERS[n][1], LAYERS[n][0], dtype=torch.bfloat16, device=self.device)
                       for n in LAYERS}
        self.m = {k: torch.zeros_like(v) for k, v in self.w.items()}
        self.v = {k: torch.zeros_like(v) for k, v in self.w.items()}
        self.mb = {k: torch.zeros_like(v) for k, v in self.b.items()}
        self.vb = {k: torch.zeros_like(v) for k, v in self.b.items()}
        self.gw = {k: torch.zeros_like(v) for k, v in self.w.items()}
        self.gb = {k: torch.zeros_like(v) for k, v in self.b.items()}
        self.step_count = 0
        # random features of X: omega (PROJ, n_vars) ~ N(0, 1), beta ~ U[0, 2 pi)
        rng = np.random.default_rng(seed + 7919)
        self.omega = torch.tensor(rng.standard_normal((PROJ, n_vars)).astype(np.float32), device=self.device)
        self.beta = torch.tensor(rng.uniform(0, 2 * np.pi, PROJ).astype(np.float32), device=self.device)
        self._ws = None
        self._pack()

    # ---- kernels -------------------------------------------------------------------
    def _lib(self):
        return _lib.lib()

    def _stream(self):
        return _lib.stream_ptr(self.device)

    def _gemm(self, A, rows, k, lda, W, n, ldw, ws, **epi):
        e = _lib.MlpEpilogue()
        e.epilogue = epi.get("mode", _lib.MLP_EPI_LINEAR)
        e.splits = epi.get("splits", 1)
        e.bias = _p(epi.get("bias"))
        e.gate = _p(epi.get("gate"))
        e.ld_gate = epi.get("ld_gate", 0)
        e.out = _p(epi.get("out"))
        e.ld_out = epi.get("ld_out", 0)
        e.out_col0 = epi.get("out_col0", 0)
        e.out_t = _p(epi.get("out_t"))
        e.ld_out_t = epi.get("ld_out_t", 0)
        e.out_t_row0 = epi.get("out_t_row0", 0)
        e.out_f32 = _p(epi.get("out_f32"))
        e.ld_out_f32 = epi.get("ld_out_f32", 0)
        e.split_stride = epi.get("split_stride", 0)
        rc = self._lib().sr_mlp_gemm(_p(A), rows, k, lda, _p(W), n, ldw, ctypes.byref(e), _p(ws.status),
                                     self._stream())
        _lib.check(rc, "sr_mlp_gemm")

    def _pack(self):
        L = self._lib()
        for n in LAYERS:
            o, i, _ = LAYERS[n]
            _lib.check(L.sr_mlp_adam(_p(self.w[n]), None, None, None, o, i, 0.0, 0.9, 0.999, 1e-8, 0.0, 0,
                                     _p(self.w_bf[n]), _p(self.w_bf_t[n]), self._stream()), "sr_mlp_adam")

    def workspace(self, rows: int) -> _Workspace:
        R = _pad_rows(rows)
        if self._ws is None or self._ws.R < R:
            self._ws = _Workspace(R, self.device, splits=min(64, R // 64))
        return self._ws

    # ---- forward -------------------------------------------------------------------
    def features(self, ops: torch.Tensor, X: torch.Tensor, Y: torch.Tensor, ws: _Workspace):
        """Fill the input rows of ``ws`` for the problems (ops (B, M) int64, Y (B, N))."""
        L = self._lib()
        B, M = ops.shape
        N = X.shape[0]
        if X.shape[1] != self.n_vars:
            raise RuntimeError(f"the network was built for {self.n_vars} variables, X has {X.shape[1]}")
        Xc, Yc = X.contiguous().float(), Y.contiguous().float()
        phi = torch.empty(N, PROJ, dtype=torch.float32, device=self.device)
        _lib.check(L.sr_mlp_random_features(_p(Xc), N, Xc.shape[1], _p(self.omega), _p(self.beta), _p(phi),
                                            self._stream()), "sr_mlp_random_features")
        sb, sm = ops.stride()
        _lib.check(L.sr_mlp_features(_p(ops), B, M, sb, sm, _p(Yc), N, _p(phi), _p(ws.hist), _p(ws.hist_t), ws.R,
                                     _p(ws.x0), _p(ws.x0_t), _p(ws.feats), self._stream()), "sr_mlp_features")

    def forward_ws(self, ws: _Workspace, rows: int):
        R, ld = _pad_rows(rows), ws.R  # rows processed; leading dimension of the transposed buffers
        # embedding of the bag of tokens -> x0[:, :64] and x0_t[:64]
        self._gemm(ws.hist, R, VOCAB, VOCAB, self.w_bf["E"], EMB, VOCAB, ws, mode=_lib.MLP_EPI_LINEAR,
                   out=ws.x0, ld_out=IN, out_col0=0, out_t=ws.x0_t, ld_out_t=ld, out_t_row0=0)
        prev, k = ws.x0, IN
        for i, name in ((1, "W1"), (2, "W2"), (3, "W3")):
            h, h_t = ws.h[i]
            self._gemm(prev, R, k, k, self.w_bf[name], HIDDEN, k, ws, mode=_lib.MLP_EPI_RELU, bias=self.b[name],
                       out=h, ld_out=HIDDEN, out_t=h_t, ld_out_t=ld)
            prev, k = h, HIDDEN
        self._gemm(prev, R, HIDDEN, HIDDEN, self.w_bf["W4"], OUT_PAD, HIDDEN, ws, mode=_lib.MLP_EPI_F32,
                   bias=self.b["W4"], out_f32=ws.out, ld_out_f32=OUT_PAD)
        return ws.out[:rows, :N_OUT]

    # ---- backward ------------------------------------------------------------------
    def _weight_grad(self, A_t, a_rows, B_t, n, R, ws, dst):
        """dst (a_rows_real x n) = A_t (a_rows x R) . B_t (n x R)^T with a split reduction
        (A_t and B_t have leading dimension ws.R)."""
        L = self._lib()
        splits = L.sr_mlp_gemm_splits_used(R, ws.splits)
        stride = TILE * ((a_rows + TILE - 1) // TILE) * n
        part = ws.part.view(-1)[: splits * stride].view(splits, -1)
        e = _lib.MlpEpilogue()
        e.epilogue = _lib.MLP_EPI_SPLIT_F32
        e.splits = ws.splits
        e.out_f32 = _p(part)
        e.ld_out_f32 = n
        e.split_stride = stride
        _lib.check(L.sr_mlp_gemm(_p(A_t), a_rows, R, ws.R, _p(B_t), n, ws.R, ctypes.byref(e), _p(ws.status),
                                 self._stream()), "sr_mlp_gemm")
        count = dst.numel()
        _lib.check(L.sr_mlp_reduce_splits(_p(part), splits, count, stride, _p(dst), self._stream()),
                   "sr_mlp_reduce_splits")

    def backward_ws(self, ws: _Workspace, rows: int, out_grad: torch.Tensor | None = None):
        """Gradients into self.gw / self.gb of the mean over rows of sum_j mask (out - target)^2,
        or, with out_grad (rows, N_OUT) fp32 given, of a loss whose gradient with
        respect to the outputs is out_grad / rows."""
        L = self._lib()
        R, ld = _pad_rows(rows), ws.R
        st = self._stream()
        if out_grad is None:
            _lib.check(L.sr_mlp_loss(_p(ws.out), R, OUT_PAD, _p(ws.target), _p(ws.mask), N_OUT, 1.0 / max(rows, 1),
                                     _p(ws.row_loss), _p(ws.d_out), OUT_PAD, _p(ws.d_out_t), ld, st), "sr_mlp_loss")
        else:
            g = torch.zeros(R, N_OUT, dtype=torch.float32, device=self.device)
            g[:rows] = out_grad
            _lib.check(L.sr_mlp_output_grad(_p(g), R, N_OUT, N_OUT, 1.0 / max(rows, 1), _p(ws.d_out), OUT_PAD,
                                            _p(ws.d_out_t), ld, st), "sr_mlp_output_grad")
        # output layer
        self._weight_grad(ws.d_out_t, TILE, ws.h[3][1], HIDDEN, R, ws, self.gw["W4"])
        _lib.check(L.sr_mlp_colsum(_p(ws.d_out_t), OUT_PAD, R, ld, _p(self.gb["W4"]), st), "sr_mlp_colsum")
        dz_prev, k_prev = ws.d_out, OUT_PAD
        for i, name, below in ((3, "W3", 2), (2, "W2", 1), (1, "W1", 0)):
            up = {3: "W4", 2: "W3", 1: "W2"}[i]
            dz, dz_t = ws.dz[i]
            h = ws.h[i][0]
            # dh_i = dz_{i+1} . W_{i+1}, gated by ReLU'(h_i)
            self._gemm(dz_prev, R, k_prev, k_prev, self.w_bf_t[up], HIDDEN, k_prev, ws,
                       mode=_lib.MLP_EPI_RELU_GRAD, gate=h, ld_gate=HIDDEN, out=dz, ld_out=HIDDEN, out_t=dz_t,
                       ld_out_t=ld)
            a_t, n_in = (ws.h[below][1], HIDDEN) if below else (ws.x0_t, IN)
            self._weight_grad(dz_t, HIDDEN, a_t, n_in, R, ws, self.gw[name])
            _lib.check(L.sr_mlp_colsum(_p(dz_t), HIDDEN, R, ld, _p(self.gb[name]), st), "sr_mlp_colsum")
            dz_prev, k_prev = dz, HIDDEN
        # d x0 = dz_1 . W1 (transposed copy only); its first 64 rows are d(embedding)
        self._gemm(ws.dz[1][0], R, HIDDEN, HIDDEN, self.w_bf_t["W1"], IN, HIDDEN, ws, mode=_lib.MLP_EPI_LINEAR,
                   out_t=ws.dx0_t, ld_out_t=ld)
        gE = torch.empty(TILE, VOCAB, device=self.device)
        self._weight_grad(ws.dx0_t, TILE, ws.hist_t, VOCAB, R, ws, gE)
        self.gw["E"].copy_(gE[:EMB])
        return ws.row_loss[:rows]

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
        L = self._lib()
        self.step_count += 1
        st = self._stream()
        for n in LAYERS:
            o, i, has_b = LAYERS[n]
            _lib.check(L.sr_mlp_adam(_p(self.w[n]), _p(self.gw[n]), _p(self.m[n]), _p(self.v[n]), o, i, lr, beta1,
                                     beta2, eps, weight_decay, self.step_count, _p(self.w_bf[n]),
                                     _p(self.w_bf_t[n]), st), "sr_mlp_adam")
            if has_b:
                _lib.check(L.sr_mlp_adam(_p(self.b[n]), _p(self.gb[n]), _p(self.mb[n]), _p(self.vb[n]), 1, o, lr,
                                         beta1, beta2, eps, 0.0, self.step_count, None, None, st), "sr_mlp_adam")

    def check_status(self):
        if self._ws is not None and int(self._ws.status.item()) != 0:
            raise RuntimeError(f"warm-start GEMM pipeline wait ran out (status {int(self._ws.status.item())})")

    # ---- user-facing ---------------------------------------------------------------
    def predict(self, ops: torch.Tensor, X: torch.Tensor, Y: torch.Tensor, chunk: int = 65536) -> torch.Tensor:
        """(B, N_OUT) predicted constants (fp32)."""
        _lib.require_cuda(ops, X, Y)
        B = ops.shape[0]
        out = torch.empty(B, N_OUT, dtype=torch.float32, device=self.device)
        for s in range(0, B, chunk):
            e = min(B, s + chunk)
            ws = self.workspace(e - s)
            self.features(ops[s:e], X, Y[s:e], ws)
            out[s:e] = self.forward_ws(ws, e - s)
        return out

    def train_batch(self, ops, X, Y, target, mask, lr=1e-3, weight_decay=0.0) -> torch.Tensor:
        """One Adam step on a batch; returns the per-row losses (device tensor)."""
        rows = ops.shape[0]
        ws = self.workspace(rows)
        ws.target.zero_()
        ws.mask.zero_()
        ws.target[:rows] = target
        ws.mask[:rows] = mask
        self.features(ops, X, Y, ws)
        self.forward_ws(ws, rows)
        loss = self.backward_ws(ws, rows)
        self.adam_step(lr=lr, weight_decay=weight_decay)
        return loss

    def state_dict(self):
        return {"w": {k: v.cpu() for k, v in self.w.items()}, "b": {k: v.cpu() for k, v in self.b.items()},
                "omega": self.omega.cpu(), "beta": self.beta.cpu(), "n_vars": self.n_vars}

    def load_state_dict(self, sd):
        for k, v in sd["w"].items():
            self.w[k].copy_(v)
        for k, v in sd["b"].items():
            self.b[k].copy_(v)
        self.omega.copy_(sd["omega"])
        self.beta.copy_(sd["beta"])
        self._pack()


def constant_targets(ops: torch.Tensor, C: torch.Tensor, n_out: int = N_OUT):
    """(B, n_out) values of the first n_out LEARNABLE_CONSTANT slots of each row of C
    (row-major order) and the (B, n_out) mask of slots that exist."""
    is_c = ops == 1
    rank = torch.cumsum(is_c.to(torch.int32), dim=1) - 1
    sel = is_c & (rank < n_out)
    B = ops.shape[0]
    tgt = torch.zeros(B, n_out, dtype=torch.float32, device=ops.device)
    msk = torch.zeros(B, n_out, dtype=torch.float32, device=ops.device)
    rows = torch.arange(B, device=ops.device).unsqueeze(1).expand_as(ops)
    tgt[rows[sel], rank[sel].long()] = C[sel].float()
    msk[rows[sel], rank[sel].long()] = 1.0
    return tgt, msk


def _first_slots(ops: torch.Tensor, n_out: int = N_OUT):
    """Selector of the first n_out LEARNABLE_CONSTANT slots of each row and their ranks."""
    is_c = ops == 1
    rank = torch.cumsum(is_c.to(torch.int32), dim=1) - 1
    sel = is_c & (rank < n_out)
    rows = torch.arange(ops.shape[0], device=ops.device).unsqueeze(1).expand_as(ops)
    return sel, rows[sel], rank[sel].long()


def fit_objective(X, Y, ops, ch, C_base, pred, clip_grad: float = 10.0):
    """Normalised MSE of every problem at C_base with its first N_OUT learnable slots
    set to pred (B, N_OUT), and its gradient with respect to pred (rows whose loss or
    gradient is not finite get a zero gradient; row norms are clipped to clip_grad).
    Evaluated with the library's forward and adjoint kernels."""
    from .evaluation import evaluate
    sel, r, k = _first_slots(ops, pred.shape[1])
    C = C_base.clone()
    C[sel] = pred[r, k]
    C.requires_grad_(True)
    N = X.shape[0]
    cache = evaluate(X, ops, ch, C)
    root = ((ops != 0).sum(1) - 1).clamp(min=0)
    f = cache.gather(1, root.view(-1, 1, 1).expand(-1, 1, N)).squeeze(1)
    w = 1.0 / (Y.var(dim=1) + 1e-6)
    mse = ((f - Y) ** 2).mean(1) * w
    ok = torch.isfinite(mse)
    torch.where(ok, mse, torch.zeros_like(mse)).sum().backward()
    g = torch.zeros_like(pred)
    g[r, k] = C.grad[sel]
    good = ok & torch.isfinite(g).all(dim=1)
    g = torch.where(good.unsqueeze(1), g, torch.zeros_like(g))
    norm = g.norm(dim=1, keepdim=True)
    g = g * torch.clamp(clip_grad / (norm + 1e-12), max=1.0)
    return mse.detach(), g


def candidate_starts(X, Y, ops, C_plain, net: WarmStartMLP | None = None, extra: int = 0, clip: float = 10.0,
                     generator: torch.Generator | None = None) -> torch.Tensor:
    """(K, B, M) candidate starting constants: the plain start C_plain first, then the
    network's start (when net is given), then `extra` further standard-normal draws
    in the learnable slots (as create_constants draws them)."""
    cands = [C_plain]
    if net is not None:
        cands.append(warm_start_constants(net, X, Y, ops, C_plain, clip))
    is_c = ops == 1
    for _ in range(extra):
        draw = torch.randn(C_plain.shape, device=C_plain.device, generator=generator)
        cands.append(torch.where(is_c, draw, C_plain))
    return torch.stack(cands)


def screened_start(X, Y, ops, ch, C_sets: torch.Tensor) -> torch.Tensor:
    """Per problem, the candidate start (C_sets (K, B, M)) with the lowest initial loss,
    all candidates measured in one launch of the screening kernel; a non-finite loss
    counts as +inf and ties keep the earlier candidate (the plain start first)."""
    from .optimization import screen_starts
    loss = screen_starts(X, Y, ops, ch, C_sets)
    loss = torch.where(torch.isfinite(loss), loss, torch.full_like(loss, float("inf")))
    best = torch.argmin(loss, dim=1)
    return C_sets[best, torch.arange(ops.shape[0], device=ops.device)]


def gated_warm_start(net: WarmStartMLP, X, Y, ops, ch, C_plain, clip: float = 10.0) -> torch.Tensor:
    """The plain initialisation as fallback and arbiter: per problem, the start (warm
    or plain) with the lower initial MSE; a non-finite loss counts as +inf and ties
    keep the plain start."""
    return screened_start(X, Y, ops, ch, candidate_starts(X, Y, ops, C_plain, net, 0, clip))


def warm_start_constants(net: WarmStartMLP, X, Y, ops, C_plain, clip: float = 10.0) -> torch.Tensor:
    """C_init with the first N_OUT learnable slots of every row set to the network's
    prediction (clipped to [-clip, clip]); every other slot keeps C_plain."""
    pred = net.predict(ops, X, Y).clamp(-clip, clip)
    is_c = ops == 1
    rank = torch.cumsum(is_c.to(torch.int32), dim=1) - 1
    sel = is_c & (rank < N_OUT)
    C = C_plain.clone()
    rows = torch.arange(ops.shape[0], device=ops.device).unsqueeze(1).expand_as(ops)
    C[sel] = pred[rows[sel], rank[sel].long()]
    return C


@dataclass
class TrainingSet:
    X: list        # per workload: (N, n_vars) inputs
    Y: list        # (B, N) targets
    ops: list      # (B, M) tapes
    target: list   # (B, N_OUT) fitted constants
    mask: list     # (B, N_OUT) 1 where the slot exists and the fit succeeded


def fitted_examples(X, Y, ops, ch, C_init, max_iter: int = 200, clip: float = 10.0, good_fraction=None):
    """Run the fused fit from C_init and turn its results into training targets: the
    fitted constants of every problem whose fit ended without error, with a finite
    loss and every constant inside [-clip, clip] (optionally only fits whose final MSE
    is below good_fraction * var(Y)).  The network then learns where the fit ends."""
    from .optimization import optimize_ex
    r = optimize_ex(X, Y, ops, ch, C_init, max_iter=max_iter, raise_errors=False)
    tgt, msk = constant_targets(ops, r.C)
    ok = torch.isfinite(r.loss) & (r.iters >= 0)
    if good_fraction is not None:
        ok &= r.loss <= good_fraction * Y.var(dim=1)
    ok &= ((tgt.abs() <= clip) | (msk == 0)).all(dim=1) & torch.isfinite(tgt).all(dim=1)
    msk = msk * ok.unsqueeze(1).float()
    return torch.nan_to_num(tgt) * msk, msk, r


def train_fit_objective(net: WarmStartMLP, problems, epochs: int = 10, batch: int = 2048, lr: float = 1e-3,
                        weight_decay: float = 1e-4, seed: int = 0) -> TrainStats:
    """Train the network to minimise the fit objective of its own predictions:
    problems is a list of (X, Y, ops, ch, C_base) on the device; each step evaluates
    the batch's expressions at the predicted constants (forward + adjoint kernels)
    and back-propagates the gradient of the normalised MSE through the network."""
    g = torch.Generator().manual_seed(seed)
    losses = []
    steps = 0
    for _ in range(epochs):
        for pi in torch.randperm(len(problems), generator=g).tolist():
            X, Y, ops, ch, Cb = problems[pi]
            B = ops.shape[0]
            perm = torch.randperm(B, generator=g).to(ops.device)
            for s in range(0, B - batch + 1, batch):
                idx = perm[s:s + batch]
                o, y = ops[idx], Y[idx]
                ws = net.workspace(batch)
                net.features(o, X, y, ws)
                pred = net.forward_ws(ws, batch).clone()
                try:
                    mse, gp = fit_objective(X, y, o, ch[idx], Cb[idx], pred)
                except RuntimeError:
                    continue  # an exact zero denominator under a nonzero gradient (error 204)
                net.backward_ws(ws, batch, out_grad=gp)
                net.adam_step(lr=lr, weight_decay=weight_decay)
                steps += 1
                if steps % 16 == 0:
                    fin = torch.isfinite(mse)
                    losses.append(mse[fin].median() if fin.any() else torch.tensor(float("nan")))
    net.check_status()
    return TrainStats(steps=steps, loss=[float(x) for x in losses])


def train(net: WarmStartMLP, data: TrainingSet, epochs: int = 10, batch: int = 4096, lr: float = 1e-3,
          weight_decay: float = 1e-4, seed: int = 0) -> TrainStats:
    """Mini-batch Adam over every (workload, row) of the training set."""
    g = torch.Generator().manual_seed(seed)
    losses = []
    steps = 0
    for _ in range(epochs):
        for wi in torch.randperm(len(data.ops), generator=g).tolist():
            B = data.ops[wi].shape[0]
            perm = torch.randperm(B, generator=g).to(data.ops[wi].device)
            for s in range(0, B - batch + 1, batch):
                idx = perm[s:s + batch]
                loss = net.train_batch(data.ops[wi][idx], data.X[wi], data.Y[wi][idx], data.target[wi][idx],
                                       data.mask[wi][idx], lr=lr, weight_decay=weight_decay)
                steps += 1
                if steps % 16 == 0:
                    losses.append(loss.sum() / data.mask[wi][idx].sum().clamp(min=1))
    net.check_status()
    return TrainStats(steps=steps, loss=[float(x) for x in losses])
