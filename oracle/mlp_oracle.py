"""CPU oracle of the warm-start network's kernels (test infrastructure only).

The warm-start network has no counterpart in the reference; this module states its
arithmetic plainly in numpy (float64 accumulation of bf16 operands) so that the
tests can check every device kernel:

* ``bf16``: round-to-nearest-even of float32 to bfloat16 (returned as float32);
* ``random_features`` / ``features``: the network's input features;
* ``gemm`` + ``epilogue``: D = A . W^T and the five epilogues of ``sr_mlp_gemm``;
* ``loss``: squared error and its output gradient;
* ``forward`` / ``backward``: the whole network with bf16 rounding at the points
  where the device rounds (after every epilogue), for end-to-end comparisons;
* ``adam``: one optimiser step.
"""
from __future__ import annotations

import numpy as np

VOCAB, EMB, FEATS, PROJ, IN, HIDDEN, OUT_PAD, N_OUT = 64, 64, 32, 28, 128, 256, 64, 8


def bf16(x) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even); NaN stays NaN."""
    a = np.ascontiguousarray(np.asarray(x, dtype=np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).copy()
    nan = np.isnan(a)
    out[nan] = np.nan
    return out.reshape(a.shape)


def from_bf16_bits(u16) -> np.ndarray:
    return (np.asarray(u16, dtype=np.uint16).astype(np.uint32) << 16).view(np.float32)


def random_features(X, omega, beta) -> np.ndarray:
    """phi (N, PROJ) = sqrt(2) cos(omega_j . x_n + beta_j)."""
    a = np.asarray(X, np.float64) @ np.asarray(omega, np.float64).T + np.asarray(beta, np.float64)
    return (np.sqrt(2.0) * np.cos(a)).astype(np.float32)


def features(ops, Y, phi):
    """hist (B, VOCAB) float32 token frequencies (as the device computes them, before
    bf16 rounding) and feats (B, FEATS) float64."""
    ops = np.asarray(ops)
    B = ops.shape[0]
    hist = np.zeros((B, VOCAB), np.float32)
    for b in range(B):
        t = ops[b][ops[b] != 0]
        L = t.size
        if L == 0:
            continue
        t = np.where((t >= 0) & (t < VOCAB), t, VOCAB - 1)
        cnt = np.bincount(t, minlength=VOCAB).astype(np.float32)
        hist[b] = cnt * (np.float32(1.0) / np.float32(L))
    Y = np.asarray(Y, np.float64)
    mu = Y.mean(1)
    d = Y - mu[:, None]
    m2, m3, m4 = (d ** 2).mean(1), (d ** 3).mean(1), (d ** 4).mean(1)
    sd = np.sqrt(m2)
    flat = ~(sd > 1e-12)
    inv = np.where(flat, 0.0, 1.0 / np.where(flat, 1.0, sd))
    z = d * inv[:, None]
    feats = np.zeros((B, FEATS))
    feats[:, 0] = np.arcsinh(mu)
    feats[:, 1] = np.log(sd + 1e-3)
    feats[:, 2] = np.where(flat, 0.0, np.clip(m3 * inv ** 3, -50, 50))
    feats[:, 3] = np.where(flat, 0.0, np.arcsinh(m4 * inv ** 4 - 3.0))
    feats[:, 4:] = z @ np.asarray(phi, np.float64) / Y.shape[1]
    feats[~np.isfinite(feats)] = 0.0
    return hist, feats


def gemm(A, W) -> np.ndarray:
    return np.asarray(A, np.float64) @ np.asarray(W, np.float64).T


def epilogue(acc, mode, bias=None, gate=None) -> np.ndarray:
    """Values before the final rounding: 0 relu, 1 linear, 2 f32, 3 relu-gate, 4 split sum."""
    z = acc + (np.asarray(bias, np.float64) if bias is not None and mode in (0, 1, 2) else 0.0)
    if mode == 0:
        return np.maximum(z, 0.0)
    if mode == 3:
        return np.where(np.asarray(gate) > 0, acc, 0.0)
    return z


def loss(out, target, mask, scale):
    """Per-row sum of mask (out - t)^2 and the gradient scale * 2 * mask * (out - t)."""
    d = np.asarray(out, np.float64)[:, :N_OUT] - target
    row = (mask * d * d).sum(1)
    g = np.zeros((out.shape[0], OUT_PAD))
    g[:, :N_OUT] = scale * 2.0 * mask * d
    return row, g


def forward(w, b, hist, feats):
    """Whole-network forward from bf16 weights w[name] (float32 arrays holding bf16
    values) and fp32 biases; activations rounded to bf16 after each epilogue."""
    hist = bf16(hist)
    emb = bf16(gemm(hist, w["E"]).astype(np.float32))
    x0 = np.zeros((hist.shape[0], IN), np.float32)
    x0[:, :EMB] = emb
    x0[:, EMB:EMB + FEATS] = bf16(np.asarray(feats, np.float32))
    acts = {"x0": x0}
    h = x0
    for i, n in ((1, "W1"), (2, "W2"), (3, "W3")):
        h = bf16(epilogue(gemm(h, w[n]), 0, b[n]).astype(np.float32))
        acts[f"h{i}"] = h
    out = epilogue(gemm(h, w["W4"]), 2, b["W4"])
    return out, acts


def backward(w, b, hist, acts, d_out):
    """Gradients of the weights and biases for an output gradient d_out (rows, OUT_PAD),
    with bf16 rounding of every propagated gradient as on the device."""
    g, gb = {}, {}
    dz = bf16(np.asarray(d_out, np.float32))
    ups = {3: "W4", 2: "W3", 1: "W2"}
    below = {3: "h2", 2: "h1", 1: "x0"}
    g["W4"] = gemm(dz.T, acts["h3"].T)
    gb["W4"] = dz.astype(np.float64).sum(0)
    for i in (3, 2, 1):
        dh = gemm(dz, w[ups[i]].T)
        dz = bf16(epilogue(dh, 3, gate=acts[f"h{i}"]).astype(np.float32))
        name = f"W{i}"
        g[name] = gemm(dz.T, acts[below[i]].T)
        gb[name] = dz.astype(np.float64).sum(0)
    dx0 = bf16(gemm(dz, w["W1"].T).astype(np.float32))
    g["E"] = gemm(dx0[:, :EMB].T, bf16(hist).T)
    return g, gb


def adam(w, g, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8, weight_decay=0.0):
    """One Adam step with decoupled weight decay; returns (w, m, v) in float64."""
    m = beta1 * m + (1 - beta1) * g
    v = beta2 * v + (1 - beta2) * g * g
    bc1, bc2 = 1 - beta1 ** step, 1 - beta2 ** step
    w = w - lr * ((m / bc1) / (np.sqrt(v / bc2) + eps) + weight_decay * w)
    return w, m, v
