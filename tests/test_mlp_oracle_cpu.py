"""CPU checks of the warm-start network's oracle (oracle/mlp_oracle.py)."""
import numpy as np
import torch

import mlp_oracle as mo


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(0)
    x = np.concatenate([rng.standard_normal(10000).astype(np.float32) * 10.0 ** rng.integers(-30, 30, 10000),
                        np.array([0.0, -0.0, 1.0, 65504.0, 1e-40, np.inf, -np.inf], np.float32)]).astype(np.float32)
    ref = torch.tensor(x).to(torch.bfloat16).float().numpy()
    np.testing.assert_array_equal(mo.bf16(x), ref)
    assert np.isnan(mo.bf16(np.array([np.nan], np.float32))).all()


def test_bf16_bits_roundtrip():
    u = np.arange(0, 65536, 7, dtype=np.uint16)
    f = mo.from_bf16_bits(u)
    finite = np.isfinite(f)
    np.testing.assert_array_equal(mo.bf16(f[finite]), f[finite])


def test_features_basic_properties():
    rng = np.random.default_rng(1)
    ops = np.array([[50, 1, 40, 10, 0, 0], [0, 0, 0, 0, 0, 0]], np.int64)
    Y = rng.standard_normal((2, 64)).astype(np.float32)
    Y[1] = 3.0
    phi = mo.random_features(rng.uniform(-3, 3, (64, 1)).astype(np.float32), rng.standard_normal((28, 1)),
                             rng.uniform(0, 6.28, 28))
    hist, f = mo.features(ops, Y, phi)
    np.testing.assert_allclose(hist[0].sum(), 1.0, rtol=1e-6)
    assert hist[0, 50] == np.float32(0.25) and hist[0, 40] == np.float32(0.25)
    assert (hist[1] == 0).all()
    assert f[1, 2] == 0 and f[1, 3] == 0 and (f[1, 4:] == 0).all()
    np.testing.assert_allclose(f[1, 0], np.arcsinh(3.0))


def test_adam_oracle_matches_torch_adamw():
    rng = np.random.default_rng(2)
    w0 = rng.standard_normal(50)
    p = torch.nn.Parameter(torch.tensor(w0, dtype=torch.float64))
    opt = torch.optim.AdamW([p], lr=1e-2, betas=(0.9, 0.999), eps=1e-8, weight_decay=1e-2)
    w, m, v = w0.copy(), np.zeros(50), np.zeros(50)
    for step in range(1, 6):
        g = rng.standard_normal(50)
        p.grad = torch.tensor(g)
        opt.step()
        w, m, v = mo.adam(w, g, m, v, step, 1e-2, weight_decay=1e-2)
    np.testing.assert_allclose(w, p.detach().numpy(), rtol=1e-12, atol=1e-12)


def test_gemm_epilogues():
    acc = np.array([[-1.0, 2.0], [0.5, -0.25]])
    np.testing.assert_array_equal(mo.epilogue(acc, 0, np.array([0.5, 0.0])), [[0.0, 2.0], [1.0, 0.0]])
    np.testing.assert_array_equal(mo.epilogue(acc, 3, gate=np.array([[1.0, 0.0], [0.0, 2.0]])),
                                  [[-1.0, 0.0], [0.0, -0.25]])
