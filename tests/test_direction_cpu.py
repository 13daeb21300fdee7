"""Accuracy of the fused fit's search direction, in the kernel's arithmetic (the oracle's
restatement, which the GPU equals bit for bit in tests/test_fit_exact_gpu.py).

Histories of (s, y) pairs come from random quadratics whose Hessian eigenvalues span
10^0 .. 10^c (y = A s with a small relative perturbation, steps of scales 10^0 .. 10^-3),
in float32.  The reference direction is the two-loop recursion in float64 on the same
float32 pairs, with rho = 1 / (s.y + eps) and gamma = s.y / (y.y + eps) of the newest
pair (lbfgs_batch.py:65-103).  The kernel's direction (the compact representation, with
two lanes per pair for histories of at most 16 pairs, or the two-loop recursion above 32)
must stay within float32 rounding of it: the relative error of the whole vector has a
median below 2^-22 and a 99th percentile below 2^-19 at every condition number up to
10^7 (measured: medians 6e-8 to 1e-7, 99th percentiles 1.2e-7 to 5.8e-7; the compact
form's 99th percentiles stay at 1.2e-7 to 2.3e-7, the two-loop recursion's reach 4.9e-7
to 5.8e-7 at condition numbers of 10^5 and above).
"""
import numpy as np
import pytest

import oracle

EPS = 1e-10


def two_loop64(S, Y, g, hist):
    n = len(S)
    h = min(n, hist)
    S, Y = S[n - h:].astype(np.float64), Y[n - h:].astype(np.float64)
    q = g.astype(np.float64).copy()
    al = np.zeros(h)
    rho = 1.0 / (np.einsum("ij,ij->i", S, Y) + EPS)
    for i in range(h - 1, -1, -1):
        al[i] = rho[i] * (S[i] @ q)
        q -= al[i] * Y[i]
    q *= (S[-1] @ Y[-1]) / (Y[-1] @ Y[-1] + EPS)
    for i in range(h):
        be = rho[i] * (Y[i] @ q)
        q += (al[i] - be) * S[i]
    return -q


def histories(seed, cond_exp, count, n=8, D=32):
    rng = np.random.default_rng(seed)
    for _ in range(count):
        Q, _r = np.linalg.qr(rng.standard_normal((n, n)))
        A = Q.T @ np.diag(10.0 ** (cond_exp * rng.random(n))) @ Q
        npairs = int(rng.integers(3, 24))
        S = np.zeros((npairs, D), np.float32)
        Y = np.zeros((npairs, D), np.float32)
        for k in range(npairs):
            s = rng.standard_normal(n) * 10.0 ** (-3 * rng.random())
            S[k, :n] = s
            Y[k, :n] = (A @ s) * (1 + 1e-3 * rng.standard_normal(n))
        g = np.zeros(D, np.float32)
        g[:n] = rng.standard_normal(n)
        yield S, Y, g


@pytest.mark.parametrize("cond_exp", [1, 3, 5, 7])
@pytest.mark.parametrize("hist,two_loop", [(10, False), (20, False), (40, False), (10, True)])
def test_direction_within_float32_rounding(cond_exp, hist, two_loop):
    errs = []
    for S, Y, g in histories(100 + cond_exp, cond_exp, 400):
        want = two_loop64(S, Y, g, hist)
        got = oracle.direction(S, Y, g, hist, 8, two_loop=two_loop).astype(np.float64)
        errs.append(np.linalg.norm(got - want) / np.linalg.norm(want))
    errs = np.array(errs)
    assert np.median(errs) < 2.0 ** -22, np.median(errs)
    assert np.percentile(errs, 99) < 2.0 ** -19, np.percentile(errs, 99)


def test_direction_of_a_scaled_identity():
    """y = 2 s for every pair: H = I / 2, so p = -g / 2 in every mode, to a few float32
    units in the last place (the vector is formed in float from terms that cancel here,
    and eps moves gamma off 1/2 by a relative 1e-10 / y.y)."""
    rng = np.random.default_rng(5)
    S = np.zeros((12, 32), np.float32)
    S[:, :8] = rng.standard_normal((12, 8))
    Y = 2 * S
    g = np.zeros(32, np.float32)
    g[:8] = rng.standard_normal(8)
    for hist, tl in ((10, False), (20, False), (40, False), (10, True)):
        np.testing.assert_allclose(oracle.direction(S, Y, g, hist, 8, two_loop=tl)[:8], -g[:8] / 2, rtol=1e-6)
