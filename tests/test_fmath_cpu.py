"""Accuracy of the library's own float32 sin, cos, exp and log (csrc/sr_fmath.h).

The kernels evaluate these four operators with sr_fmath.h and the oracle's
kernel-arithmetic mode compiles the same file on the host, so a fit over tapes with
them is reproducible bit for bit (tests/test_fit_exact_gpu.py); this file checks the
functions themselves against the double-precision functions of the host's libm.

Over every float32 input (2^32 of them, checked once with the same checker at step
1) the largest errors are: sin 1.544 ulp, cos 1.540 ulp, exp 0.939 ulp, log 0.876
ulp, with every special value (NaN, +-inf, +-0, overflow to inf, underflow to 0)
where the correctly rounded result has it.  CUDA's own float functions are
documented at 2 ulp (sinf, cosf, expf) and 1 ulp (logf).  Here a strided sweep over
all inputs plus dense sweeps where the methods are weakest (near multiples of pi/2,
the reduction thresholds, the subnormal and overflow edges) run in a few seconds.
"""
import numpy as np
import pytest

import oracle

BOUND = {"sin": 1.55, "cos": 1.55, "exp": 0.94, "log": 0.88}


def f32_bits(x):
    return int(np.float32(x).view(np.uint32))


@pytest.mark.parametrize("name", ["sin", "cos", "exp", "log"])
def test_strided_sweep_over_all_inputs(name):
    for lo, hi in ((0x00000000, 0x7F7FFFFF), (0x80000000, 0xFF7FFFFF)):
        worst, at, bad, n = oracle.fmath_error(name, lo, hi, 4099)
        assert n > 500_000 and bad == 0
        assert worst <= BOUND[name], f"{name}: {worst:.3f} ulp at {at!r}"


@pytest.mark.parametrize("name", ["sin", "cos"])
def test_dense_sweeps_of_the_reduction(name):
    """Every float in [0, 8] (multiples of pi/2 up to 5), around 2^19 where the
    three-part reduction hands over to Payne-Hanek, and around 2^24 and 2^60."""
    ranges = [(0.0, 8.0), (524288.0 * 0.999, 524288.0 * 1.001), (2.0 ** 24 * 0.999, 2.0 ** 24 * 1.001),
              (2.0 ** 60, 2.0 ** 60 * 1.001)]
    for a, b in ranges:
        worst, at, bad, n = oracle.fmath_error(name, f32_bits(a), f32_bits(b), 3)
        assert bad == 0 and worst <= BOUND[name], f"{name} on [{a}, {b}]: {worst:.3f} ulp at {at!r}"


def test_dense_sweeps_of_exp_and_log():
    """exp near its overflow and subnormal edges and around 0; log of subnormals, of
    values around 1 and near sqrt(2) where the significand is halved."""
    for name, a, b in (("exp", 80.0, 89.0), ("exp", -104.0, -87.0), ("exp", -0.01, 0.01),
                       ("log", 1e-45, 1.2e-38), ("log", 0.99, 1.01), ("log", 1.41, 1.42)):
        lo, hi = sorted((f32_bits(a), f32_bits(b)))
        worst, at, bad, n = oracle.fmath_error(name, lo, hi, 1 if hi - lo < 3_000_000 else 7)
        assert bad == 0 and worst <= BOUND[name], f"{name} on [{a}, {b}]: {worst:.3f} ulp at {at!r}"


def test_special_values():
    inf, nan = np.float32(np.inf), np.float32(np.nan)
    x = np.array([0.0, -0.0, inf, -inf, nan], np.float32)
    s, c, e, lg = (oracle.fmath(n, x) for n in ("sin", "cos", "exp", "log"))
    assert s[0] == 0 and not np.signbit(s[0]) and s[1] == 0 and np.signbit(s[1])
    assert np.isnan(s[2:]).all() and np.isnan(c[2:]).all() and (c[:2] == 1).all()
    assert (e[:2] == 1).all() and e[2] == inf and e[3] == 0 and np.isnan(e[4])
    assert lg[0] == -inf and lg[1] == -inf and lg[2] == inf and np.isnan(lg[3]) and np.isnan(lg[4])
    assert np.isnan(oracle.fmath("log", np.array([-1.0, -1e-45], np.float32))).all()
    big = np.array([88.72283, 88.7228394, 89.0, 1e30], np.float32)
    assert np.isfinite(oracle.fmath("exp", big[:1])).all() and (oracle.fmath("exp", big[1:]) == inf).all()
    assert oracle.fmath("exp", np.array([-103.0], np.float32))[0] > 0
    assert oracle.fmath("exp", np.array([-104.5, -1e30], np.float32)).max() == 0


def test_exact_values():
    """Values the methods produce exactly: e^0 = 1, log 1 = 0, log 2^k = k ln 2 rounded."""
    assert oracle.fmath("exp", np.array([0.0], np.float32))[0] == 1.0
    assert oracle.fmath("log", np.array([1.0], np.float32))[0] == 0.0
    k = np.arange(-149, 128)
    x = np.ldexp(np.ones_like(k, dtype=np.float32), k).astype(np.float32)
    want = (k * np.log(2.0)).astype(np.float32)
    got = oracle.fmath("log", x)
    assert np.abs(got.astype(np.float64) - k * np.log(2.0)).max() <= np.spacing(np.abs(want)).max()
