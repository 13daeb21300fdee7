"""Derives the polynomial sr_fmath.h uses for log (run: python sr_fmath_coefficients.py).

log(1 + f) = f - f^2/2 + f^3 h(f) for f in [sqrt(1/2) - 1, sqrt(2) - 1].  h is fitted
as a degree-8 polynomial to (log(1 + f) - f + f^2/2) / f^3, evaluated with mpmath at
40 digits: weighted least squares on 4000 Chebyshev nodes, the weight being the
size of f^3 h relative to log(1 + f) (so the fit minimises the error of the final
result), then iteratively reweighted towards the largest errors (a Remez-like
equalisation of the error).  The coefficients are rounded to float32 and printed as
the Horner chain of sr_fmath.h, highest degree first, with the fit's own error in
units of the last place of the result.
"""
import mpmath as mp
import numpy as np

DEG = 8


def fit(deg=DEG, nodes=4000, rounds=30):
    mp.mp.dps = 40
    a, b = float(mp.sqrt(0.5) - 1), float(mp.sqrt(2) - 1)
    xs = np.cos(np.pi * (np.arange(nodes) + 0.5) / nodes) * (b - a) / 2 + (b + a) / 2

    def rem(f):
        f = mp.mpf(f)
        if abs(f) < 1e-6:
            return mp.mpf(1) / 3 - f / 4 + f ** 2 / 5 - f ** 3 / 6
        return (mp.log1p(f) - f + f * f / 2) / f ** 3

    ys = np.array([float(rem(x)) for x in xs])
    w = np.abs(xs) ** 3 / np.abs([float(mp.log1p(x)) for x in xs])
    A = np.vander(xs, deg + 1, increasing=True)
    coef = np.linalg.lstsq(A * w[:, None], ys * w, rcond=None)[0]
    for _ in range(rounds):
        err = (A @ coef - ys) * w
        wt = 1 + 50 * (np.abs(err) / np.abs(err).max()) ** 2
        coef = np.linalg.lstsq(A * (w * wt)[:, None], ys * w * wt, rcond=None)[0]
    c32 = coef.astype(np.float32)
    ulps = float(np.abs((A @ c32.astype(np.float64) - ys) * w).max() / 2.0 ** -24)
    return c32, ulps


if __name__ == "__main__":
    c, ulps = fit()
    print(f"/* fit error {ulps:.3f} ulp */")
    print(f"float h = SRM_FMA(f, {repr(float(c[-1]))}f, {repr(float(c[-2]))}f);")
    for k in range(len(c) - 3, -1, -1):
        print(f"h = SRM_FMA(f, h, {repr(float(c[k]))}f);")
