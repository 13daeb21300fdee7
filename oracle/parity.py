"""Parity criteria shared by the GPU tests and smoke() (test infrastructure).

Device and host libm differ by a few ulps in transcendental functions, and long
tapes amplify such differences through cancellation, so values computed along
a whole tape cannot be compared with a flat relative tolerance.  Two criteria
are used instead:

* local: every node value of the device cache is recomputed by the oracle from
  the device's own child values; IEEE-exact operations (+ - * /, sqrt, inv,
  neg, square, floor, ceil, leaves) and the library's own sin, cos, exp and log
  must agree bit for bit, CUDA's other transcendental functions within a few
  ulps, and NaN placement exactly.
* accuracy: against the FP64 oracle, the device's float32 result must be within
  1e-5 relative, or no less accurate than the reference float32 result (the
  reference's own CPU output, or the float32 oracle) up to a factor of 4.
"""
import numpy as np

import oracle

EXACT = {0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 14, 15, 23, 24, 27, 28, 40, 41, 42, 43}
# sin, cos, exp, log, ln: the kernels' own functions (sr_fmath.h), reproduced bit for bit
KERNEL_MATH = {10, 11, 12, 13, 25}
ULP_TRANSC = 8
ULP_POW = 16


def ulp_dist(a, b):
    a = np.asarray(a, np.float32)
    b = np.asarray(b, np.float32)
    ia = a.view(np.int32).astype(np.int64)
    ib = b.view(np.int32).astype(np.int64)
    ia = np.where(ia < 0, -(ia & 0x7FFFFFFF), ia)
    ib = np.where(ib < 0, -(ib & 0x7FFFFFFF), ib)
    return np.abs(ia - ib)


def check_local(X, ops, ch, C, cache):
    """Node-by-node check of a device cache (B, M, N) against the oracle."""
    X = np.asarray(X, np.float32)
    B, M, N = cache.shape
    bb, kk = np.nonzero(np.ones((B, M), bool))
    op = ops[bb, kk].copy()
    op[(op >= 50 + X.shape[1]) | ((op > 44) & (op < 50)) | (op < 0)] = 9  # codes the reference evaluates to 0
    c0 = np.maximum(ch[bb, kk, 0], 0)
    c1 = np.maximum(ch[bb, kk, 1], 0)
    a = cache[bb, c0]                       # (B*M, N)
    b = cache[bb, c1]
    cv = np.repeat(C[bb, kk][:, None], N, 1)
    var = np.clip(op - 50, 0, X.shape[1] - 1)
    xv = X[:, var].T                        # (B*M, N)
    opn = np.repeat(op[:, None], N, 1)
    ref = oracle.node_fwd(opn.ravel(), a.ravel(), b.ravel(), cv.ravel(), xv.ravel()).reshape(a.shape)
    km = np.isin(opn, list(KERNEL_MATH))
    if km.any():  # the same function on both sides: the same bits
        ref[km] = oracle.node_fwd(opn[km], a[km], b[km], cv[km], xv[km], kernel_math=True)
    got = cache[bb, kk]
    nan_r, nan_g = np.isnan(ref), np.isnan(got)
    assert np.array_equal(nan_r, nan_g), f"local NaN placement differs for ops {np.unique(opn[nan_r != nan_g])}"
    both = ~nan_r
    d = ulp_dist(got[both], ref[both])
    tol = np.where(np.isin(opn[both], list(EXACT | KERNEL_MATH)), 0, np.where(opn[both] == 44, ULP_POW, ULP_TRANSC))
    with np.errstate(invalid="ignore"):
        tiny = (np.abs(got[both].astype(np.float64) - ref[both]) <= 1e-37) | (got[both] == ref[both])
    bad = (d > tol) & ~tiny
    if bad.any():
        i = np.argmax(d - tol)
        raise AssertionError(f"local mismatch: op {opn[both][i]} got {got[both][i]!r} ref {ref[both][i]!r} "
                             f"({d[i]} ulp), {bad.sum()} entries")
    return {"nodes": int(got.size), "max_ulp": int(d.max(initial=0))}


def check_accuracy(got, ref32, ref64, rtol=1e-5, atol=1e-6, min_frac_tight=0.999, gross=1e3, max_outliers=None,
                   abs_scale=None):
    """Device float32 result vs the reference float32 result and the FP64 oracle.

    * at least ``min_frac_tight`` of the entries within rtol of the reference result;
    * the device's error against FP64 is not worse than the reference's, in
      distribution: median and 99.9th percentile of the relative error within 2x;
    * no entry is grossly worse: |got - ref64| <= gross * |ref32 - ref64| + rtol|ref64| + atol,
      except where float32 itself is ill-conditioned (ref32 and FP64 disagree by
      more than 1e-3 relative, or in NaN/inf placement), and except at most
      ``max_outliers`` entries (default max(2, 1e-5 of the entries)): an ulp-level
      difference upstream of a discontinuous operation (floor, ceil, a comparison
      in a domain check, tan near a pole) can move one value far although every
      node is exact given its inputs, which check_local verifies separately.

    abs_scale (the sum of the absolute values of the terms an entry adds up) makes the
    percentile test measure errors relative to max(|ref64|, abs_scale): for sums whose
    order is not fixed (atomic accumulation, in the reference too) the rounding error
    scales with the terms, not with a cancelled total.
    """
    got = np.asarray(got, np.float64)
    ref32 = np.asarray(ref32, np.float64)
    ref64 = np.asarray(ref64, np.float64)
    with np.errstate(invalid="ignore", over="ignore", divide="ignore"):
        tight = (np.abs(got - ref32) <= rtol * np.abs(ref32) + atol) | (np.isnan(got) & np.isnan(ref32)) | (got == ref32)
        err_g = np.abs(got - ref64)
        err_r = np.abs(ref32 - ref64)
        boundary = (np.isnan(ref64) != np.isnan(ref32)) | (np.isinf(ref64) != np.isinf(ref32)) | ~np.isfinite(err_r) \
            | (err_r > 1e-3 * np.abs(ref64))
        not_gross = err_g <= gross * err_r + rtol * np.abs(ref64) + atol
    ok = tight | not_gross | boundary
    allowed = max(2, int(1e-5 * ok.size)) if max_outliers is None else max_outliers
    assert (~ok).sum() <= allowed, (f"{(~ok).sum()} entries grossly less accurate than the reference float32 result; first at "
                      f"{np.argwhere(~ok)[:3].tolist()}: got {got[~ok][:3]}, ref32 {ref32[~ok][:3]}, ref64 {ref64[~ok][:3]}")
    frac = float(tight.mean()) if tight.size else 1.0
    assert frac >= min_frac_tight, f"only {frac:.5f} of the entries within {rtol} of the reference float32 result"
    fin = np.isfinite(got) & np.isfinite(ref32) & np.isfinite(ref64) & ~boundary & ok
    stats = {"frac_tight": frac}
    if fin.any():
        scale = np.maximum(np.abs(ref64[fin]), 1e-30)
        if abs_scale is not None:
            scale = np.maximum(scale, np.asarray(abs_scale, np.float64)[fin])
        rg = err_g[fin] / scale
        rr = err_r[fin] / scale
        for q in (50.0, 99.9):
            pg, pr = np.percentile(rg, q), np.percentile(rr, q)
            assert pg <= 2.0 * pr + 1e-7, f"{q}th percentile relative error vs FP64 {pg:.3g} > 2 x reference {pr:.3g}"
            stats[f"p{q}_rel_err_device"] = float(pg)
            stats[f"p{q}_rel_err_reference"] = float(pr)
    return stats


def first_divergence(run_a, run_b, idx, max_iter, rtol=1e-4):
    """For the problems idx, the first iteration count k (0..max_iter) at which the
    constants of run_a(k, idx) and run_b(k, idx) part by more than rtol relative or
    in NaN placement; max_iter + 1 where they never do.  Problems are independent of
    the rest of their batch, so each run fits only the problems asked about."""
    idx = np.asarray(idx)
    first = np.full(idx.size, max_iter + 1)
    for k in range(max_iter + 1):
        a = np.asarray(run_a(k, idx), np.float64)
        b = np.asarray(run_b(k, idx), np.float64)
        with np.errstate(invalid="ignore", divide="ignore"):
            rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-30)
        d = ((np.isnan(a) != np.isnan(b)) | (np.nan_to_num(rel, nan=0.0) > rtol)).any(1)
        first = np.where((first > max_iter) & d, k, first)
    return first


def oracle_fit_like(r, X, Y, ops, ch, C, **kw):
    """The oracle's kernel-arithmetic fit (dot_mode 2) of the problems of a device fit
    r (a FitResult), each with the launch shape its kernel launch used (r.shapes);
    kw are the fit's options (max_iter, line_search_fn, ...).  Returns the oracle's
    outputs in batch order, as oracle.optimize does."""
    ops = np.asarray(ops)
    B, M = ops.shape
    N = np.asarray(X).shape[0]
    spl = oracle.kernel_slot_registers(ops)
    out = dict(C=np.empty((B, M), np.float32), Y=np.empty((B, N), np.float32), iters=np.empty(B, np.int32),
               evals=np.empty(B, np.int64), loss=np.empty(B, np.float32), err=0)
    Yb = None if Y is None else np.broadcast_to(np.asarray(Y, np.float32), (B, N))
    for idx, V, W in r.shapes:
        idx = idx.cpu().numpy().astype(np.int64) if hasattr(idx, "cpu") else np.asarray(idx, np.int64)
        o = oracle.optimize(X, None if Yb is None else Yb[idx], ops[idx], np.asarray(ch)[idx], np.asarray(C)[idx],
                            dot_mode=2, warps=W, points_per_lane=V, slot_registers=spl, **kw)
        for k in ("C", "Y", "iters", "evals", "loss"):
            out[k][idx] = o[k]
        out["err"] = out["err"] or o["err"]
    return out


def fit_bits_differ(r, o):
    """Per problem: does the device fit r differ from the oracle's o in any bit of its
    constants, root values or loss, or in its iteration or closure count (NaN
    compares as NaN)."""
    def bits(a, b):
        a = np.ascontiguousarray(a, np.float32)
        b = np.ascontiguousarray(b, np.float32)
        na, nb = np.isnan(a), np.isnan(b)
        d = (na != nb) | (~na & ~nb & (a.view(np.uint32) != b.view(np.uint32)))
        return d.reshape(d.shape[0], -1).any(1)
    bad = (r.iters.cpu().numpy() != o["iters"]) | (r.evals.cpu().numpy() != o["evals"])
    bad |= bits(r.C.cpu().numpy(), o["C"]) | bits(r.loss.cpu().numpy(), o["loss"])
    if r.Y is not None:
        bad |= bits(r.Y.cpu().numpy(), o["Y"])
    return bad
