"""Recipe: the reference's own CPU ``optimize`` against the oracle's port of it, on the
same problems, in the development container (where the reference checkout exists and
``build_ref.py`` has compiled its extension).

The timed CPU baseline on the GPU host is the port (``sr_oracle.c``, OpenMP over
problems), because the reference's sources do not exist there.  This recipe shows
what that choice means: it times the reference's ``symbolic_torch.optimize``
(``symbolic_torch/optimization.py:9-112``, ``symbolic_torch/lbfgs_batch.py:61-326``,
its C++ CPU evaluation through OpenMP) and the port on the same seeded problems, with
the same thread count, and compares their final MSEs and constants.

    python oracle/time_reference_cpu.py --workload readme --n 1024
    python oracle/time_reference_cpu.py --workload ragged --n 128
    python oracle/time_reference_cpu.py --workload eval --n 4096

The ``eval`` workload times ``symbolic_torch.evaluation.evaluate`` and the backward of the sum
of its root rows w.r.t. C (``symbolic_torch/evaluation.py:4-34``,
``src/symbolic_evaluation.cpp:39-168``) against the port's forward and adjoint, on
tapes of the evaluation benchmark (M=64, N=1024, 4 variables, mean length 20).

Prints one JSON line per run.  Test infrastructure only: nothing in the package
imports it.
"""
from __future__ import annotations

import argparse
import json
import os
import sys
import time

import numpy as np
import torch

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))

import build_ref  # noqa: E402
import oracle  # noqa: E402

from cudasymbolicregression_gb300 import workloads  # noqa: E402


def _roots(X, ops, ch, C):
    cache = oracle.eval_fwd(X, ops, ch, C)
    root = np.maximum((ops != 0).sum(1) - 1, 0)
    return cache[np.arange(ops.shape[0]), root]


def problems(workload: str, n: int, seed: int):
    """The first n problems of a benchmark workload: README problem (N=100, 100
    iterations) or the held-out ragged problems (N=512, 200 iterations)."""
    if workload == "readme":
        return workloads.readme_fit(B=n, N=100, seed=seed), 100
    wl = workloads.ragged_fit_chunks(B=4096, N=512, M=64, seed=seed, n_chunks=1, root_eval=_roots)
    return wl, 200


def compare_eval(ref, n: int, seed: int):
    """Forward + adjoint of the root rows: the reference's CPU evaluate and autograd
    backward against the port's, with the constant gradients compared."""
    from cudasymbolicregression_gb300 import tapes
    M, N = 64, 1024
    rng = np.random.default_rng(seed)
    X = rng.uniform(-3, 3, (N, 4)).astype(np.float32)
    C = rng.standard_normal((n, M)).astype(np.float32)
    # no exact-zero denominator at these points: the reference raises error 204 for one
    tb = tapes.generate(n, M, seed=seed + 1, mean_length=20.0, n_vars=4, p_const_leaf=0.2, X_screen=X, C_screen=C)
    root = np.maximum((tb.ops != 0).sum(1) - 1, 0)
    gout = np.zeros((n, M, N), np.float32)
    gout[np.arange(n), root] = 1.0

    t0 = time.perf_counter()
    oracle.eval_fwd(X, tb.ops, tb.ch, C)
    t1 = time.perf_counter()
    gC_port, _, err = oracle.eval_bwd(X, tb.ops, tb.ch, C, gout, want_gx=False)
    assert err == 0, err
    t2 = time.perf_counter()
    del gout

    Ct = torch.from_numpy(C).requires_grad_(True)
    t3 = time.perf_counter()
    y = ref.evaluation.evaluate(torch.from_numpy(X), torch.from_numpy(tb.ops), torch.from_numpy(tb.ch), Ct)
    t4 = time.perf_counter()
    y[torch.arange(n), torch.from_numpy(root)].sum().backward()
    t5 = time.perf_counter()
    gC_ref = Ct.grad.numpy()
    fin = np.isfinite(gC_ref) & np.isfinite(gC_port)
    close = np.abs(gC_port[fin] - gC_ref[fin]) <= 1e-5 * np.maximum(np.abs(gC_ref[fin]), 1.0)
    print(json.dumps({
        "workload": "eval", "tapes": n, "M": M, "N": N,
        "threads": {"port": oracle.num_threads(), "reference": torch.get_num_threads()},
        "reference_s": {"forward": t4 - t3, "backward": t5 - t4},
        "port_s": {"forward": t1 - t0, "backward": t2 - t1},
        "port_over_reference": (t5 - t3) / (t2 - t0),
        "grad_C_nan_placement_equal": bool(np.array_equal(np.isnan(gC_ref), np.isnan(gC_port))),
        "grad_C_within_1e-5": float(close.mean()),
    }), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", choices=("readme", "ragged", "eval"), default="readme")
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args()
    ref = build_ref.load_reference()
    oracle.build()
    if args.workload == "eval":
        compare_eval(ref, args.n, args.seed)
        return
    wl, max_iter = problems(args.workload, args.n, args.seed)
    idx = np.arange(min(args.n, wl.ops.shape[0]))
    X, Y, ops, ch, C = wl.X, wl.Y[idx], wl.ops[idx], wl.ch[idx], wl.C[idx]

    t0 = time.perf_counter()
    port = oracle.optimize(X, Y, ops, ch, C, max_iter=max_iter, dot_mode=0)
    t_port = time.perf_counter() - t0

    def T(a):
        return torch.from_numpy(np.ascontiguousarray(a))
    t0 = time.perf_counter()
    C_ref, Y_ref = ref.optimize(T(X), T(Y), T(ops), T(ch), T(C), max_iter=max_iter)
    t_ref = time.perf_counter() - t0

    mse_ref = ((Y_ref.numpy().astype(np.float64) - Y) ** 2).mean(1)
    mse_port = ((port["Y"].astype(np.float64) - Y) ** 2).mean(1)
    fin = np.isfinite(mse_ref) & np.isfinite(mse_port)
    rel = np.abs(mse_port - mse_ref) / np.maximum(np.abs(mse_ref), 1e-30)
    n = len(idx)
    print(json.dumps({
        "workload": args.workload, "problems": n, "max_iter": max_iter,
        "threads": {"port": oracle.num_threads(), "reference": torch.get_num_threads()},
        "reference_expr_per_s": n / t_ref, "port_expr_per_s": n / t_port,
        "port_over_reference": t_ref / t_port,
        "finite_both": int(fin.sum()),
        "final_mse_within_1e-4_rel": float((rel[fin] <= 1e-4).mean()),
        "constants_bit_identical": float(np.mean(np.all(port["C"] == C_ref.numpy(), axis=1))),
        "median_final_mse": {"reference": float(np.median(mse_ref[fin])), "port": float(np.median(mse_port[fin]))},
    }), flush=True)


if __name__ == "__main__":
    main()
