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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--workload", choices=("readme", "ragged"), default="readme")
    ap.add_argument("--n", type=int, default=1024)
    ap.add_argument("--seed", type=int, default=0)
    args = ap.parse_args()
    ref = build_ref.load_reference()
    oracle.build()
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
