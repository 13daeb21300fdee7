"""Benchmark: expressions fitted per second, warm-started vs plain fused fit.

Default workload (one "step" = one fit of the whole batch): the learned warm start
evaluated on held-out problems -- B=65536 ragged problems (tapes of uniform length
3..64 over {+,-,*,/,sin,cos,exp,log}, 0..8 learnable constants, n_variables=2,
N=512 points, X ~ U[-3, 3], each target a hidden random expression + N(0, 0.01^2)
noise), fitted with history 10, max_iter=200, strong Wolfe, tolerance_grad=1e-7.
Before timing, the warm-start network is trained (untimed) on the fits of
`--train-sets` x 65536 other problems (16: 1,048,576 fits): first on the constants
the plain fit found, then on the fit objective itself.  Arms timed on the same batch:
  plain : optimize() from the randn constants;
  warm  : per problem the lower initial loss of the plain start and the network's
          start (features + 5 tensor-core GEMMs), both measured in one launch of the
          screening kernel, then optimize();
  ablation: randn_gate (the network replaced by one randn draw), net_multistart and
          randn_multistart (two more randn draws added to both: four candidates);
  start_at_own_answer: every problem started at the constants its own plain fit
          ended with, the most any warm start can gain under the same stopping rule
          (max_iter, tolerance_grad); on this workload about 1.1x, because about half
          of the finite fits run to max_iter with the float32 gradient above the
          tolerance even from their own optimum.
Seeded synthetic data; no dataset is involved.

`value`   = B / (device time of one warm step), inputs resident in HBM, L2 flushed
            (256 MiB write) before each step; `plain` holds the plain arm.
`quality` = per arm: median final MSE over the problems the plain arm leaves finite
            (a non-finite result counts as +inf), the share of problems that end
            finite and finite fits per second, the share of closures spent on them,
            iterations on the finite problems (median, mean, share that reach
            tolerance_grad, median iterations of those), iterations and closures over
            all problems.
`e2e`     = the warm arm through the public API from pinned host buffers (H2D of X,
            Y, Ops, Ch, C_init and D2H of C_final, Y_final inside the timed region).
`roofline`= the fit kernel's algorithmic FP32 rate (op table in
            cudasymbolicregression_gb300/workloads.py) over its CUDA-event time.
`cpu_baseline` = the CPU oracle port of the reference's optimize() (plain start; the
            reference has no warm start) on the first 512 problems, all host threads.

Other workloads: --workload ragged (the plain fit of B=16384 such problems),
--workload readme (the README problem: expressions from its small grammar fitted to
2.5 cos(X_0) - 1.5, warm vs plain), --workload eval (evaluate forward + adjoint of a
dense root-row gradient at B=65536, M=64, N=1024; value = algorithmic HBM bytes /
step time).
--workload search (the full search round): every round samples B=262144 new
expressions (tapes over {+,-,*,/,sin,cos,exp,log}, 3 variables, padded length 64) and
fits them (max_iter=100) to N=2048 points of one hidden seeded 5-operator target, for
--rounds rounds (candidates from the grammar object on the device, --candidates pcfg,
or the host generator, --candidates tapes); the plain arm starts from randn, the warm arm from the gated
network, which is trained online on every finished round's fits.  Reported per arm:
wall-clock to the first MSE < 1e-6 and expressions fitted/s over all rounds.
--workload sample (the grammar object feeding a search): B=1048576 expressions drawn
from a 17-rule grammar (infix padded to --N=64 tokens), parsed to postfix and linked
(child table) on the device, one host synchronisation per step; value = expressions/s.
--workload gemm: the warm-start network's tensor-core GEMM (sr_mlp_gemm) at a size where
its efficiency shows: D (--B=262144 rows x 256) = A (262144 x --N=4096) . W (256 x 4096)^T
in bf16 with fp32 accumulation and a bf16 epilogue, 512 of them back to back per step;
value = TFLOP/s (2 rows n k per GEMM), roofline against the measured bf16 peak (a
256-wide product reads each A element for 512 flops, so the shape sits at the ridge of
the bf16 and HBM roofs).
--impl reference runs only the CPU port (the reference's own CPU path, restated).
Multi-GPU: one process per GPU; every rank fits its own batch (independent seeds, no
collective), value = all problems / max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np  # noqa: E402
import torch  # noqa: E402

METRIC = "expressions fitted/s at fixed final MSE, warm-start vs plain fused, 1 GB300"
UNIT = "expressions/s"
M_DEFAULT = 64
MAX_ITER = 200
EVAL_METRIC = "evaluation forward+adjoint throughput (algorithmic HBM bytes)"
DEFAULTS = {"warmstart": (65536, 512), "ragged": (16384, 512), "readme": (65536, 100), "eval": (65536, 1024),
            "search": (262144, 2048), "sample": (1048576, 64), "gemm": (262144, 4096)}
SAMPLE_METRIC = "expressions sampled from a grammar, parsed to postfix and linked (child table) per second"
GEMM_METRIC = "warm-start network GEMM throughput on the tensor cores (tcgen05, bf16 operands, fp32 accumulation)"
GEMM_N = 256  # the network's widest layer
GEMM_REPS = 512  # GEMMs per step of the gemm workload (a step long enough to sample its clocks)

# DRAM bytes (read + write) of one launch of the dominant kernel on the default
# workloads, from ncu captures of a 4x / 16x smaller batch scaled by the number of
# problems (profiles/fit_lbfgs_ragged_B16384_N512.txt,
# profiles/eval_forward_B4096_N1024.txt, profiles/eval_backward_B4096_N1024.txt).
# The fit kernel's traffic per problem is set by N, M and the history, not by the
# operator set, so the warm-start line's held-out problems (same lengths, M and N)
# scale the same B=4096 ragged capture.
FIT_TRAFFIC_BYTES = {("ragged", 16384, 512): 4 * (10738176 + 2048),
                     ("warmstart", 65536, 512): 16 * (10738176 + 2048)}
# Pipe and issue utilisation of the fit kernel (percent of peak, active cycles) from the
# same capture, the kernel of commit a0a780f (profiles/fit_lbfgs_ragged_B16384_N512.txt):
# an interpreter whose instructions are mostly integer and control work.
FIT_PROFILE = {"commit": "a0a780f", "issue_active_pct": 53.9, "fp32_pipe_pct": 14.9, "xu_pipe_pct": 1.73,
               "alu_pipe_pct": 48.7, "lsu_pipe_pct": 25.1, "fp64_pipe_pct": 1.68, "warps_active_pct": 23.1,
               "capture": "ncu --set full, ragged B=4096, N=512"}
# The adjoint call: its length-class grids (which stage the cached value rows of the real
# nodes beside the grad_out rows) and the concurrent padding check, captured with three
# classes; the split of the longest class at 48 nodes moves the same rows.
EVAL_TRAFFIC_BYTES = {("eval_forward_kernel", 65536, 1024): 16 * (1611520 + 1012199000),
                      ("eval_backward_kernel", 65536, 1024): 16 * (1364424192 + 13661696)}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "sm_max_mhz": 2070.0}, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle samples while the timed region runs."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def load_oracle():
    """The oracle (the CPU baseline only), built, with every host thread
    this process may use (a launcher such as torch.distributed.run sets
    OMP_NUM_THREADS=1 for its ranks)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    oracle.set_num_threads(len(os.sched_getaffinity(0)))
    return oracle


def cpu_sample_run(wl, n_sample: int, max_iter: int = MAX_ITER):
    """The CPU oracle port of optimize() (plain start) on the first n_sample problems."""
    oracle = load_oracle()
    idx = np.arange(min(n_sample, wl.ops.shape[0]))
    t0 = time.perf_counter()
    r = oracle.optimize(wl.X, wl.Y[idx], wl.ops[idx], wl.ch[idx], wl.C[idx], max_iter=max_iter, dot_mode=0)
    dt = time.perf_counter() - t0
    return len(idx) / dt, dt, oracle.num_threads(), r


def cpu_fit_workload(args, B, N):
    """The first problems of the benchmark's workload, built on the host only (the
    reference arm runs no GPU code): the same seeds as the GPU batch."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from cudasymbolicregression_gb300 import workloads

    def roots(X, ops, ch, C):
        cache = oracle.eval_fwd(X, ops, ch, C)
        root = np.maximum((ops != 0).sum(1) - 1, 0)
        return cache[np.arange(ops.shape[0]), root]
    if args.workload == "readme":
        return workloads.readme_fit(B=min(B, args.cpu_sample), N=N, seed=args.seed)
    if args.workload == "ragged":
        return workloads.ragged_fit(B=B, N=N, M=M_DEFAULT, seed=args.seed, root_eval=roots)
    return workloads.ragged_fit_chunks(B=B, N=N, M=M_DEFAULT, seed=args.seed, n_chunks=1, root_eval=roots)


def cpu_grammar_run(n, L, seed):
    """The oracle's sampler, parser and child table (OpenMP) on n expressions of the
    sampling workload: (expressions/s, seconds, threads)."""
    oracle = load_oracle()
    from cudasymbolicregression_gb300.pcfg import ProbabilisticContextFreeGrammar
    from cudasymbolicregression_gb300.workloads import SEARCH_GRAMMAR
    p = ProbabilisticContextFreeGrammar(SEARCH_GRAMMAR, "E", L, 3, torch.device("cpu"))
    t0 = time.perf_counter()
    rows, e1 = oracle.pcfg_sample(p._tables_np, p.get_symbol_id("E"), n, L, 64, seed)
    post, e2 = oracle.infix_parse(rows, 3)
    _, e3 = oracle.postfix_children(post)
    dt = time.perf_counter() - t0
    assert not (e1.any() or e2.any() or e3.any())
    return n / dt, dt, oracle.num_threads()


def run_reference(args, rank):
    if rank != 0:
        return
    B, N = args.B, args.N
    if args.workload == "gemm":
        print(json.dumps({"impl": "reference", "unavailable": "the warm-start network has no counterpart in the "
                          "reference"}), flush=True)
        return
    if args.workload == "sample":
        n = min(B, args.cpu_sample_expr)
        vals = []
        threads = 1
        for i in range(args.warmup + args.steps):
            v, dt, threads = cpu_grammar_run(n, N, args.seed + i)
            if i >= args.warmup:
                vals.append(v)
        value = statistics.median(vals)
        line = {"metric": SAMPLE_METRIC, "value": value, "unit": "expressions/s", "n_gpus": args.gpus,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * n / value,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int64",
                "data": "synthetic", "impl": "reference",
                "config": {"workload": f"grammar sampling: {n} expressions, infix padded to {N} (CPU sample)"},
                "cpu_baseline": {"value": value, "unit": "expressions/s", "cores": threads, "kind": "port",
                                 "sample": f"{n} expressions per step: sample, postfix, child table"},
                "e2e": {"value": value, "unit": "expressions/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
                "host_cores": os.cpu_count()}
        print(json.dumps(line), flush=True)
        return
    if args.workload == "eval":
        from cudasymbolicregression_gb300 import tapes
        rng = np.random.default_rng(args.seed)
        X = rng.uniform(-3, 3, (N, 4)).astype(np.float32)
        n = min(B, args.cpu_eval_sample)
        tb = tapes.generate(n, M_DEFAULT, seed=args.seed + 1, mean_length=20.0, n_vars=4, p_const_leaf=0.2)

        class _W:
            pass
        wl = _W()
        wl.X, wl.ops, wl.ch = X, tb.ops, tb.ch
        wl.C = rng.standard_normal((n, M_DEFAULT)).astype(np.float32)
        vals = []
        for i in range(args.warmup + args.steps):
            v, dt, ntapes, threads = cpu_eval_sample(wl, n, seconds=2.0)
            if i >= args.warmup:
                vals.append(v)
        value, unit, sample = statistics.median(vals), "GB/s", f"{n} tapes per pass, forward + adjoint"
        metric, workload = EVAL_METRIC, f"eval forward+adjoint: M={M_DEFAULT}, N={N}, n_vars=4 (CPU sample)"
        ms = None
    else:
        wl = cpu_fit_workload(args, B, N)
        n = args.cpu_sample
        vals = []
        threads = 1
        for i in range(args.warmup + args.steps):
            v, dt, threads, _ = cpu_sample_run(wl, n, max_iter=MAX_ITER if args.workload != "readme" else 100)
            if i >= args.warmup:
                vals.append(v)
        value, unit = statistics.median(vals), UNIT
        sample = f"first {n} problems of the workload, plain start, full max_iter"
        metric, workload = METRIC, f"{args.workload}: B={B}, N={N} (CPU sample of {n} problems)"
        ms = 1000.0 * n / value
    line = {"metric": metric, "value": value, "unit": unit, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": {"workload": workload},
            "cpu_baseline": {"value": value, "unit": unit, "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "host_cores": os.cpu_count()}
    print(json.dumps(line), flush=True)


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world, dev):
    from cudasymbolicregression_gb300 import sharding
    return sharding.max_over_ranks(x, device=dev) if world > 1 else x


def timed_steps(step, steps, flush):
    """CUDA-event time of each call of step(kernel_events) (L2 flushed before each)."""
    evs, kevs, r = [], [], None
    for _ in range(steps):
        flush.fill_(1.0)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        kev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
        e0.record()
        r = step(kev)
        e1.record()
        evs.append((e0, e1))
        kevs.append(kev)
    torch.cuda.synchronize()
    t = statistics.mean(a.elapsed_time(b) / 1000.0 for a, b in evs)
    tk = statistics.mean(a.elapsed_time(b) / 1000.0 for a, b in kevs)
    return t, tk, r


def fit_quality(r, ref_finite, max_iter, step_s=None):
    """Quality of one arm: median final MSE over the plain arm's finite problems
    (non-finite results count as +inf); the share of problems that end finite and the
    rate at which finite fits are produced; the share of closures spent on problems
    that end finite; iterations on the finite problems (median, mean, the share that
    reach tolerance_grad before max_iter, and the median iterations of those)."""
    loss = r.loss.cpu().numpy()
    it = r.iters.cpu().numpy()
    ev = r.evals.cpu().numpy().astype(np.float64)
    fin = np.isfinite(loss) & (it >= 0)
    lf = np.where(np.isfinite(loss), loss, np.inf)[ref_finite]
    conv = fin & (it < max_iter)
    q = {"median_final_mse": float(np.median(lf)) if lf.size else None,
         "p25_final_mse": float(np.percentile(lf, 25)) if lf.size else None,
         "finite_fraction": float(fin.mean()), "error_problems": int((it < 0).sum()),
         "mean_iters": float(it.mean()), "median_iters": float(np.median(it)),
         "stopped_before_max_iter": float(((it >= 0) & (it < max_iter)).mean()),
         "mean_closures": float(ev.mean()),
         "closure_share_finite": float(ev[fin].sum() / max(ev.sum(), 1.0)),
         "finite": {"median_iters": float(np.median(it[fin])) if fin.any() else None,
                    "mean_iters": float(it[fin].mean()) if fin.any() else None,
                    "converged_share": float(conv.sum() / max(fin.sum(), 1)),
                    "median_iters_to_tolerance": float(np.median(it[conv])) if conv.any() else None}}
    if step_s:
        q["finite_fitted_per_s"] = float(fin.sum() / step_s)
    return q


def paired_quality(r_warm, r_plain):
    """Per problem, the warm arm's final MSE against the plain arm's: over the problems
    finite in both, the shares within 1e-4 relative, lower and higher (with the median
    ratio of those that differ), and the problems finite in one arm only.

    Also the median final MSE of each arm over the problems finite in either arm
    (non-finite results count as +inf).  The median over the plain arm's finite problems
    (fit_quality) charges the warm arm +inf for every problem that only the plain start
    fits and ignores the ones that only the warm start fits; over the union both arms
    are charged alike."""
    a = r_warm.loss.cpu().numpy().astype(np.float64)
    b = r_plain.loss.cpu().numpy().astype(np.float64)
    fa, fb = np.isfinite(a) & (r_warm.iters.cpu().numpy() >= 0), np.isfinite(b) & (r_plain.iters.cpu().numpy() >= 0)
    return paired_stats(a, b, fa, fb)


def paired_stats(a, b, fa, fb):
    """paired_quality on arrays: final MSEs a (warm) and b (plain), finite masks fa, fb."""
    both = fa & fb
    either = fa | fb
    ua = np.where(fa, a, np.inf)[either]
    ub = np.where(fb, b, np.inf)[either]
    aa, bb = a[both], b[both]
    same = np.abs(aa - bb) <= 1e-4 * np.maximum(np.abs(bb), 1e-30)
    lower, higher = (aa < bb) & ~same, (aa > bb) & ~same
    diff = ~same
    ratio = np.maximum(aa[diff], 1e-30) / np.maximum(bb[diff], 1e-30)
    n = max(int(both.sum()), 1)
    return {"finite_in_both": int(both.sum()), "same_within_1e-4": float(same.sum() / n),
            "warm_lower": float(lower.sum() / n), "warm_higher": float(higher.sum() / n),
            "median_ratio_where_different": float(np.median(ratio)) if ratio.size else None,
            "finite_only_warm": int((fa & ~fb).sum()), "finite_only_plain": int((fb & ~fa).sum()),
            "finite_in_either": int(either.sum()),
            "median_final_mse_either_finite": {"warm": float(np.median(ua)) if ua.size else None,
                                               "plain": float(np.median(ub)) if ub.size else None}}


def fp64_check(r, X, Y, ops, ch, sample=4096):
    """The reported final MSE of a sample of finite problems against an FP64
    evaluation of the same constants (the library's float64 forward kernel): the
    median and largest relative difference."""
    import cudasymbolicregression_gb300 as sr
    loss = r.loss
    idx = torch.nonzero(torch.isfinite(loss)).flatten()[:sample]
    if idx.numel() == 0:
        return None
    o, c = ops[idx], ch[idx]
    with torch.no_grad():
        out = sr.evaluation.evaluate(X.double(), o, c, r.C[idx].double())
        root = ((o != 0).sum(1) - 1).clamp(min=0)
        f = out[torch.arange(idx.numel(), device=out.device), root]
        mse64 = ((f - Y[idx].double()) ** 2).mean(1)
    rel = ((loss[idx].double() - mse64).abs() / mse64.abs().clamp(min=1e-300)).cpu().numpy()
    rel = rel[np.isfinite(rel)]
    return {"problems": int(idx.numel()), "median_rel_diff": float(np.median(rel)) if rel.size else None,
            "max_rel_diff": float(rel.max()) if rel.size else None}


def train_warm_start(args, dev, n_vars):
    """The warm-start network trained (untimed) on the fits of other problems."""
    from cudasymbolicregression_gb300 import warmstart, workloads
    T = lambda a: torch.tensor(a, device=dev)  # noqa: E731
    probs, data = [], warmstart.TrainingSet([], [], [], [], [])
    t0 = time.perf_counter()
    for s in range(args.train_sets):
        if args.workload == "readme":
            wl = workloads.readme_fit(B=16384, seed=10_000 + s)
            mi = 100
        else:
            wl = workloads.ragged_fit(B=65536, N=args.N, M=M_DEFAULT, seed=10_000 + s, device=str(dev))
            mi = MAX_ITER
        X, Y, O, Ch, C = T(wl.X), T(wl.Y), T(wl.ops), T(wl.ch), T(wl.C)
        tgt, msk, _ = warmstart.fitted_examples(X, Y, O, Ch, C, max_iter=mi)
        probs.append((X, Y, O, Ch, C))
        data.X.append(X)
        data.Y.append(Y)
        data.ops.append(O)
        data.target.append(tgt)
        data.mask.append(msk)
    t_data = time.perf_counter() - t0
    net = warmstart.WarmStartMLP(device=dev, seed=args.seed, n_vars=n_vars)
    s1 = warmstart.train(net, data, epochs=args.train_epochs, batch=2048, lr=2e-3)
    s2 = warmstart.train_fit_objective(net, probs, epochs=args.train_epochs, batch=2048, lr=5e-4)
    torch.cuda.synchronize()
    info = {"training_problems": int(sum(p[2].shape[0] for p in probs)), "data_s": round(t_data, 1),
            "train_s": round(time.perf_counter() - t0 - t_data, 1), "steps": s1.steps + s2.steps,
            "objective": "constants of the plain fits, then the normalised fit MSE of the predictions"}
    return net, info


def run_fit(args, rank, world, local):
    import cudasymbolicregression_gb300 as sr
    from cudasymbolicregression_gb300 import warmstart, workloads

    dev = torch.device("cuda", local)
    B, N = args.B, args.N
    seed = args.seed + 1000 * rank
    if args.workload == "readme":
        wl = workloads.readme_fit(B=B, N=N, seed=seed)
        n_vars, max_iter = 1, 100
    elif args.workload == "ragged":
        wl = workloads.ragged_fit(B=B, N=N, M=M_DEFAULT, seed=seed, device=str(dev))
        n_vars, max_iter = 2, MAX_ITER
    else:
        wl = workloads.ragged_fit_chunks(B=B, N=N, M=M_DEFAULT, seed=seed, device=str(dev))
        n_vars, max_iter = 2, MAX_ITER
    warm = args.workload != "ragged"
    Xd, Yd, Od, Chd, Cd = (torch.tensor(a, device=dev) for a in (wl.X, wl.Y, wl.ops, wl.ch, wl.C))
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)
    net, train_info = train_warm_start(args, dev, n_vars) if warm else (None, None)
    draws = torch.Generator(device=dev)

    def fit_from(Cs, kev=None):
        return sr.optimize_ex(Xd, Yd, Od, Chd, Cs, max_iter=max_iter, raise_errors=False, kernel_events=kev)

    def plain_step(kev=None):
        return fit_from(Cd, kev)

    def screened(use_net, extra):
        """A step from the best of the plain start, the network's start (use_net) and
        `extra` randn draws, screened in one launch."""
        def step(kev=None):
            draws.manual_seed(seed + 17)
            Cs = warmstart.candidate_starts(Xd, Yd, Od, Cd, net if use_net else None, extra, generator=draws)
            return fit_from(warmstart.screened_start(Xd, Yd, Od, Chd, Cs), kev)
        return step

    arms = {"plain": plain_step}
    if warm:
        # warm: the network's start against the plain start; the ablations replace the
        # network by randn draws, and add two more draws to both (four candidates)
        arms.update({"warm": screened(True, 0), "randn_gate": screened(False, 1),
                     "net_multistart": screened(True, 2), "randn_multistart": screened(False, 3)})
    for _ in range(args.warmup):
        for fn in arms.values():
            fn()
    if warm:
        # the best any start can do: every problem starts at the constants its own plain
        # fit ended with (fixed before timing)
        C_own = plain_step().C
        C_own = torch.where(torch.isfinite(C_own), C_own, Cd)
        arms["own_answer"] = lambda kev=None: fit_from(C_own, kev)
        arms["own_answer"]()
    torch.cuda.synchronize()
    barrier(world)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("timed")
    timed = {}
    with ClockSampler(local) as clk:
        for name, fn in arms.items():
            timed[name] = timed_steps(fn, args.steps, flush)
    torch.cuda.nvtx.range_pop()
    barrier(world)
    t_plain, tk_plain, r_plain = timed["plain"]
    t_plain = max_over_ranks(t_plain, world, dev)
    head = "warm" if warm else "plain"
    head_t, head_tk, head_r = timed[head]
    head_t = max_over_ranks(head_t, world, dev)
    value = B * world / head_t

    ref_finite = np.isfinite(r_plain.loss.cpu().numpy())
    q_plain = fit_quality(r_plain, ref_finite, max_iter, t_plain)
    q_head = fit_quality(head_r, ref_finite, max_iter, head_t)
    q_head["fp64_check"] = fp64_check(head_r, Xd, Yd, Od, Chd)
    if warm:
        q_plain["fp64_check"] = fp64_check(r_plain, Xd, Yd, Od, Chd)
    evals = head_r.evals.cpu().numpy().astype(np.float64)
    flops = float((wl.flops_per_closure() * evals).sum())
    achieved_tflops = flops / head_tk / 1e12
    pk, pk_kind = peaks()
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = sm_count * 128 * 2 * float(pk.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12

    e2e = None
    if not args.no_e2e:
        hX, hY, hO, hCh, hC = (torch.tensor(a).pin_memory() for a in (wl.X, wl.Y, wl.ops, wl.ch, wl.C))
        h2d = sum(t.numel() * t.element_size() for t in (hX, hY, hO, hCh, hC))
        # the results come back into pinned host buffers, as the inputs go out of them
        Cf_h = torch.empty(tuple(wl.C.shape), dtype=torch.float32).pin_memory()
        Yf_h = torch.empty(tuple(wl.Y.shape), dtype=torch.float32).pin_memory()
        e2e_times = []
        for _ in range(max(1, args.steps)):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            X_, Y_, O_, Ch_, C_ = (t.to(dev, non_blocking=True) for t in (hX, hY, hO, hCh, hC))
            if warm:
                C_ = warmstart.gated_warm_start(net, X_, Y_, O_, Ch_, C_)
            re = sr.optimize_ex(X_, Y_, O_, Ch_, C_, max_iter=max_iter, raise_errors=False)
            Cf_h.copy_(re.C, non_blocking=True)
            Yf_h.copy_(re.Y, non_blocking=True)
            torch.cuda.current_stream(dev).synchronize()
            e2e_times.append(time.perf_counter() - t0)
        d2h = Cf_h.numel() * 4 + Yf_h.numel() * 4
        e2e = {"value": B * world / statistics.median(e2e_times), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h), "arm": "warm" if warm else "plain"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:  # the CPU baseline is an N=1 figure
        v, dt, threads, _ = cpu_sample_run(wl, args.cpu_sample, max_iter=max_iter)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"first {args.cpu_sample} problems, plain start, full max_iter={max_iter} ({dt:.1f} s)"}

    if rank == 0:
        names = {"warmstart": f"learned warm start on held-out ragged problems: B={B}, tapes U[3,64] over "
                              f"+-*/ sin cos exp log, 0..8 constants, n_vars=2, N={N}, history 10, "
                              f"max_iter={max_iter}, strong_wolfe, tol 1e-7",
                 "ragged": f"ragged batched L-BFGS: B={B} tapes U[3,64], 0..8 constants, n_vars=2, N={N}, "
                           f"history 10, max_iter={max_iter}, strong_wolfe, tol 1e-7, plain randn init",
                 "readme": f"README problem: B={B} expressions of the README grammar (infix <= 32 tokens), "
                           f"N={N}, Y = 2.5 cos(X0) - 1.5, max_iter={max_iter}, strong_wolfe, tol 1e-7"}
        # per step: tape staging + fit; the warm arm adds the network (random features,
        # features, 5 GEMMs), and tape staging + one screening launch
        launches_per_step = 2 + (9 if warm else 0)
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": head_t * 1000.0, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": names[args.workload], "B": B, "N": N, "M": M_DEFAULT if args.workload != "readme" else 32,
                           "arm": "warm" if warm else "plain", "l2": "flushed (256 MiB write) between steps"},
                "roofline": {"bound": "fp32", "achieved": achieved_tflops, "peak": fp32_peak, "unit": "TFLOP/s",
                             "frac": achieved_tflops / fp32_peak,
                             "traffic": FIT_TRAFFIC_BYTES.get((args.workload, B, N)),
                             "kernel": "fit_lbfgs_kernel", "kernel_ms": head_tk * 1000.0,
                             "issue_active_pct": FIT_PROFILE["issue_active_pct"],
                             "fp32_pipe_pct": FIT_PROFILE["fp32_pipe_pct"], "xu_pipe_pct": FIT_PROFILE["xu_pipe_pct"],
                             "ncu_profile": FIT_PROFILE,
                             "peak_kind": f"nominal: {sm_count} SMs x 128 FP32 lanes x 2 x sm_max_mhz "
                                          f"({pk_kind} clock); no measured FP32 peak exists"},
                "quality": q_head,
                "gpu_launches": launches_per_step * args.steps,
                "clocks": clk.summary()}
        if warm:
            line["plain"] = {"value": B * world / t_plain, "ms_per_step": t_plain * 1000.0, "quality": q_plain,
                             "kernel_ms": tk_plain * 1000.0}
            line["warm_vs_plain"] = (B * world / head_t) / (B * world / t_plain)
            line["fixed_final_mse"] = bool(q_head["median_final_mse"] <= q_plain["median_final_mse"] * 1.0001)
            line["paired_final_mse"] = paired_quality(head_r, r_plain)
            med = line["paired_final_mse"]["median_final_mse_either_finite"]
            line["fixed_final_mse_either_finite"] = bool(med["warm"] is not None and med["plain"] is not None
                                                         and med["warm"] <= med["plain"] * 1.0001)
            line["warm_start_training"] = train_info
            line["warm_start_candidates"] = ("per problem the lower initial loss of the plain randn start and the "
                                             "network's start, both measured in one launch of the screening kernel")
            extra = {}
            for name in ("randn_gate", "net_multistart", "randn_multistart", "own_answer"):
                t, tk, r = timed[name]
                t = max_over_ranks(t, world, dev)
                extra[name] = {"value": B * world / t, "ms_per_step": t * 1000.0, "vs_plain": t_plain / t,
                               "quality": fit_quality(r, ref_finite, max_iter, t)}
            extra["randn_gate"]["arm"] = "the plain start and one randn draw, screened alike"
            extra["net_multistart"]["arm"] = "the plain start, the network's start and 2 randn draws"
            extra["randn_multistart"]["arm"] = "the plain start and 3 randn draws"
            line["ablation"] = {k: extra[k] for k in ("randn_gate", "net_multistart", "randn_multistart")}
            line["start_at_own_answer"] = dict(
                extra["own_answer"],
                arm="every problem starts at the constants its own plain fit ended with: the most any warm start "
                    "can gain under the same stopping rule (max_iter, tolerance_grad)")
        if e2e:
            line["e2e"] = e2e
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)


def eval_bytes(ops: np.ndarray, N: int):
    """Algorithmic HBM bytes per tape of the forward (cache written once, node words,
    tape summary and constants read once) and of the adjoint (dense gradient read
    once, gradient of C written once, node words and constants read once)."""
    B, M = ops.shape
    fwd = 4 * M * N + 4 * M + 16 + 4 * M
    bwd = 4 * M * N + 4 * M + 4 * M + 16 + 4 * M
    return fwd * B, bwd * B


def cpu_eval_sample(wl, chunk: int, seconds: float = 10.0):
    """The CPU oracle port of the reference's forward + adjoint over consecutive
    chunks of the workload's tapes (wrapping around) until `seconds` have passed;
    returns algorithmic GB/s, seconds and tapes processed."""
    oracle = load_oracle()
    B, M = wl.ops.shape
    N = wl.X.shape[0]
    chunk = min(chunk, B)
    gout = np.zeros((chunk, M, N), np.float32)
    done, nbytes, start, t_total = 0, 0, 0, 0.0
    while t_total < seconds:
        idx = np.arange(start, start + chunk) % B
        ops, ch, C = wl.ops[idx], wl.ch[idx], wl.C[idx]
        gout[:] = 0.0
        gout[np.arange(chunk), np.maximum((ops != 0).sum(1) - 1, 0)] = 1.0
        t0 = time.perf_counter()
        oracle.eval_fwd(wl.X, ops, ch, C)
        oracle.eval_bwd(wl.X, ops, ch, C, gout, want_gx=False)
        t_total += time.perf_counter() - t0
        fb, bb = eval_bytes(ops, N)
        nbytes += fb + bb
        done += chunk
        start = (start + chunk) % B
    return nbytes / t_total / 1e9, t_total, done, oracle.num_threads()


def run_eval(args, rank, world, local):
    import cudasymbolicregression_gb300 as sr
    from cudasymbolicregression_gb300 import _lib, workloads
    from cudasymbolicregression_gb300.tape import compile_tapes

    dev = torch.device("cuda", local)
    B, N = args.B, args.N
    wl = workloads.eval_batch(B=B, N=N, M=M_DEFAULT, seed=args.seed + 1000 * rank, device=str(dev))
    M = M_DEFAULT
    Xd = torch.tensor(wl.X, device=dev)
    Od = torch.tensor(wl.ops, device=dev)
    Chd = torch.tensor(wl.ch, device=dev)
    Cd = torch.tensor(wl.C, device=dev).requires_grad_(True)
    root = torch.tensor(np.maximum((wl.ops != 0).sum(1) - 1, 0), device=dev)
    G = torch.zeros((B, M, N), dtype=torch.float32, device=dev)
    G[torch.arange(B, device=dev), root] = 1.0
    fwd_bytes, bwd_bytes = eval_bytes(wl.ops, N)

    def step():
        out = sr.evaluation.evaluate(Xd, Od, Chd, Cd)
        gC, = torch.autograd.grad(out, Cd, G)
        return gC

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    evs = []
    barrier(world)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("timed")
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            step()
            e1.record()
            evs.append((e0, e1))
        torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    barrier(world)
    t_step = statistics.mean(a.elapsed_time(b) / 1000.0 for a, b in evs)
    t_step = max_over_ranks(t_step, world, dev)
    value = (fwd_bytes + bwd_bytes) * world / t_step / 1e9

    # the two kernels alone, through the C ABI, on the launching stream
    tapes = compile_tapes(Od, Chd, Xd.shape[1])
    L = _lib.lib()
    st = _lib.stream_ptr(dev)
    cache = torch.empty((B, M, N), dtype=torch.float32, device=dev)
    gCk = torch.empty((B, M), dtype=torch.float32, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    Cp = Cd.detach()

    def fwd_k():
        _lib.check(L.sr_eval_forward_f32(_lib.ptr(Xd), N, Xd.shape[1], _lib.ptr(tapes.desc), _lib.ptr(tapes.meta),
                                         _lib.ptr(tapes.order), B, M, tapes.max_len, _lib.ptr(Cp), M, 1,
                                         _lib.ptr(cache), st), "sr_eval_forward_f32")

    def bwd_k():
        _lib.check(L.sr_eval_backward_f32(_lib.ptr(Xd), N, Xd.shape[1], _lib.ptr(tapes.desc), _lib.ptr(tapes.meta),
                                          _lib.ptr(tapes.order), B, M, tapes.max_len, _lib.ptr(Cp), M, 1,
                                          _lib.ptr(cache), _lib.ptr(G), _lib.ptr(gCk), None, _lib.ptr(status), st),
                   "sr_eval_backward_f32")

    ktimes = {}
    for name, fn in (("eval_forward_kernel", fwd_k), ("eval_backward_kernel", bwd_k)):
        for _ in range(3):
            fn()
        ts = []
        for _ in range(max(3, args.steps)):
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            ts.append((e0, e1))
        torch.cuda.synchronize()
        ktimes[name] = statistics.mean(a.elapsed_time(b) / 1000.0 for a, b in ts)
    assert int(status.item()) == 0
    del cache

    e2e = None
    if not args.no_e2e:
        hX = torch.tensor(wl.X).pin_memory()
        hO = torch.tensor(wl.ops).pin_memory()
        hCh = torch.tensor(wl.ch).pin_memory()
        hC = torch.tensor(wl.C).pin_memory()
        h2d = sum(t.numel() * t.element_size() for t in (hX, hO, hCh, hC))
        gC_h = torch.empty(tuple(wl.C.shape), dtype=torch.float32).pin_memory()
        loss_h = torch.empty((), dtype=torch.float32).pin_memory()
        ts = []
        for _ in range(max(1, args.steps)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            Xh, Oh, Chh = (t.to(dev, non_blocking=True) for t in (hX, hO, hCh))
            Ch_ = hC.to(dev, non_blocking=True).requires_grad_(True)
            out = sr.evaluation.evaluate(Xh, Oh, Chh, Ch_)
            rt = (Oh != 0).sum(1) - 1
            loss = out.gather(1, rt.clamp(min=0).view(-1, 1, 1).expand(-1, 1, N)).sum()
            loss.backward()
            gC_h.copy_(Ch_.grad, non_blocking=True)
            loss_h.copy_(loss.detach(), non_blocking=True)
            torch.cuda.current_stream(dev).synchronize()
            ts.append(time.perf_counter() - t0)
            del out, loss
        d2h = gC_h.numel() * 4 + loss_h.numel() * 4
        e2e = {"value": (fwd_bytes + bwd_bytes) * world / statistics.median(ts) / 1e9, "unit": "GB/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "path": "evaluate() + loss=sum of root outputs + loss.backward() from pinned host buffers"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:  # the CPU baseline is an N=1 figure
        v, dt, ntapes, threads = cpu_eval_sample(wl, args.cpu_eval_sample)
        cpu = {"value": v, "unit": "GB/s", "cores": threads, "kind": "port",
               "sample": f"{ntapes} tapes in chunks of {args.cpu_eval_sample}, forward + adjoint ({dt:.1f} s)"}

    if rank == 0:
        pk, pk_kind = peaks()
        hbm = float(pk["hbm_gbs"])
        dom = max(ktimes, key=ktimes.get)
        dom_bytes = bwd_bytes if dom == "eval_backward_kernel" else fwd_bytes
        ach = dom_bytes / ktimes[dom] / 1e9
        line = {"metric": EVAL_METRIC, "value": value, "unit": "GB/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_step * 1000.0, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": f"eval forward+adjoint: B={B} tapes, M={M}, N={N}, n_vars=4, mean length ~20, "
                                       "dense root-row gradient", "B": B, "N": N, "M": M,
                           "l2": f"inputs larger than L2 (cache {B * M * N * 4 / 1e9:.1f} GB)"},
                "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                             "traffic": EVAL_TRAFFIC_BYTES.get((dom, B, N)), "kernel": dom, "peak_kind": pk_kind},
                "kernels": {k: {"ms": v * 1000.0,
                                "GB/s": (bwd_bytes if k == "eval_backward_kernel" else fwd_bytes) / v / 1e9}
                            for k, v in ktimes.items()},
                "expressions_per_s": B * world / t_step,
                # per step: tape compile, padding fill, padding check, and one forward and
                # one adjoint grid per length class (<= 16, <= 32, longer) the batch reaches
                "gpu_launches": (3 + 2 * (1 + (tapes.max_len > 16) + (tapes.max_len > 32))) * args.steps,
                "clocks": clk.summary()}
        if e2e:
            line["e2e"] = e2e
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)


def search_target(X, seed, dev):
    """A hidden target: a random tape with exactly five operator nodes and N(0, 1)
    constants whose root values are finite and not constant, evaluated at X."""
    import cudasymbolicregression_gb300 as sr
    from cudasymbolicregression_gb300 import tapes
    rng = np.random.default_rng(seed)
    for attempt in range(1000):
        tb = tapes.generate(64, M_DEFAULT, seed=seed * 1000 + attempt, lengths=rng.integers(6, 12, 64), n_vars=X.shape[1],
                            p_const_leaf=0.3)
        for b in range(64):
            ops = tb.ops[b]
            nop = int(((ops >= 10) & (ops < 50)).sum())
            if nop != 5:
                continue
            C = rng.standard_normal((1, M_DEFAULT)).astype(np.float32)
            with torch.no_grad():
                out = sr.evaluation.evaluate(torch.tensor(X, device=dev), torch.tensor(ops[None], device=dev),
                                             torch.tensor(tb.ch[b][None], device=dev), torch.tensor(C, device=dev))
            y = out[0, int((ops != 0).sum()) - 1].cpu().numpy()
            if np.isfinite(y).all() and y.std() > 1e-2 and np.abs(y).max() < 1e3:
                return y.astype(np.float32), ops, tb.ch[b], C[0]
    raise RuntimeError("no target found")


def run_search(args, rank, world, local):
    """Config 5: rounds of sampling + fitting against one hidden target, plain vs warm."""
    import cudasymbolicregression_gb300 as sr
    from cudasymbolicregression_gb300 import warmstart, workloads, tapes

    dev = torch.device("cuda", local)
    B, N, n_vars, max_iter = args.B, args.N, 3, 100
    rng = np.random.default_rng(args.seed + 1000 * rank)
    X = rng.uniform(-3, 3, (N, n_vars)).astype(np.float32)
    y, t_ops, _, _ = search_target(X, args.seed + 17, dev)
    Xd = torch.tensor(X, device=dev)
    Yd = torch.tensor(y, device=dev).unsqueeze(0).expand(B, N).contiguous()
    Xs = X[rng.choice(N, size=32, replace=False)]
    net = warmstart.WarmStartMLP(device=dev, seed=args.seed, n_vars=n_vars)
    arms = {"plain": {"t": 0.0, "first_hit_s": None, "best": float("inf"), "mean_closures": []},
            "warm": {"t": 0.0, "first_hit_s": None, "best": float("inf"), "mean_closures": [], "train_s": 0.0}}
    gen_s = 0.0
    # one-time set-up (library load, kernel attributes, workspace sizes) off the clock
    tw = tapes.generate(512, M_DEFAULT, seed=1, mean_length=8.0, n_vars=n_vars, p_const_leaf=0.3)
    sr.optimize_ex(Xd, Yd[:512], torch.tensor(tw.ops, device=dev), torch.tensor(tw.ch, device=dev),
                   torch.randn(512, M_DEFAULT, device=dev), max_iter=2, raise_errors=False)
    warmstart.gated_warm_start(net, Xd, Yd[:512], torch.tensor(tw.ops, device=dev), torch.tensor(tw.ch, device=dev),
                               torch.randn(512, M_DEFAULT, device=dev))
    # the training step's first call loads torch's gather/scatter kernels (seconds, once per process)
    warm_net = warmstart.WarmStartMLP(device=dev, seed=args.seed + 1, n_vars=n_vars)
    warmstart.train_fit_objective(warm_net, [(Xd[:256], Yd[:512, :256].contiguous(), torch.tensor(tw.ops, device=dev),
                                              torch.tensor(tw.ch, device=dev), torch.randn(512, M_DEFAULT, device=dev))],
                                  epochs=1, batch=512, lr=5e-4)
    torch.cuda.synchronize()
    n_train = min(B, 16384)
    n_pts = min(N, 256)
    grammar = None
    if args.candidates == "pcfg":
        from cudasymbolicregression_gb300.pcfg import ProbabilisticContextFreeGrammar
        grammar = ProbabilisticContextFreeGrammar(workloads.SEARCH_GRAMMAR, "E", M_DEFAULT, n_vars, dev)
        grammar.sample(1024)  # first launch (kernel attributes) off the clock
    with ClockSampler(local) as clk:
        for r in range(args.rounds):
            t0 = time.perf_counter()
            if args.candidates == "pcfg":
                # the grammar object on the device: sample -> postfix -> child table, randn constants
                torch.manual_seed(args.seed * 100 + r)
                O, Ch = grammar.sample(B)
                C = sr.create_constants(O)
            else:
                C0 = rng.standard_normal((B, M_DEFAULT)).astype(np.float32)
                tb = tapes.generate(B, M_DEFAULT, seed=args.seed * 100 + r, mean_length=8.0, n_vars=n_vars,
                                    p_const_leaf=0.3, X_screen=Xs, C_screen=C0,
                                    screen_fn=lambda o, c, Xs_, Cs_: workloads._gpu_zero_denominators(
                                        Xs_, o, c, Cs_, str(dev)))
                O, Ch, C = (torch.tensor(a, device=dev) for a in (tb.ops, tb.ch, C0))
            torch.cuda.synchronize()
            gen_s += time.perf_counter() - t0
            for name in ("plain", "warm"):
                a = arms[name]
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                Cs = C if (name == "plain" or r == 0) else warmstart.gated_warm_start(net, Xd, Yd, O, Ch, C)
                res = sr.optimize_ex(Xd, Yd, O, Ch, Cs, max_iter=max_iter, raise_errors=False)
                e1.record()
                e1.synchronize()
                a["t"] += e0.elapsed_time(e1) / 1000.0
                from cudasymbolicregression_gb300 import sharding
                best, _ = sharding.best_over_ranks(res.loss, offset=rank * B, device=dev)  # over all ranks
                a["best"] = min(a["best"], best)
                if a["first_hit_s"] is None and best < 1e-6:
                    a["first_hit_s"] = a["t"]
                a["mean_closures"].append(float(res.evals.float().mean()))
                if name == "plain":
                    plain_res = res
            # the warm arm's network learns from this round's plain fits (timed into the warm arm)
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            # a sample of the round's problems; the fit objective on a subset of the points
            sel = torch.randperm(B, device=dev)[:n_train]
            tgt, msk = warmstart.constant_targets(O[sel], plain_res.C[sel])
            ok = torch.isfinite(plain_res.loss[sel]) & (plain_res.iters[sel] >= 0)
            ok &= ((tgt.abs() <= 10) | (msk == 0)).all(dim=1) & torch.isfinite(tgt).all(dim=1)
            msk = msk * ok.unsqueeze(1).float()
            data = warmstart.TrainingSet([Xd], [Yd[sel]], [O[sel]], [torch.nan_to_num(tgt) * msk], [msk])
            warmstart.train(net, data, epochs=2, batch=4096, lr=2e-3)
            warmstart.train_fit_objective(net, [(Xd[:n_pts], Yd[sel, :n_pts].contiguous(), O[sel], Ch[sel], C[sel])],
                                          epochs=1, batch=4096, lr=5e-4)
            torch.cuda.synchronize()
            tr = time.perf_counter() - t1
            arms["warm"]["train_s"] += tr
            arms["warm"]["t"] += tr
    if rank == 0:
        total = B * args.rounds
        out = {}
        for name, a in arms.items():
            out[name] = {"expressions_per_s": total / a["t"], "seconds": a["t"], "first_mse_below_1e-6_s": a["first_hit_s"],
                         "best_mse": a["best"], "mean_closures_per_round": a["mean_closures"]}
            if "train_s" in a:
                out[name]["online_training_s"] = a["train_s"]
        line = {"metric": METRIC, "value": out["warm"]["expressions_per_s"], "unit": UNIT, "n_gpus": world,
                "steps": args.rounds, "warmup": 0, "ms_per_step": 1000.0 * arms["warm"]["t"] / args.rounds,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": f"full search round: {args.rounds} rounds of B={B} new expressions ("
                                       + ("drawn on the device from a 17-rule grammar, mean postfix length 6.7"
                                          if args.candidates == "pcfg" else "host generator, mean length 8")
                                       + f", padded 64, +-*/ sin cos exp log, 3 variables) fitted to N={N} points of "
                                       "one hidden 5-operator target, max_iter=100; warm arm trained online after "
                                       "every round", "B": B, "N": N, "candidates": args.candidates,
                           "target_ops": [int(v) for v in t_ops[t_ops != 0]]},
                "arms": out, "warm_vs_plain": out["warm"]["expressions_per_s"] / out["plain"]["expressions_per_s"],
                "generation_s": gen_s, "clocks": clk.summary()}
        print(json.dumps(line), flush=True)


def run_sample(args, rank, world, local):
    """The grammar object feeding a search: sample(B) = sampler -> infix to postfix ->
    child table on the device, one host synchronisation (the error check) per step."""
    from cudasymbolicregression_gb300 import _lib
    from cudasymbolicregression_gb300.pcfg import ProbabilisticContextFreeGrammar
    from cudasymbolicregression_gb300.workloads import SEARCH_GRAMMAR

    dev = torch.device("cuda", local)
    B, L = args.B, args.N
    pcfg = ProbabilisticContextFreeGrammar(SEARCH_GRAMMAR, "E", L, 3, dev)
    torch.manual_seed(args.seed + 1000 * rank)
    for _ in range(args.warmup):
        ops, ch = pcfg.sample(B)
    torch.cuda.synchronize()
    evs = []
    barrier(world)
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            ops, ch = pcfg.sample(B)
            e1.record()
            evs.append((e0, e1))
        torch.cuda.synchronize()
    barrier(world)
    t_step = max_over_ranks(statistics.mean(a.elapsed_time(b) / 1000.0 for a, b in evs), world, dev)
    value = B * world / t_step
    ok = int((ops != 0).any(dim=1).sum())
    mean_len = float((ops != 0).sum(dim=1).float().mean())

    # the three kernels alone, through the C ABI, on the launching stream
    lib, st = _lib.lib(), _lib.stream_ptr(dev)
    nt, cum, rp, rc = pcfg._tables
    infix = torch.empty((B, L), dtype=torch.int64, device=dev)
    post = torch.empty((B, L), dtype=torch.int64, device=dev)
    chk = torch.empty((B, L, 2), dtype=torch.int64, device=dev)
    err = torch.empty((3, B), dtype=torch.int64, device=dev)
    start = pcfg.get_symbol_id("E")
    calls = {
        "sample_infix_kernel": lambda: lib.sr_pcfg_sample_infix(_lib.ptr(nt), _lib.ptr(cum), _lib.ptr(rp), _lib.ptr(rc),
                                                                int(nt.numel() - 1), start, B, L, 64, 12345,
                                                                _lib.ptr(infix), _lib.ptr(err[0]), st),
        "infix_parse_kernel<postfix>": lambda: lib.sr_infix_to_postfix(_lib.ptr(infix), B, L, 3, _lib.ptr(post),
                                                                       _lib.ptr(err[1]), st),
        "postfix_children_kernel": lambda: lib.sr_postfix_children(_lib.ptr(post), B, L, 3, _lib.ptr(chk),
                                                                   _lib.ptr(err[2]), st),
    }
    algo = {"sample_infix_kernel": B * (L * 8 + 8), "infix_parse_kernel<postfix>": B * (2 * L * 8 + 8),
            "postfix_children_kernel": B * (L * 8 + 2 * L * 8 + 8)}
    ktimes = {}
    for name, fn in calls.items():
        for _ in range(3):
            _lib.check(fn(), name)
        ts = []
        for _ in range(max(3, args.steps)):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            _lib.check(fn(), name)
            e1.record()
            ts.append((e0, e1))
        torch.cuda.synchronize()
        ktimes[name] = statistics.mean(a.elapsed_time(b) / 1000.0 for a, b in ts)
    assert int((err != 0).sum()) == 0

    e2e = None
    if not args.no_e2e:
        h_ops = torch.empty((B, L), dtype=torch.int64).pin_memory()
        h_ch = torch.empty((B, L, 2), dtype=torch.int64).pin_memory()
        ts = []
        for _ in range(max(1, args.steps)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            o, c = pcfg.sample(B)
            h_ops.copy_(o, non_blocking=True)
            h_ch.copy_(c, non_blocking=True)
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        e2e = {"value": B * world / statistics.median(ts), "unit": "expressions/s", "h2d_bytes_per_step": 0,
               "d2h_bytes_per_step": int(B * L * 8 * 3),
               "path": "ProbabilisticContextFreeGrammar.sample(B), then Ops and Ch copied to pinned host memory"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:  # the CPU baseline is an N=1 figure
        n = min(B, args.cpu_sample_expr)
        v, dt, threads = cpu_grammar_run(n, L, args.seed)
        cpu = {"value": v, "unit": "expressions/s", "cores": threads, "kind": "port",
               "sample": f"{n} expressions: sample, postfix, child table ({dt:.2f} s)"}

    if rank == 0:
        pk, pk_kind = peaks()
        hbm = float(pk["hbm_gbs"])
        dom = max(ktimes, key=ktimes.get)
        ach = algo[dom] / ktimes[dom] / 1e9
        line = {"metric": SAMPLE_METRIC, "value": value, "unit": "expressions/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_step * 1000.0, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "int64", "data": "synthetic",
                "config": {"workload": f"grammar sampling: B={B} expressions of a 17-rule grammar (+ - * / sin cos exp "
                                       f"log over X_0..X_2 and C), infix padded to {L} tokens, then postfix and the "
                                       "child table", "B": B, "L": L, "mean_postfix_length": mean_len,
                           "nonempty": ok, "l2": f"outputs larger than L2 ({B * L * 32 / 1e9:.1f} GB per step)"},
                "roofline": {"bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s", "frac": ach / hbm,
                             "traffic": None, "kernel": dom, "peak_kind": pk_kind},
                "kernels": {k: {"ms": v * 1000.0, "GB/s": algo[k] / v / 1e9} for k, v in ktimes.items()},
                "gpu_launches": 3 * args.steps, "clocks": clk.summary()}
        if e2e:
            line["e2e"] = e2e
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)


def run_gemm(args, rank, world, local):
    import ctypes
    from cudasymbolicregression_gb300 import _lib

    dev = torch.device("cuda", local)
    rows, k, n = args.B, args.N, GEMM_N
    g = torch.Generator(device=dev)
    g.manual_seed(args.seed + 1000 * rank)
    A = (torch.randn((rows, k), generator=g, device=dev) * 0.1).to(torch.bfloat16)
    W = (torch.randn((n, k), generator=g, device=dev) * 0.1).to(torch.bfloat16)
    out = torch.empty((rows, n), dtype=torch.bfloat16, device=dev)
    status = torch.zeros(1, dtype=torch.int32, device=dev)
    L, st = _lib.lib(), _lib.stream_ptr(dev)
    epi = _lib.MlpEpilogue()
    epi.epilogue = _lib.MLP_EPI_LINEAR
    epi.ld_out = n

    def gemm(a, w, o):
        epi.out = o.data_ptr()
        _lib.check(L.sr_mlp_gemm(ctypes.c_void_p(a.data_ptr()), rows, k, k, ctypes.c_void_p(w.data_ptr()), n, k,
                                 ctypes.byref(epi), ctypes.c_void_p(status.data_ptr()), st), "sr_mlp_gemm")

    for _ in range(args.warmup):
        for _r in range(GEMM_REPS):
            gemm(A, W, out)
    torch.cuda.synchronize()
    # a block of rows against torch's product of the same bf16 operands (fp32 accumulation;
    # the outputs are rounded to bf16)
    ref = A[:1024].float() @ W.float().T
    rel = float((out[:1024].float() - ref).abs().max() / ref.abs().max())
    assert int(status.item()) == 0 and rel < 1e-2, (int(status.item()), rel)
    flops = 2.0 * rows * n * k
    nbytes = 2.0 * (rows * k + n * k + rows * n)
    barrier(world)
    torch.cuda.synchronize()
    evs = []
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _r in range(GEMM_REPS):
                gemm(A, W, out)
            e1.record()
            evs.append((e0, e1))
        torch.cuda.synchronize()
    barrier(world)
    t_step = max_over_ranks(statistics.mean(a.elapsed_time(b) / 1000.0 for a, b in evs), world, dev)
    t = t_step / GEMM_REPS  # one GEMM
    value = flops * world / t / 1e12

    e2e = None
    if not args.no_e2e:
        hA, hW = A.cpu().pin_memory(), W.cpu().pin_memory()
        hO = torch.empty((rows, n), dtype=torch.bfloat16).pin_memory()
        ts = []
        for _ in range(max(1, args.steps)):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            a_d, w_d = hA.to(dev, non_blocking=True), hW.to(dev, non_blocking=True)
            gemm(a_d, w_d, out)
            hO.copy_(out, non_blocking=True)
            torch.cuda.synchronize()
            ts.append(time.perf_counter() - t0)
        e2e = {"value": flops * world / statistics.median(ts) / 1e12, "unit": "TFLOP/s",
               "h2d_bytes_per_step": int(2 * (rows * k + n * k)), "d2h_bytes_per_step": int(2 * rows * n),
               "path": "one sr_mlp_gemm with A and W copied from pinned host memory and D copied back"}

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        # numpy's float32 matmul (the host BLAS, all cores) of the first 8192 rows
        m = min(rows, 8192)
        a32, w32 = A[:m].float().cpu().numpy(), W.float().cpu().numpy()
        a32 @ w32.T
        t0 = time.perf_counter()
        reps = 0
        while time.perf_counter() - t0 < 3.0:
            a32 @ w32.T
            reps += 1
        dt = (time.perf_counter() - t0) / reps
        cpu = {"value": 2.0 * m * n * k / dt / 1e12, "unit": "TFLOP/s", "cores": os.cpu_count(), "kind": "port",
               "sample": f"numpy float32 matmul of {m} x {k} by {k} x {n} ({reps} repetitions)"}

    if rank == 0:
        pk, pk_kind = peaks()
        peak = float(pk["bf16_tflops"])
        hbm = float(pk["hbm_gbs"])
        line = {"metric": GEMM_METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_step * 1000.0, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "bf16", "data": "synthetic",
                "config": {"workload": f"D ({rows} x {n}) = A ({rows} x {k}) . W ({n} x {k})^T, bf16 operands, "
                                       "fp32 accumulation, bf16 output", "rows": rows, "k": k, "n": n,
                           "l2": f"inputs larger than L2 ({rows * k * 2 / 1e9:.1f} GB of A)",
                           "gemms_per_step": GEMM_REPS, "ms_per_gemm": t * 1000.0,
                           "max_rel_err_first_1024_rows": rel},
                "roofline": {"bound": "tensor", "achieved": value, "peak": peak, "unit": "TFLOP/s",
                             "frac": value / peak, "traffic": None, "kernel": "mlp::gemm_kernel<256>",
                             "peak_kind": pk_kind + " (bf16 burst)",
                             "hbm": {"GB/s": nbytes / t / 1e9, "frac": nbytes / t / 1e9 / hbm}},
                "gpu_launches": args.steps * GEMM_REPS, "clocks": clk.summary()}
        if e2e:
            line["e2e"] = e2e
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="warmstart", choices=list(DEFAULTS))
    ap.add_argument("--B", type=int, default=None)
    ap.add_argument("--N", type=int, default=None)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--train-sets", type=int, default=16)
    ap.add_argument("--train-epochs", type=int, default=4)
    ap.add_argument("--rounds", type=int, default=10)
    ap.add_argument("--cpu-sample", type=int, default=512)
    ap.add_argument("--cpu-eval-sample", type=int, default=4096)
    ap.add_argument("--cpu-sample-expr", type=int, default=1048576)
    ap.add_argument("--candidates", default="pcfg", choices=["pcfg", "tapes"],
                    help="search workload: candidates from the device grammar sampler or the host generator")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()
    dB, dN = DEFAULTS[args.workload]
    args.B = dB if args.B is None else args.B
    args.N = dN if args.N is None else args.N

    rank, world, local = dist_env()
    if args.impl == "reference":
        # the CPU port on rank 0 alone: no GPU and no process group; the other ranks
        # exit without work
        run_reference(args, rank)
        return
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    if args.workload == "eval":
        run_eval(args, rank, world, local)
    elif args.workload == "search":
        run_search(args, rank, world, local)
    elif args.workload == "sample":
        run_sample(args, rank, world, local)
    elif args.workload == "gemm":
        run_gemm(args, rank, world, local)
    else:
        run_fit(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
