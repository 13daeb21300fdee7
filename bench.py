"""Benchmark: expressions fitted per second by the fused batched L-BFGS kernel.

Workload (one "step"): the ragged batched L-BFGS configuration -- B=16384 tapes of
uniform length 3..64 with 0..8 learnable constants, n_variables=2, N=512 points,
X ~ U[-3, 3], targets = hidden random expressions + N(0, 0.01^2) noise, history 10,
max_iter=200, strong Wolfe, tolerance_grad=1e-7 -- fitted by one optimize() call.
Seeded synthetic data (no dataset is involved).

`value`   = B / (device time of one step), inputs resident in HBM, L2 flushed
            between steps (a 256 MiB buffer is rewritten before each timed step).
`e2e`     = the same through optimize() from pinned host buffers, host->device
            copies of X, Y, Ops, Ch, C_init and the device->host copy of
            C_final, Y_final inside the timed region.
`roofline`= the fit kernel's algorithmic FP32 rate (op table in
            cudasymbolicregression_gb300/workloads.py) over its CUDA-event time.
`cpu_baseline` = the CPU oracle port of the reference's optimize() on a bounded
            sample of the same problems, all host threads.

--impl reference runs only that CPU port (the reference's own CPU path,
restated) and prints its line.
Multi-GPU: one process per GPU; every rank fits its own batch of B problems
(independent seeds, no collective), value = all problems / max time.

--workload eval measures the evaluation path instead (B=65536 tapes of padded
length 64 over {+,-,*,/,sin,cos,exp,log,X0..X3,C}, mean length about 20,
N=1024, X ~ U[-3, 3], C ~ N(0, 1)): one step is evaluate() forward plus the
adjoint of a dense gradient that is 1 on every root row (the gradient of the sum
of root outputs), value = algorithmic HBM bytes / step time.
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
B_DEFAULT, N_DEFAULT, M_DEFAULT = 16384, 512, 64
MAX_ITER = 200
EVAL_METRIC = "evaluation forward+adjoint throughput (algorithmic HBM bytes)"
EVAL_B, EVAL_N = 65536, 1024

# DRAM bytes (read + write) of one launch of the dominant kernel on the default
# workloads, from ncu captures of a 4x / 16x smaller batch scaled by the number of
# problems (profiles/fit_lbfgs_ragged_B16384_N512.txt,
# profiles/eval_forward_B4096_N1024.txt).
FIT_TRAFFIC_BYTES = {(16384, 512): 4 * (10722048 + 24576)}
EVAL_TRAFFIC_BYTES = {("eval_forward_kernel", 65536, 1024): 16 * (1611520 + 1012199000)}


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


def cpu_sample_run(wl, n_sample: int, threads: int | None = None):
    """The CPU oracle port of optimize() on the first n_sample problems."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # the checker / CPU baseline only
    oracle.build()
    if threads:
        os.environ["OMP_NUM_THREADS"] = str(threads)
    idx = np.arange(min(n_sample, wl.B))
    t0 = time.perf_counter()
    r = oracle.optimize(wl.X, wl.Y[idx], wl.ops[idx], wl.ch[idx], wl.C[idx], max_iter=MAX_ITER, dot_mode=0)
    dt = time.perf_counter() - t0
    return len(idx) / dt, dt, oracle.num_threads(), r


def run_reference(args, rank):
    if rank != 0:
        return
    from cudasymbolicregression_gb300 import workloads
    wl = workloads_cpu_fit(args)
    n = args.cpu_sample
    vals = []
    cores = os.cpu_count()
    for i in range(args.warmup + args.steps):
        v, dt, threads, _ = cpu_sample_run(wl, n)
        if i >= args.warmup:
            vals.append(v)
    value = statistics.median(vals)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1000.0 * n / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic", "impl": "reference",
            "config": {"workload": f"ragged batched L-BFGS, B={args.B}, N={args.N}, M={M_DEFAULT}, "
                                   f"max_iter={MAX_ITER}, strong_wolfe (CPU sample of {n} problems)"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": f"first {n} problems of the workload, full max_iter={MAX_ITER}"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "host_cores": cores}
    print(json.dumps(line), flush=True)


def workloads_cpu_fit(args):
    """The same seeded workload, hidden targets evaluated by the CPU port (the
    reference arm runs no GPU code)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from cudasymbolicregression_gb300 import workloads

    def roots(X, ops, ch, C):
        cache = oracle.eval_fwd(X, ops, ch, C)
        root = np.maximum((ops != 0).sum(1) - 1, 0)
        return cache[np.arange(ops.shape[0]), root]
    return workloads.ragged_fit(B=args.B, N=args.N, M=M_DEFAULT, seed=args.seed, root_eval=roots)


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, world, dev):
    if world > 1:
        import torch.distributed as dist
        t = torch.tensor([x], device=dev, dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())
    return x


def run_fit(args, rank, world, local):
    import cudasymbolicregression_gb300 as sr
    from cudasymbolicregression_gb300 import workloads

    dev = torch.device("cuda", local)
    wl = workloads.ragged_fit(B=args.B, N=args.N, M=M_DEFAULT, seed=args.seed + 1000 * rank)
    Xd = torch.tensor(wl.X, device=dev)
    Yd = torch.tensor(wl.Y, device=dev)
    Od = torch.tensor(wl.ops, device=dev)
    Chd = torch.tensor(wl.ch, device=dev)
    Cd = torch.tensor(wl.C, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step(kev=None):
        return sr.optimize_ex(Xd, Yd, Od, Chd, Cd, max_iter=MAX_ITER, raise_errors=False, kernel_events=kev)

    for _ in range(args.warmup):
        r = step()
    torch.cuda.synchronize()

    evs, kevs = [], []
    barrier(world)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_push("timed")
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            kev = (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
            e0.record()
            r = step(kev)
            e1.record()
            evs.append((e0, e1))
            kevs.append(kev)
        torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    barrier(world)
    t_step = statistics.mean(a.elapsed_time(b) / 1000.0 for a, b in evs)
    t_kernel = statistics.mean(a.elapsed_time(b) / 1000.0 for a, b in kevs)
    t_step = max_over_ranks(t_step, world, dev)
    value = args.B * world / t_step

    # quality and work accounting from the last step
    iters = r.iters.cpu().numpy()
    evals = r.evals.cpu().numpy().astype(np.float64)
    loss = r.loss.cpu().numpy()
    flops = float((wl.flops_per_closure() * evals).sum())
    achieved_tflops = flops / t_kernel / 1e12
    pk, pk_kind = peaks()
    sm_count = torch.cuda.get_device_properties(dev).multi_processor_count
    fp32_peak = sm_count * 128 * 2 * float(pk.get("sm_max_mhz", 2070.0)) * 1e6 / 1e12

    # end-to-end through the public API from pinned host buffers
    e2e = None
    if not args.no_e2e:
        hX = torch.tensor(wl.X).pin_memory()
        hY = torch.tensor(wl.Y).pin_memory()
        hO = torch.tensor(wl.ops).pin_memory()
        hCh = torch.tensor(wl.ch).pin_memory()
        hC = torch.tensor(wl.C).pin_memory()
        h2d = sum(t.numel() * t.element_size() for t in (hX, hY, hO, hCh, hC))
        e2e_times = []
        for i in range(max(1, args.steps)):
            flush.fill_(1.0)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            re = sr.optimize_ex(hX.to(dev, non_blocking=True), hY.to(dev, non_blocking=True),
                                hO.to(dev, non_blocking=True), hCh.to(dev, non_blocking=True),
                                hC.to(dev, non_blocking=True), max_iter=MAX_ITER, raise_errors=False)
            Cf_h, Yf_h = re.C.cpu(), re.Y.cpu()
            e2e_times.append(time.perf_counter() - t0)
        d2h = Cf_h.numel() * 4 + Yf_h.numel() * 4
        e2e = {"value": args.B * world / statistics.median(e2e_times), "unit": UNIT, "h2d_bytes_per_step": int(h2d),
               "d2h_bytes_per_step": int(d2h)}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        v, dt, threads, _ = cpu_sample_run(wl, args.cpu_sample)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"first {args.cpu_sample} problems, full max_iter={MAX_ITER} ({dt:.1f} s)"}

    if rank == 0:
        fin = np.isfinite(loss)
        traffic = FIT_TRAFFIC_BYTES.get((args.B, args.N))
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_step * 1000.0, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": f"ragged batched L-BFGS: B={args.B} tapes, lengths U[3,64], 0..8 constants, "
                                       f"n_vars=2, N={args.N}, history 10, max_iter={MAX_ITER}, strong_wolfe, "
                                       "tol 1e-7, plain randn init",
                           "B": args.B, "N": args.N, "M": M_DEFAULT, "l2": "flushed (256 MiB write) between steps"},
                "roofline": {"bound": "fp32", "achieved": achieved_tflops, "peak": fp32_peak, "unit": "TFLOP/s",
                             "frac": achieved_tflops / fp32_peak, "traffic": traffic,
                             "kernel": "fit_lbfgs_kernel", "kernel_ms": t_kernel * 1000.0,
                             "peak_kind": f"nominal: {sm_count} SMs x 128 FP32 lanes x 2 x sm_max_mhz "
                                          f"({pk_kind} clock); no measured FP32 peak exists"},
                "quality": {"median_final_mse": float(np.median(loss[fin])) if fin.any() else None,
                            "error_problems": int((iters < 0).sum()),
                            "nan_fraction": float(1 - fin.mean()), "mean_iters": float(iters.mean()),
                            "mean_closures": float(evals.mean())},
                "gpu_launches": 2 * args.steps,
                "clocks": clk.summary()}
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
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle  # the checker / CPU baseline only
    oracle.build()
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
    B = args.B if args.B != B_DEFAULT else EVAL_B
    N = args.N if args.N != N_DEFAULT else EVAL_N
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
                                          _lib.ptr(tapes.order), B, M, tapes.max_len, _lib.ptr(Cp), M, 1, _lib.ptr(G),
                                          _lib.ptr(gCk), None, _lib.ptr(status), st), "sr_eval_backward_f32")

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
            gC_h, loss_h = Ch_.grad.cpu(), loss.detach().cpu()
            ts.append(time.perf_counter() - t0)
            del out, loss
        d2h = gC_h.numel() * 4 + loss_h.numel() * 4
        e2e = {"value": (fwd_bytes + bwd_bytes) * world / statistics.median(ts) / 1e9, "unit": "GB/s",
               "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
               "path": "evaluate() + loss=sum of root outputs + loss.backward() from pinned host buffers"}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
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
                "gpu_launches": 3 * args.steps,
                "clocks": clk.summary()}
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
    ap.add_argument("--workload", default="fit", choices=["fit", "eval"])
    ap.add_argument("--B", type=int, default=B_DEFAULT)
    ap.add_argument("--N", type=int, default=N_DEFAULT)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-sample", type=int, default=512)
    ap.add_argument("--cpu-eval-sample", type=int, default=4096)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    args = ap.parse_args()

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    if args.impl == "reference":
        run_reference(args, rank)
    else:
        torch.cuda.set_device(local)
        if args.workload == "fit":
            run_fit(args, rank, world, local)
        else:
            run_eval(args, rank, world, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
