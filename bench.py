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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--B", type=int, default=B_DEFAULT)
    ap.add_argument("--N", type=int, default=N_DEFAULT)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-sample", type=int, default=48)
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
        return

    import cudasymbolicregression_gb300 as sr
    from cudasymbolicregression_gb300 import workloads

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    wl = workloads.ragged_fit(B=args.B, N=args.N, M=M_DEFAULT, seed=args.seed + 1000 * rank)
    Xd = torch.tensor(wl.X, device=dev)
    Yd = torch.tensor(wl.Y, device=dev)
    Od = torch.tensor(wl.ops, device=dev)
    Chd = torch.tensor(wl.ch, device=dev)
    Cd = torch.tensor(wl.C, device=dev)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=dev)

    def step():
        return sr.optimize_ex(Xd, Yd, Od, Chd, Cd, max_iter=MAX_ITER, raise_errors=False)

    for _ in range(args.warmup):
        r = step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    evs = []
    barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.fill_(1.0)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record()
            r = step()
            e1.record()
            evs.append((e0, e1))
        torch.cuda.synchronize()
    barrier()
    times = [a.elapsed_time(b) / 1000.0 for a, b in evs]
    t_step = sum(times) / len(times)
    if world > 1:
        import torch.distributed as dist
        tt = torch.tensor([t_step], device=dev)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        t_step = float(tt.item())
    value = args.B * world / t_step

    # quality and work accounting from the last step
    iters = r.iters.cpu().numpy()
    evals = r.evals.cpu().numpy().astype(np.float64)
    loss = r.loss.cpu().numpy()
    flops = float((wl.flops_per_closure() * evals).sum())
    achieved_tflops = flops / t_step / 1e12
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
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": t_step * 1000.0, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": f"ragged batched L-BFGS: B={args.B} tapes, lengths U[3,64], 0..8 constants, "
                                       f"n_vars=2, N={args.N}, history 10, max_iter={MAX_ITER}, strong_wolfe, "
                                       "tol 1e-7, plain randn init",
                           "B": args.B, "N": args.N, "M": M_DEFAULT, "l2": "flushed (256 MiB write) between steps"},
                "roofline": {"bound": "fp32", "achieved": achieved_tflops, "peak": fp32_peak, "unit": "TFLOP/s",
                             "frac": achieved_tflops / fp32_peak, "traffic": None,
                             "peak_kind": f"nominal {sm_count} SMs x 128 FP32 lanes x 2 x sm_max_mhz ({pk_kind} clock)"},
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
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
