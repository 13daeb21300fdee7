"""bench.py's contract on the host: no top-level name defined twice (a later
definition silently replaces an earlier one), and the reference arm of every
workload prints one JSON line with the keys the contract asks for."""
import ast
import collections
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "..")


def test_no_top_level_name_defined_twice():
    tree = ast.parse(open(os.path.join(ROOT, "bench.py")).read())
    names = [n.name for n in tree.body if isinstance(n, (ast.FunctionDef, ast.ClassDef))]
    dup = [k for k, v in collections.Counter(names).items() if v > 1]
    assert not dup, dup


@pytest.mark.parametrize("workload,extra", [("warmstart", ["--cpu-sample", "8"]), ("eval", ["--cpu-eval-sample", "64"]),
                                            ("sample", ["--cpu-sample-expr", "4096"])])
def test_reference_arm_prints_contract_line(workload, extra):
    cmd = [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--workload", workload,
           "--steps", "1", "--warmup", "1"] + extra
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "impl", "cpu_baseline",
                "e2e", "config"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_reference_arm_under_torchrun_prints_once():
    """Two ranks under torch.distributed.run: rank 0 alone runs the CPU port and prints
    the line, the other rank exits 0 without work."""
    import socket
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference",
           "--gpus", "2", "--workload", "sample", "--cpu-sample-expr", "4096", "--steps", "1", "--warmup", "1"]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0


def test_paired_statistics_charge_both_arms_alike():
    """The union median charges +inf to whichever arm leaves a problem non-finite; the
    plain-conditioned one would charge only the warm arm."""
    import numpy as np
    import bench
    inf = np.inf
    a = np.array([1.0, 2.0, 3.0, inf, 5.0, 0.5, 0.7])      # warm
    b = np.array([1.0, 2.5, inf, 4.0, inf, inf, 0.7])      # plain
    p = bench.paired_stats(a, b, np.isfinite(a), np.isfinite(b))
    assert p["finite_in_both"] == 3 and p["finite_only_warm"] == 3 and p["finite_only_plain"] == 1
    assert p["finite_in_either"] == 7
    assert p["warm_lower"] == 1 / 3 and p["warm_higher"] == 0 and p["same_within_1e-4"] == 2 / 3
    med = p["median_final_mse_either_finite"]
    assert med["warm"] == 2.0 and med["plain"] == 4.0
