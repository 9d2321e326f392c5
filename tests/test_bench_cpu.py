"""bench.py's reference arm on the CPU: the JSON line the benchmark contract
asks for (one line on rank 0, nothing on the other ranks, exit status 0).
The arm times the oracle's restatement of the reference's CPU annealers on
the host cores, so it needs no GPU."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KEYS = {"metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better",
        "scaling", "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"}


def run_bench(*argv, rank=0):
    env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2" if rank else "1")
    p = subprocess.run([sys.executable, "bench.py", *argv], cwd=ROOT, env=env,
                       capture_output=True, text=True, timeout=600)
    assert p.returncode == 0, p.stderr[-2000:]
    return [ln for ln in p.stdout.splitlines() if ln.strip()]


def check_line(lines, unit):
    assert len(lines) == 1, lines
    d = json.loads(lines[0])
    assert KEYS <= set(d), KEYS - set(d)
    assert d["impl"] == "reference"
    assert d["unit"] == unit and d["value"] > 0
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in (
        "port", "reference", "reference_algorithm_port")
    assert d["e2e"] == {"value": d["value"], "unit": unit, "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert isinstance(d["config"], dict) and "workload" in d["config"]
    return d


def test_reference_arm_ensemble():
    """The reference arm anneals the GPU leg's own blocks (here a 2-structure
    ensemble) and states the same config dictionary the GPU leg states."""
    import argparse
    sys.path.insert(0, ROOT)
    import bench
    d = check_line(run_bench("--impl", "reference", "--steps", "2", "--warmup", "1",
                             "--structures", "2"), "moves/s")
    assert d["metric"] == "MC moves/s" and d["higher_is_better"] is True
    bench.set_workload(2, bench.ANNEAL["milestone_steps"])
    want = bench.ensemble_config(argparse.Namespace(resync=bench.RESYNC), 1)
    bench.set_workload(64, bench.ANNEAL["milestone_steps"])
    assert d["config"] == want
    assert d["config"]["regions"] == 48 and d["config"]["fp64_resync_every"] == 1000
    assert d["structures_per_s"] > 0 and d["steps"] == 2


def test_size_shares_keep_the_distribution():
    sys.path.insert(0, ROOT)
    import bench
    bench.set_workload(64, bench.ANNEAL["milestone_steps"])
    blocks = bench.ensemble_blocks(0)
    assert len(blocks) == 64 * 24
    parts = bench.size_shares(blocks, 8)
    assert sorted(b for p in parts for b in p) == sorted(blocks)
    means = [sum(n for n, _ in p) / len(p) for p in parts]
    assert max(means) / min(means) < 1.1


@pytest.mark.parametrize("workload,unit", [("targets", "arcs/s"), ("smooth", "moves/s"),
                                           ("heatmap", "moves/s"), ("plain", "moves/s"),
                                           ("stress", "iterations/s")])
def test_reference_arm_workloads(workload, unit):
    check_line(run_bench("--impl", "reference", "--workload", workload, "--cpu-budget", "1"),
               unit)


@pytest.mark.parametrize("workload", ["ensemble", "smooth", "heatmap", "targets"])
def test_reference_arm_other_ranks_print_nothing(workload):
    assert run_bench("--impl", "reference", "--workload", workload, "--steps", "1",
                     "--warmup", "0", rank=1) == []


def test_smooth_line_counts_window_class_launches(monkeypatch):
    """The genome-smoothing line claims one launch per window class it runs
    (regions with 20+ free beads at 32 slots, the rest at 8), with the
    library's calls replaced by fakes: the line's bookkeeping only."""
    import argparse
    import types

    sys.path.insert(0, ROOT)
    import bench
    from pmmc_gb300 import capi

    class FakeCtx:
        def __init__(self, device):
            pass

        def set_seed(self, seed):
            pass

    def fake_packed(ctx, off, pos, dtn, fixed, prm, steps, *a, **k):
        res = [types.SimpleNamespace(moves=10, rel_error=0.0) for _ in range(len(off) - 1)]
        return pos.copy(), res, 100.0

    class NoClocks:
        def __init__(self, device):
            pass

        def start(self):
            pass

        def stop(self):
            return {}

    monkeypatch.setattr(capi, "Context", FakeCtx)
    monkeypatch.setattr(capi, "smooth_batch_anneal_packed", fake_packed)
    monkeypatch.setattr(bench, "smooth_cpu_baseline", lambda sweeps, budget: {"value": 1.0})
    monkeypatch.setattr(bench, "ClockSampler", NoClocks)
    line = bench.smooth_record(argparse.Namespace(moves=0, steps=3, warmup=1, cpu_budget=0))
    assert line["gpu_launches"] == 2 * 3
    assert "kernel_launches_per_step" not in line
