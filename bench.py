"""Benchmark: batched arc-level annealing of an ensemble (64 structures x 24
anchor blocks, block sizes log-uniform 32..2048 beads, 1.5 arcs per bead),
the configuration the batched-vs-plain metric is quoted on.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

A step anneals every block of the ensemble once (T0 5, cooling 0.9999,
milestones every 50k moves with improvement threshold 0.99 -- the reference
CPU schedule of MonteCarloArcs -- and an FP64 energy recompute every 1000
moves, --resync) in one CUDA-graph launch of the persistent work-stealing
kernels.  Inputs are seeded synthetic regions (no datasets ship with the
reference).  Rank r of N anneals its own ensemble (seeds 64r..64r+63): weak
scaling, no collective.

One JSON line on rank 0: value = MC moves/s over all ranks (device time,
CUDA events on the launching stream); structures/s beside it; e2e = the same
metric through the host-buffer C-ABI call (staging, copies and result reads
inside the timed region), the max over ranks; roofline of the annealing
kernel against the measured HBM peak, its per-move shared-memory/FP32 basis
and the latency bound of the critical chain; cpu_baseline = the reference's
CPU annealer (the oracle's bit-identical restatement) on one equal part of
the same ensemble on all host cores.  At N = 1 the line also carries a
sub-record per other configuration ("configs": plain, heatmap, heatmap
batch, smoothing, serving), each with its CPU baseline timed on this host.

--impl reference anneals the same ensemble's blocks with the reference's CPU
annealer on all host cores (warm-up and timed parts of equal size
distribution) and prints the same config.

Other lines (--workload): plain, heatmap, heatmap-batch, smooth, serve,
distmap, equidistant, targets, stress (pmmc_gb300/workloads.py describes
each); every line carries its CPU baseline, and --impl reference prints the
reference arm of the chosen line.
"""
from __future__ import annotations

import argparse
import json
import math
import multiprocessing as mp
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

N_STRUCT, N_BLOCKS = 64, 24
ANNEAL = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=50000, improvement=0.99)
RESYNC = 1000
STEP = 0.5
WORKLOAD = (f"arcs_ensemble_{N_STRUCT}x{N_BLOCKS}_blocks32-2048_1.5arcs_per_bead_"
            f"T0=5_cool0.9999_milestone50k_thr0.99")


def set_workload(structures: int, milestone: int) -> None:
    global N_STRUCT, WORKLOAD
    N_STRUCT = structures
    ANNEAL["milestone_steps"] = milestone
    WORKLOAD = (f"arcs_ensemble_{N_STRUCT}x{N_BLOCKS}_blocks32-2048_1.5arcs_per_bead_"
                f"T0=5_cool0.9999_milestone{milestone // 1000}k_thr0.99")


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# --------------------------------------------------------------------------
# CPU leg (the oracle restates MonteCarloArcs bit for bit; see oracle/)
# --------------------------------------------------------------------------
def _cpu_block(args):
    n, seed = args
    from oracle import oracle as O
    from pmmc_gb300 import synth
    r = synth.arcs_region(n, arcs_per_bead=1.5, seed=seed)
    pr = O.ArcsProblem(r.pos, r.dense())
    t = time.perf_counter()
    _, res = O.arcs_anneal(pr, O.Params(**ANNEAL), STEP, seed)
    return res.moves, time.perf_counter() - t, n


def ensemble_blocks(rank: int = 0, world: int = 1):
    """(beads, region seed) of every block of a rank's ensemble, the regions
    the GPU leg anneals (synth.ensemble_block_specs)."""
    from pmmc_gb300 import synth
    from pmmc_gb300.replicas import shard_seeds
    seeds = shard_seeds(rank, max(world, rank + 1), N_STRUCT)
    return [b for st in synth.ensemble_block_specs(N_STRUCT, N_BLOCKS, seeds=seeds) for b in st]


def size_shares(blocks, shares: int):
    """The blocks split into `shares` parts of the same size distribution:
    block of size rank i (largest first) goes to part i mod shares."""
    order = sorted(range(len(blocks)), key=lambda k: (-blocks[k][0], k))
    parts = [[] for _ in range(shares)]
    for i, k in enumerate(order):
        parts[i % shares].append(blocks[k])
    return parts


def cpu_anneal_blocks(pool, blocks):
    """The reference CPU annealer (MonteCarloArcs, restated by the oracle
    bit for bit, libc stream seeded by the region seed) over `blocks` on the
    pool's processes, largest block first.  Returns moves, wall s, CPU s."""
    jobs = sorted(blocks, key=lambda b: -b[0])
    t0 = time.perf_counter()
    moves = cpu_s = 0.0
    for mv, dt, _ in pool.imap_unordered(_cpu_block, jobs):
        moves += mv
        cpu_s += dt
    return moves, time.perf_counter() - t0, cpu_s


def cpu_ensemble_sample(share: int = 8):
    """CPU baseline of the default line, bounded: one of `share` equal parts
    of the ensemble's own blocks (same size distribution) annealed on every
    host core at once."""
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    part = size_shares(ensemble_blocks(0), share)[0]
    with mp.get_context("spawn").Pool(cores) as pool:
        pool.map(_cpu_block, [(32, 7 + k) for k in range(cores)])  # start-up, imports
        moves, wall, cpu_s = cpu_anneal_blocks(pool, part)
    return {"moves": moves, "wall_s": wall, "cpu_s": cpu_s, "blocks": len(part),
            "cores": cores, "moves_per_s": moves / wall, "share": share}


def _cpu_request(args):
    k, n = args
    from oracle import oracle as O
    from pmmc_gb300 import workloads as W
    r = W.serve_region(k, n)
    pr = O.ArcsProblem(r.pos, r.dense())
    t = time.perf_counter()
    prm = {k_: v for k_, v in W.SERVE_ANNEAL.items() if k_ != "resync_every"}
    _, res = O.arcs_anneal(pr, O.Params(**prm), W.SERVE_STEP, W.serve_seed(k))
    return k, n, res.moves, time.perf_counter() - t


def cpu_serve_baseline(n_req: int, budget_s: float = 20.0):
    """The reference CPU annealer (oracle port) behind the same trace: a
    bounded sample of the trace's requests is annealed on every host core,
    service time is fitted as a + b*n over the sample, and a FIFO queue with
    one server per core replays the whole trace (arrivals, sizes) with those
    service times.  Returns latency percentiles and capacity."""
    import heapq
    from oracle import oracle as O
    from pmmc_gb300 import workloads as W
    O.build()
    cores = os.cpu_count() or 1
    sizes, arrivals = W.serve_trace(n_req)
    rng = np.random.default_rng(5)
    idx = rng.permutation(n_req)[:max(4 * cores, 32)]
    jobs = [(int(k), int(sizes[k])) for k in idx]
    ctx = mp.get_context("spawn")
    t0 = time.perf_counter()
    samp = []
    with ctx.Pool(cores) as pool:
        for out in pool.imap_unordered(_cpu_request, jobs):
            samp.append(out)
            if time.perf_counter() - t0 > budget_s and len(samp) >= 8:
                pool.terminate()
                break
    ns = np.array([x[1] for x in samp], float)
    ts = np.array([x[3] for x in samp], float)
    mv = np.array([x[2] for x in samp], float)
    b, a = np.polyfit(ns, ts, 1) if len(set(ns)) > 1 else (0.0, float(ts.mean()))
    service = np.maximum(a + b * sizes, 1e-4)
    free = [0.0] * cores
    heapq.heapify(free)
    lat = np.empty(n_req)
    for k in range(n_req):
        f = heapq.heappop(free)
        start = max(f, arrivals[k])
        done = start + service[k]
        heapq.heappush(free, done)
        lat[k] = (done - arrivals[k]) * 1e3
    return {"value": cores / float(service.mean()), "unit": "structures/s", "cores": cores,
            "kind": "port",
            "sample": f"{len(samp)} of the trace's requests annealed by the oracle port on "
                      f"{cores} cores ({float(ts.sum()):.1f} CPU s), service time fitted "
                      f"a + b*n, FIFO queue of {cores} servers replayed over the trace",
            "moves_per_s_per_core": float(mv.sum() / ts.sum()),
            "latency_ms_p50_at_200rps": float(np.percentile(lat, 50)),
            "latency_ms_p99_at_200rps": float(np.percentile(lat, 99))}


def _cpu_plain(seed):
    from oracle import oracle as O
    from pmmc_gb300 import workloads as W
    r = W.plain_region()
    pr = O.ArcsProblem(r.pos, r.dense())
    t = time.perf_counter()
    _, res = O.arcs_anneal(pr, O.Params(**W.PLAIN_ANNEAL), 0.5, seed)
    return res.moves, time.perf_counter() - t


def distmap_main(args):
    """Expected-distance map line beside the reference's host transform (the
    oracle port, bit-identical to it) on one core, timed on a 4096 x 4096
    sample and scaled per entry."""
    from oracle import oracle as O
    from pmmc_gb300 import workloads as W
    O.build()
    cs = W.distmap_contact(4096, seed=6)
    t = time.perf_counter()
    O.distance_heatmap(cs, 1, 100.0, -0.333, 2.0)
    dt = time.perf_counter() - t
    cpu = {"value": cs.size / dt, "unit": "entries/s", "cores": 1, "kind": "port",
           "sample": f"one 4096 x 4096 map ({dt:.2f} s)"}
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        print(json.dumps({"metric": "matrix entries/s", "value": cpu["value"],
                          "unit": "entries/s", "n_gpus": 0, "steps": 1, "warmup": 0,
                          "ms_per_step": dt * 1e3, "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                          "data": "synthetic", "impl": "reference",
                          "config": {"workload": "distance_heatmap"}, "cpu_baseline": cpu,
                          "e2e": {"value": cpu["value"], "unit": "entries/s",
                                  "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    sampler = ClockSampler(0)
    sampler.start()
    line = W.distmap(args)
    line["clocks"] = sampler.stop()
    line["gpu_launches"] = 3 * args.steps
    line["cpu_baseline"] = cpu
    print(json.dumps(line))


def equidistant_main(args):
    """Equidistant-model line beside the reference's CPU interpolation (the
    oracle port, bit-identical to it: a linear scan of the level per point)
    on one core, timed on 20000 points from the middle of the chromosome
    (the scan's average length) and scaled per point."""
    from oracle import oracle as O
    from pmmc_gb300 import workloads as W
    O.build()
    gpos, start, end, pos = W.equidistant_level()
    res = args.n or 100
    mid = int(gpos[len(gpos) // 2])
    stop = mid + res * 20_000 - 1
    t = time.perf_counter()
    pts = O.equidistant(gpos, pos, int(end[0]), int(start[-1]), mid, stop, res)
    dt = time.perf_counter() - t
    cpu = {"value": len(pts) / dt, "unit": "points/s", "cores": 1, "kind": "port",
           "sample": f"{len(pts)} points from mid-chromosome ({dt:.2f} s)"}
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        print(json.dumps({"metric": "points/s", "value": cpu["value"], "unit": "points/s",
                          "n_gpus": 0, "steps": 1, "warmup": 0, "ms_per_step": dt * 1e3,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                          "dtype": "f32", "data": "synthetic", "impl": "reference",
                          "config": {"workload": "equidistant"}, "cpu_baseline": cpu,
                          "e2e": {"value": cpu["value"], "unit": "points/s",
                                  "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    sampler = ClockSampler(0)
    sampler.start()
    line = W.equidistant(args)
    line["clocks"] = sampler.stop()
    line["gpu_launches"] = args.steps
    line["cpu_baseline"] = cpu
    print(json.dumps(line))


def targets_main(args):
    """Anchor-level expected-distance line beside the reference's host
    builder (the oracle port, bit-identical to it: a linear anchor scan per
    long-arc end) on one core, timed on the same chromosome with a quarter
    of the long arcs and scaled per arc."""
    from oracle import oracle as O
    from pmmc_gb300 import workloads as W
    O.build()
    n_long = args.n or 2_000_000
    sample = W.targets_problem(n_long // 4)
    units = len(sample["arc_start"]) + n_long // 4
    t = time.perf_counter()
    O.anchor_targets(sample)
    dt = time.perf_counter() - t
    cpu = {"value": units / dt, "unit": "arcs/s", "cores": 1, "kind": "port",
           "sample": f"{W.TARGETS_ANCHORS} anchors, {len(sample['arc_start'])} arcs and "
                     f"{n_long // 4} long arcs ({dt:.2f} s)"}
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        print(json.dumps({"metric": "arcs/s", "value": cpu["value"], "unit": "arcs/s",
                          "n_gpus": 0, "steps": 1, "warmup": 0, "ms_per_step": dt * 1e3,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                          "dtype": "int32", "data": "synthetic", "impl": "reference",
                          "config": {"workload": "anchor_targets"}, "cpu_baseline": cpu,
                          "e2e": {"value": cpu["value"], "unit": "arcs/s",
                                  "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    sampler = ClockSampler(0)
    sampler.start()
    line = W.targets(args)
    line["clocks"] = sampler.stop()
    # own kernels per call: long_map, long_resolve, pair_emit, csr_finish (the
    # two radix sorts are the CUDA toolkit's CUB)
    line["gpu_launches"] = 4 * args.steps
    line["cpu_baseline"] = cpu
    print(json.dumps(line))


def stress_main(args):
    """Stress-refinement line beside the reference's host descent (the oracle
    port, bit-identical to it) on one core, timed over the first 100
    iterations of the same chromosome (pair building included, as in the
    reference) and scaled per iteration."""
    from oracle import oracle as O
    from pmmc_gb300 import workloads as W
    O.build()
    t = W.stress_problem()
    t0 = time.perf_counter()
    _, _, out = O.stress_refine(t, 100, W.STRESS_LR)
    dt = time.perf_counter() - t0
    cpu = {"value": out["iterations"] / dt, "unit": "iterations/s", "cores": 1, "kind": "port",
           "sample": f"{out['iterations']} iterations of {W.STRESS_ANCHORS} anchors, "
                     f"{out['n_pairs']} pairs ({dt:.2f} s)"}
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        print(json.dumps({"metric": "iterations/s", "value": cpu["value"],
                          "unit": "iterations/s", "n_gpus": 0, "steps": 1, "warmup": 0,
                          "ms_per_step": dt * 1e3, "higher_is_better": True,
                          "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                          "data": "synthetic", "impl": "reference",
                          "config": {"workload": "stress_refine"}, "cpu_baseline": cpu,
                          "e2e": {"value": cpu["value"], "unit": "iterations/s",
                                  "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    sampler = ClockSampler(0)
    sampler.start()
    line = W.stress(args)
    line["clocks"] = sampler.stop()
    line["gpu_launches"] = args.steps
    line["cpu_baseline"] = cpu
    print(json.dumps(line))


def _cpu_heatmap(job):
    scale, cap, incremental = job
    from oracle import oracle as O
    from pmmc_gb300 import workloads as W
    base, _ = W.heatmap_maps(1)
    heat = base.heat if scale == 1.0 else (base.heat * np.float32(scale)).astype(np.float32)
    pr = O.HeatmapProblem(base.pos, heat, base.diag, base.bounds)
    prm = O.Params(**W.HEATMAP_ANNEAL, max_moves=cap)
    t = time.perf_counter()
    _, res = O.heatmap_anneal(pr, prm, 1.0, 7, incremental=incremental)
    return res.moves, time.perf_counter() - t


def _cpu_pool(fn, jobs, cores):
    """Runs one job per core at once; returns the moves, the sum of the jobs'
    own rates (moves / own time, process start-up excluded) and the wall
    time."""
    t0 = time.perf_counter()
    if cores == 1:
        res = [fn(j) for j in jobs]
    else:
        with mp.get_context("spawn").Pool(cores) as pool:
            res = pool.map(fn, jobs)
    return (sum(r[0] for r in res), sum(r[0] / r[1] for r in res),
            time.perf_counter() - t0)


def heatmap_cpu_baseline(n_maps: int, budget_s: float) -> dict:
    """The reference's heatmap annealer on the host (MonteCarloHeatmap,
    restated by the oracle bit for bit), one map per core (one core for the
    single-chain line).  Its own form re-scores the whole 2048-bead map after
    every move (O(N^2) per move); the baseline reported is an O(N)-incremental
    form of the same annealer (local scores of the moved bead), the faster
    CPU code, with the reference's own form beside it."""
    from oracle import oracle as O
    from pmmc_gb300 import workloads as W
    O.build()
    cores = 1 if n_maps == 1 else max(1, min(os.cpu_count() or 1, n_maps))
    _, scales = W.heatmap_maps(max(n_maps, cores))
    mv, dt = _cpu_heatmap((1.0, 2000, True))
    cap = int(min(100_000, max(2000, mv / dt * budget_s / 2)))
    _, rate, wall = _cpu_pool(_cpu_heatmap, [(float(scales[k]), cap, True)
                                             for k in range(cores)], cores)
    full_cap = 20
    _, frate, fwall = _cpu_pool(_cpu_heatmap, [(float(scales[k]), full_cap, False)
                                               for k in range(cores)], cores)
    return {"value": rate, "unit": "moves/s", "cores": cores, "kind": "port",
            "sample": f"{cores} map(s) x {cap} moves at once, O(N) local scores per move "
                      f"({wall:.1f} s)",
            "reference_form": {"value": frate, "unit": "moves/s", "cores": cores,
                               "sample": f"{cores} map(s) x {full_cap} moves at once, "
                                         f"re-scoring the whole map per move ({fwall:.1f} s)"}}


def heatmap_record(args, n_maps: int) -> dict:
    """Heatmap-level line (one chain, or one chain per distinct map) with the
    reference's heatmap annealer on the host cores beside it: its own form
    (a full re-score per move) timed on a capped number of moves and
    extrapolated to the line's moves, and the O(N)-incremental form."""
    # CPU baseline first, so that its process pool starts before the first
    # GPU call; the batch's default (two maps per SM) exceeds the host cores
    cpu = heatmap_cpu_baseline(n_maps if n_maps > 0 else 2 * (os.cpu_count() or 1),
                               args.cpu_budget)
    from pmmc_gb300 import workloads as W
    sampler = ClockSampler(0)
    sampler.start()
    line = W.heatmap(args, n_maps)
    line["clocks"] = sampler.stop()
    line["gpu_launches"] = args.steps  # one heatmap_anneal_kernel launch per call
    moves = line["config"]["moves_per_step"] / line["config"]["maps"]
    ref = cpu["reference_form"]
    ref["extrapolated_s_per_chain"] = moves / (ref["value"] / ref["cores"])
    line["cpu_baseline"] = cpu
    return line


def heatmap_main(args, n_maps: int):
    """Heatmap-level line beside the reference's heatmap annealer."""
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        maps = n_maps if n_maps > 0 else 2 * (os.cpu_count() or 1)
        cpu = heatmap_cpu_baseline(maps, args.cpu_budget)
        ref = dict(cpu["reference_form"], kind="reference_algorithm_port")
        print(json.dumps({"metric": "MC moves/s", "value": ref["value"], "unit": "moves/s",
                          "n_gpus": 0, "steps": 1, "warmup": 0, "ms_per_step": None,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                          "dtype": "f64", "data": "synthetic", "impl": "reference",
                          "config": {"workload": f"heatmap_{maps}x2048"},
                          "cpu_baseline": ref, "incremental_port": cpu,
                          "e2e": {"value": ref["value"], "unit": "moves/s",
                                  "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    print(json.dumps(heatmap_record(args, n_maps)))


def _cpu_smooth(job):
    segs, sweeps = job
    from oracle import oracle as O
    from pmmc_gb300 import workloads as W
    moves = 0
    t = time.perf_counter()
    for pos, dtn, fixed in segs:
        free = int((fixed == 0).sum())
        prm = O.Params(**W.SMOOTH_ANNEAL, k_stretch=0.1, k_squeeze=0.1,
                       max_moves=sweeps * free)
        _, res = O.smooth_anneal(O.SmoothProblem(pos, dtn, fixed), prm, 0.5, 3)
        moves += res.moves
    return moves, time.perf_counter() - t


def smooth_cpu_baseline(sweeps: int, budget_s: float) -> dict:
    """The reference's smoothing annealer (MonteCarloArcsSmooth, restated by
    the oracle bit for bit) over the workload's regions on every host core,
    each region for the same sweeps as the GPU line; a seeded random subset
    of the regions, as many as about budget_s of wall time covers."""
    from oracle import oracle as O
    from pmmc_gb300 import workloads as W
    O.build()
    segs = W.smooth_segments()
    order = np.random.default_rng(5).permutation(len(segs))
    chunks = [([segs[i] for i in order[k:k + 32]], sweeps) for k in range(0, len(segs), 32)]
    cores = os.cpu_count() or 1
    moves, cpu_s, done = 0, 0.0, 0
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(cores) as pool:
        for mv, dt in pool.imap_unordered(_cpu_smooth, chunks):
            moves += mv
            cpu_s += dt
            done += 1
            if time.perf_counter() - t0 > budget_s:
                pool.terminate()
                break
    wall = time.perf_counter() - t0
    # every core ran chunks at once: the mean rate of a core times the cores
    return {"value": moves / cpu_s * cores, "unit": "moves/s", "cores": cores, "kind": "port",
            "sample": f"{done * 32} of {len(segs)} regions x {sweeps} sweeps "
                      f"({cpu_s:.1f} CPU s in {wall:.1f} s)"}


def smooth_record(args) -> dict:
    """Genome-smoothing line with the reference's smoothing annealer on every
    host core beside it."""
    sweeps = args.moves or 20_000
    cpu = smooth_cpu_baseline(sweeps, args.cpu_budget)
    from pmmc_gb300 import workloads as W
    sampler = ClockSampler(0)
    sampler.start()
    line = W.smooth(args)
    line["clocks"] = sampler.stop()
    # the window classes' smooth_window_kernel launches, side by side
    line["gpu_launches"] = args.steps * line.pop("kernel_launches_per_step")
    line["cpu_baseline"] = cpu
    return line


def smooth_main(args):
    """Genome-smoothing line beside the reference's smoothing annealer on
    every host core."""
    sweeps = args.moves or 20_000
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        cpu = smooth_cpu_baseline(sweeps, args.cpu_budget)
        print(json.dumps({"metric": "MC moves/s", "value": cpu["value"], "unit": "moves/s",
                          "n_gpus": 0, "steps": 1, "warmup": 0, "ms_per_step": None,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                          "dtype": "f64", "data": "synthetic", "impl": "reference",
                          "config": {"workload": f"genome_smoothing_{sweeps}sweeps"},
                          "cpu_baseline": cpu,
                          "e2e": {"value": cpu["value"], "unit": "moves/s",
                                  "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}))
        return
    print(json.dumps(smooth_record(args)))


def _cpu_plain_pool(cores: int):
    """Independent anneals of the config-0 region, one per core at once:
    (completed anneals, wall s)."""
    t = time.perf_counter()
    with mp.get_context("spawn").Pool(cores) as pool:
        pool.map(_cpu_plain, range(42, 42 + cores))
    return cores, time.perf_counter() - t


def plain_record(args) -> dict:
    """Config-0 line: the plain drop-in call with the reference CPU annealer
    (the oracle port, bit-identical to it) beside it: one core for one
    structure, every core for structures/s."""
    from oracle import oracle as O
    from pmmc_gb300 import workloads as W
    O.build()
    mv, dt = _cpu_plain(42)
    cores = os.cpu_count() or 1
    done, wall = _cpu_plain_pool(cores)
    sampler = ClockSampler(0)
    sampler.start()
    line = W.plain(args)
    line["clocks"] = sampler.stop()
    line["gpu_launches"] = args.steps * 2
    line["structures_per_s"] = 1e3 / line["ms_per_step"]
    line["cpu_baseline"] = {"value": mv / dt, "unit": "moves/s", "cores": 1, "kind": "port",
                            "sample": f"one full anneal of the region ({mv} moves, {dt:.2f} s)",
                            "structures_per_s_all_cores": done / wall,
                            "all_cores": f"{done} anneals (seeds 42..) on {cores} cores at "
                                         f"once, {wall:.1f} s wall"}
    return line


def plain_main(args):
    """Config-0 line: the plain drop-in call beside the reference CPU
    annealer (the oracle port, bit-identical to it) on one core."""
    from oracle import oracle as O
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        O.build()
        mv, dt = _cpu_plain(42)
        v = mv / dt
        print(json.dumps({"metric": "MC moves/s", "value": v, "unit": "moves/s", "n_gpus": 0,
                          "steps": 1, "warmup": 0, "ms_per_step": dt * 1e3,
                          "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                          "dtype": "f64", "data": "synthetic", "impl": "reference",
                          "config": {"workload": "arcs_plain_256beads_400arcs_seed42"},
                          "cpu_baseline": {"value": v, "unit": "moves/s", "cores": 1,
                                           "kind": "port", "sample": "one full anneal"},
                          "e2e": {"value": v, "unit": "moves/s", "h2d_bytes_per_step": 0,
                                  "d2h_bytes_per_step": 0}}))
        return
    print(json.dumps(plain_record(args)))


def serve_record(args) -> dict:
    """Serving line with the same trace through a host-core queue beside it."""
    from pmmc_gb300 import workloads as W
    n_req = args.requests or 5000
    cpu = cpu_serve_baseline(n_req, args.cpu_budget)
    sampler = ClockSampler(0)
    sampler.start()
    line = W.serve(args)
    line["clocks"] = sampler.stop()
    line["gpu_launches"] = line["saturated"]["waves"]
    line["cpu_baseline"] = cpu
    return line


def serve_main(args):
    from pmmc_gb300 import workloads as W
    n_req = args.requests or 5000
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        cb = cpu_serve_baseline(n_req, args.cpu_budget)
        line = {"metric": "structures/s", "value": cb["value"], "unit": "structures/s",
                "n_gpus": 0, "steps": 1, "warmup": 0, "ms_per_step": None,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f64", "data": "synthetic", "impl": "reference",
                "config": {"workload": "serve", "requests": n_req},
                "cpu_baseline": cb,
                "e2e": {"value": cb["value"], "unit": "structures/s",
                        "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return
    print(json.dumps(serve_record(args)))


# --------------------------------------------------------------------------
# GPU helpers
# --------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi clocks and throttle reasons while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def traffic_per_launch():
    """DRAM bytes of one annealing launch from the committed ncu summary
    (profiles/traffic_per_launch.txt: '<kernel> <workload> <bytes>')."""
    p = os.path.join(ROOT, "profiles", "traffic_per_launch.txt")
    if not os.path.exists(p):
        return None
    for line in open(p):
        f = line.split()
        if len(f) >= 3 and f[0] == "arcs_anneal_kernel" and f[1] == "config2":
            return float(f[2])
    return None


def make_inputs(rank: int, world: int = 1):
    from pmmc_gb300 import capi, synth
    from pmmc_gb300.replicas import shard_seeds
    ens = synth.arcs_ensemble(N_STRUCT, N_BLOCKS, seeds=shard_seeds(rank, max(world, rank + 1),
                                                                    N_STRUCT))
    regs = [r for s in ens for r in s]
    inputs = [capi.ArcsInput(r.pos, *r.csr()) for r in regs]
    return regs, inputs


def staged_bytes(inputs):
    """Host->device bytes of one staging of the batch (positions as float4,
    row pointers, arc entries {col,target} + reciprocal) and device->host
    bytes of the results (xyz positions + one result record per block)."""
    h2d = d2h = 0
    for x in inputs:
        nnz = int(x.row_ptr[-1])
        h2d += 16 * x.n + 4 * (x.n + 1) + 12 * nnz + 80
        d2h += 12 * x.n + 56
    return h2d, d2h


def flush_l2(buf):
    buf.fill_(1)


def run_gpu(args, rank, world):
    import torch

    from pmmc_gb300 import build, capi
    build.build()
    torch.cuda.set_device(0 if world == 1 else int(os.environ.get("LOCAL_RANK", rank)))
    dev = torch.cuda.current_device()
    ctx = capi.Context(dev)
    ctx.set_seed(2024 + rank)
    regs, inputs = make_inputs(rank, world)
    prm = capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_CPU,
                              resync_every=args.resync, **ANNEAL)
    steps = [STEP] * len(inputs)
    batch = capi.ArcsBatch(ctx, inputs, prm, steps, chains=1, use_graph=True, lanes=args.lanes,
                           drawing_warp=args.drawing_warp)
    classes = batch.classes()
    stream = torch.cuda.Stream()
    l2 = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    # warm-up (graph capture happens on the first run)
    for _ in range(args.warmup):
        batch.run(stream.cuda_stream)
        batch.results()
    # moves and launches of a pass (from the first timed pass when there is
    # no warm-up)
    moves_per_step, n_launch = batch.stats()[1:] if args.warmup > 0 else (None, None)
    # ---- timed region ----
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clocks = ClockSampler(dev)
    clocks.start()
    kernel_ms = []
    t_wall = time.perf_counter()
    for _ in range(args.steps):
        with torch.cuda.stream(stream):
            flush_l2(l2)
        batch.run(stream.cuda_stream)
        ms, mv, nl = batch.stats()
        if moves_per_step is None:
            moves_per_step, n_launch = mv, nl
        assert mv == moves_per_step
        kernel_ms.append(ms)
    torch.cuda.synchronize()
    t_wall = time.perf_counter() - t_wall
    clk = clocks.stop()
    if world > 1:
        torch.distributed.barrier()
    pos, res = batch.results()
    step_ms = sum(kernel_ms) / len(kernel_ms)
    rel_err = max(r.rel_error for r in res)
    status_bad = sum(1 for r in res if r.status not in (0,))
    # ---- e2e through the host-buffer call ----
    e2e_ms = []
    r2 = []
    for k in range(args.e2e_steps):
        torch.cuda.synchronize()
        t = time.perf_counter()
        p2, r2 = _batch_anneal_host(ctx, inputs, prm, steps, args.lanes, args.drawing_warp)
        e2e_ms.append((time.perf_counter() - t) * 1e3)
    e2e_moves = sum(r.moves for r in r2)
    h2d, d2h = staged_bytes(inputs)
    # ---- plain drop-in form: one structure, blocks annealed one call each ----
    plain_s = None
    if rank == 0 and args.plain:
        t = time.perf_counter()
        for x in inputs[:N_BLOCKS]:
            capi.arcs_anneal(ctx, x, prm, STEP, 1)
        plain_s = time.perf_counter() - t
    batch.close()
    # ---- latency bound: the chain with the most moves, its region alone on
    # the device (same launch choice), time per move x its moves in the pass
    crit = max(range(len(res)), key=lambda u: res[u].moves)
    alone = capi.ArcsBatch(ctx, [inputs[crit]], prm, [STEP], chains=1, use_graph=False,
                           lanes=args.lanes, drawing_warp=args.drawing_warp)
    per_move = []
    for _ in range(3):
        alone.run()
        a_ms, a_moves, _ = alone.stats()
        per_move.append(a_ms / max(a_moves, 1))
    alone.close()
    crit_ms = min(per_move) * res[crit].moves
    return dict(step_ms=step_ms, moves=moves_per_step, kernel_ms=kernel_ms, wall=t_wall,
                clocks=clk, rel_err=rel_err, bad=status_bad, e2e_ms=e2e_ms,
                e2e_moves=e2e_moves, h2d=h2d, d2h=d2h, plain_s=plain_s, n_launch=n_launch,
                n_units=len(inputs), classes=classes,
                crit={"region_beads": int(inputs[crit].n), "moves": int(res[crit].moves),
                      "ms_per_move_alone": min(per_move), "bound_ms": crit_ms})


def _batch_anneal_host(ctx, inputs, prm, steps, lanes=0, drawing_warp=False):
    import ctypes as C

    from pmmc_gb300 import capi
    arr = (capi.ArcsProblem * len(inputs))(*[x.struct() for x in inputs])
    st = np.ascontiguousarray(steps, dtype=np.float32)
    tot = sum(x.n for x in inputs)
    pos = np.zeros((tot, 3), np.float32)
    res = (capi.Result * len(inputs))()
    opts = capi.BatchOpts(1, 0, int(lanes), int(bool(drawing_warp)))
    ctx.check(capi.lib().pmmc_arcs_batch_anneal(ctx.h, len(inputs), arr, C.byref(prm),
                                                st.ctypes.data_as(C.c_void_p), C.byref(opts),
                                                pos.ctypes.data_as(C.c_void_p), res))
    return pos, list(res)


def algorithmic_bytes(inputs, moves):
    """HBM bytes one launch must move: each region's positions (float4),
    row pointers and arc entries (12 B) read once, positions (12 B/bead) and
    one result record written once."""
    b = 0
    for x in inputs:
        nnz = int(x.row_ptr[-1])
        b += 16 * x.n + 4 * (x.n + 1) + 12 * nnz + 12 * x.n + 56
    return b


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--drawing-warp", action="store_true",
                    help="with fixed --lanes 1 or 2: a second warp per chain draws the moves")
    ap.add_argument("--resync", type=int, default=RESYNC,
                    help="FP64 energy recompute every this many moves of a chain")
    ap.add_argument("--no-plain", dest="plain", action="store_false")
    ap.add_argument("--cpu-budget", type=float, default=20.0,
                    help="seconds of CPU-baseline work per line (0: none)")
    ap.add_argument("--cpu-share", type=int, default=8,
                    help="default line's CPU baseline: 1 of this many equal parts of the "
                         "ensemble's blocks")
    ap.add_argument("--no-configs", dest="configs", action="store_false",
                    help="default line without the sub-records of the other configurations")
    ap.add_argument("--structures", type=int, default=N_STRUCT,
                    help="ensemble size (smaller for profiling runs)")
    ap.add_argument("--milestone", type=int, default=ANNEAL["milestone_steps"],
                    help="milestone interval (smaller for profiling runs)")
    ap.add_argument("--workload", default="ensemble",
                    choices=["ensemble", "plain", "heatmap", "heatmap-batch", "smooth",
                             "serve", "distmap", "equidistant", "targets", "stress"],
                    help="ensemble: the batched arc-level ensemble (default line); "
                         "heatmap: one 2048-bead heatmap chain; heatmap-batch: one chain "
                         "per distinct 2048-bead map, one per SM; smooth: genome-scale "
                         "subanchor smoothing; serve: the request loop on a Poisson trace")
    ap.add_argument("--maps", type=int, default=0, help="heatmap-batch: number of maps")
    ap.add_argument("--moves", type=int, default=0,
                    help="moves per chain (heatmap/smooth); stress: maximum iterations")
    ap.add_argument("--requests", type=int, default=0, help="serve: requests in the trace")
    ap.add_argument("--n", type=int, default=0,
                    help="distmap: matrix size; equidistant: resolution; targets: long arcs")
    ap.add_argument("--lanes", type=int, default=-1,
                    help="lanes per proposal of the batched form (2, 4, 8, 32; -1 = autotune)")
    args = ap.parse_args()
    set_workload(args.structures, args.milestone)
    if args.workload == "serve":
        serve_main(args)
        return
    if args.workload == "plain":
        plain_main(args)
        return
    if args.workload == "distmap":
        distmap_main(args)
        return
    if args.workload == "equidistant":
        equidistant_main(args)
        return
    if args.workload == "targets":
        targets_main(args)
        return
    if args.workload == "stress":
        stress_main(args)
        return
    if args.workload == "heatmap":
        heatmap_main(args, 1)
        return
    if args.workload == "heatmap-batch":
        heatmap_main(args, args.maps or 0)
        return
    if args.workload == "smooth":
        smooth_main(args)
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    config = ensemble_config(args, world)

    if args.impl == "reference":
        # the reference's own CPU annealer (the oracle's bit-identical
        # restatement; the reference sources do not travel to the GPU host)
        # on all host cores, over the GPU leg's own blocks
        if rank != 0:
            return
        reference_main(args, config)
        return

    # CPU baseline first (spawn pool, before any CUDA call in this process)
    cpu = (cpu_ensemble_sample(args.cpu_share)
           if rank == 0 and args.cpu_budget > 0 else None)
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", rank)))
        dist.init_process_group("nccl")
    r = run_gpu(args, rank, world)
    # max over ranks (replicas: the only cross-rank step), for the device
    # time and for the end-to-end time alike
    from pmmc_gb300.replicas import combine
    dev = "cuda" if world > 1 else None
    step_ms, total_moves = combine(r["step_ms"], float(r["moves"]), device=dev)
    e2e_ms_local = min(r["e2e_ms"]) if r["e2e_ms"] else 0.0
    e2e_ms, e2e_moves = combine(e2e_ms_local, float(r["e2e_moves"]), device=dev)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    if rank != 0:
        return
    value = total_moves / (step_ms * 1e-3)
    structs = world * N_STRUCT / (step_ms * 1e-3)
    e2e_val = e2e_moves / (e2e_ms * 1e-3) if e2e_ms > 0 else None
    peak, peak_kind = measured_peaks()
    _, inputs = make_inputs(0)
    alg = algorithmic_bytes(inputs, r["moves"])
    achieved = alg / (r["step_ms"] * 1e-3) / 1e9
    traffic = traffic_per_launch()
    from pmmc_gb300 import workloads as W
    deg = sum(int(x.row_ptr[-1]) for x in inputs) / sum(x.n for x in inputs)
    sm_mhz = r["clocks"].get("sm_mhz") or 2070.0
    line = {
        "metric": "MC moves/s", "value": value, "unit": "moves/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": config,
        "moves_per_step": total_moves,
        "launch": {"launch_classes": [{"lanes": la, "chains_per_cta": w, "items": it,
                                       "arcs_in_smem": nb, "drawing_warp": dw}
                                      for la, w, it, nb, dw in r["classes"]],
                   "tuning": "autotuned" if args.lanes == -1 else f"lanes={args.lanes}"},
        "structures_per_s": structs,
        "final_energy_rel_error_max": r["rel_err"],
        "chains_not_ok": r["bad"],
        "e2e": {"value": e2e_val, "unit": "moves/s", "h2d_bytes_per_step": r["h2d"],
                "d2h_bytes_per_step": r["d2h"], "ms_per_step": e2e_ms},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "peak_source": peak_kind,
                     "note": "serial Metropolis chains: one warp per chain, latency-bound; "
                             "HBM carries only the one-time staging (roofline_smem: the "
                             "per-move basis; latency_bound: the critical chain)"},
        # per move: 2 x deg pair terms (deg = arc-list entries per bead of the
        # ensemble), each a 16-byte position and an 8-byte arc entry, ~15 FLOP
        "roofline_smem": W._smem_roofline(value / world, 2 * deg * 24.0, 2 * deg * 15.0,
                                          sm_mhz),
        "latency_bound": {"critical_region_beads": r["crit"]["region_beads"],
                          "critical_chain_moves": r["crit"]["moves"],
                          "ms_per_move_alone": r["crit"]["ms_per_move_alone"],
                          "bound_ms": r["crit"]["bound_ms"],
                          "frac": r["crit"]["bound_ms"] / r["step_ms"],
                          "note": "the chain with the most moves, its region annealed alone: "
                                  "no pass can be shorter than its moves x time per move"},
        "clocks": r["clocks"],
        "gpu_launches": r["n_launch"] * args.steps,
    }
    if r["plain_s"] is not None:
        line["plain_structures_per_s"] = 1.0 / r["plain_s"]
        line["batched_over_plain"] = structs / world / (1.0 / r["plain_s"])
    if cpu:
        mps = total_moves / world / N_STRUCT   # moves per structure (this arm)
        line["cpu_baseline"] = {"value": cpu["moves_per_s"], "unit": "moves/s",
                                "cores": cpu["cores"], "kind": "port",
                                "sample": f"1 of {cpu['share']} equal parts of the ensemble's "
                                          f"own blocks ({cpu['blocks']} blocks, same size "
                                          f"distribution) on {cpu['cores']} cores at once, "
                                          f"largest first: completed moves / "
                                          f"{cpu['wall_s']:.1f} s wall",
                                "structures_per_s": cpu["moves_per_s"] / mps}
    if rank == 0 and world == 1 and args.configs:
        line["configs"] = config_records(args)
    print(json.dumps(line))


def ensemble_config(args, world):
    """The workload as both arms state it (same dictionary)."""
    return {"workload": WORKLOAD, "structures": N_STRUCT * world,
            "blocks_per_structure": N_BLOCKS, "regions": N_STRUCT * N_BLOCKS * world,
            "block_seeds": "structure s: sizes from seed 10000 + s, block b from 1000 s + b",
            "fp64_resync_every": args.resync,
            "l2": "GPU leg: a 256 MB buffer is written between timed steps (L2 is 129 MB)",
            "parallelism": f"replicas x{world}"}


def reference_main(args, config):
    """The reference arm on the GPU leg's own ensemble: its 1536 blocks split
    into warmup + steps parts of the same size distribution; the warm-up
    parts run untimed, the timed parts as one pass of a process pool over
    every host core, largest block first.  Wall-clock moves/s and
    structures/s."""
    from oracle import oracle as O
    O.build()
    cores = os.cpu_count() or 1
    shares = size_shares(ensemble_blocks(0), args.warmup + args.steps)
    warm = [b for p in shares[:args.warmup] for b in p]
    timed = [b for p in shares[args.warmup:] for b in p]
    with mp.get_context("spawn").Pool(cores) as pool:
        if warm:
            cpu_anneal_blocks(pool, warm)
        moves, wall, cpu_s = cpu_anneal_blocks(pool, timed)
    v = moves / wall
    structs = len(timed) / N_BLOCKS / wall
    line = {
        "impl": "reference", "metric": "MC moves/s", "value": v, "unit": "moves/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": wall / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic", "config": config,
        "moves_per_step": moves / args.steps,
        "structures_per_s": structs,
        "cpu_baseline": {"value": v, "unit": "moves/s", "cores": cores, "kind": "port",
                         "sample": f"the ensemble's {len(timed)} timed blocks ({args.steps} of "
                                   f"{args.warmup + args.steps} equal parts of its "
                                   f"{len(timed) + len(warm)} blocks) on {cores} cores, "
                                   f"{wall:.1f} s wall ({cpu_s:.0f} CPU s)",
                         "structures_per_s": structs},
        "e2e": {"value": v, "unit": "moves/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))


def config_records(args) -> dict:
    """The other configurations beside the default line, each with its value,
    roofline, e2e through the host-buffer C call and its CPU baseline timed
    on this host's cores in the same run: 0 plain (one 256-bead region),
    1 heatmap (one 2048-bead chain, 100k moves; the two-maps-per-SM batch as
    the HBM-bound form), 3 genome smoothing (20k sweeps), 4 serving (5000
    requests at 200/s)."""
    out = {}
    budget = max(5.0, min(args.cpu_budget, 15.0))

    def ns(**kw):
        base = dict(steps=3, warmup=1, moves=0, requests=0, n=0, maps=0, impl="ours",
                    cpu_budget=budget)
        base.update(kw)
        return argparse.Namespace(**base)

    def timed(name, fn):
        t = time.perf_counter()
        try:
            rec = fn()
        except Exception as e:  # a failing sub-record must not lose the main line
            rec = {"error": f"{type(e).__name__}: {e}"}
        rec["record_wall_s"] = time.perf_counter() - t
        out[name] = rec

    timed("0_plain", lambda: plain_record(ns(steps=5, warmup=2)))
    timed("1_heatmap", lambda: heatmap_record(ns(), 1))
    timed("1_heatmap_batch", lambda: heatmap_record(ns(), 0))
    timed("3_smooth", lambda: smooth_record(ns()))
    timed("4_serve", lambda: serve_record(ns()))
    return out


if __name__ == "__main__":
    main()
