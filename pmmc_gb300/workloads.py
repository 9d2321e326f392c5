"""Benchmark lines for the heatmap and smoothing kernels (bench.py
--workload heatmap | heatmap-batch | smooth).

heatmap        one chain on a 2048-bead map (contact map |i-j|^-1 x
               lognormal(0.5), 20 TADs x3, expected distance c^-1/3), T0 5,
               cooling 0.9999, milestones every 100k moves: moves/s.
heatmap-batch  one chain per distinct 2048-bead map (16 MB each; the
               generated map scaled by a per-map factor), one map per SM by
               default: the form whose rows stream from HBM; reports HBM GB/s
               of the row traffic (4 bytes per row entry per move).
smooth         genome-scale smoothing: 23 chromosomes (~300k beads, anchors
               every Poisson(10) beads, fixed), split at the anchors into
               independent regions; 20k sweeps (moves = 20k x free beads).
"""
from __future__ import annotations

import json
import os
import time

import numpy as np

from . import capi, synth


def _peak():
    p = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                     "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return float(json.load(open(p))["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _heatmap(args, n_maps):
    import torch
    torch.cuda.init()
    ctx = capi.Context(0)
    base = synth.heatmap_region(2048, seed=7)
    # distinct maps in memory (the rows of every chain stream from HBM): the
    # generated map scaled by a per-map factor
    rng = np.random.default_rng(11)
    scales = [1.0] + list(rng.uniform(0.8, 1.25, n_maps - 1))
    inputs = [capi.HeatmapInput(base.pos, (base.heat * np.float32(sc)).astype(np.float32),
                                base.diag, base.bounds) for sc in scales]
    moves = args.moves or (100_000 if n_maps == 1 else 20_000)
    prm = capi.default_params(capi.LEVEL_HEATMAP, max_temp=5.0, dt_temp=0.9999,
                              milestone_steps=100_000, improvement=0.99,
                              schedule=capi.SCHEDULE_CPU, max_moves=moves)
    times, total = [], 0
    for k in range(args.warmup + args.steps):
        ctx.set_seed(7)
        out, res, ms, _ = capi.heatmap_batch_anneal(ctx, inputs, prm, [1.0] * len(inputs))
        if k >= args.warmup:
            times.append(ms)
            total = sum(r.moves for r in res)
    ms = float(np.mean(times))
    row_bytes = 4 * 2048
    achieved = total * row_bytes / (ms * 1e-3) / 1e9
    peak, kind = _peak()
    line = {
        "metric": "MC moves/s", "value": total / (ms * 1e-3), "unit": "moves/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"heatmap_{n_maps}x2048_T0=5_cool0.9999_moves{moves}",
                   "maps": n_maps, "moves_per_step": total},
        "final_energy_rel_error_max": max(r.rel_error for r in res),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "peak_source": kind,
                     "algorithmic_bytes_per_move": row_bytes},
    }
    print(json.dumps(line))


def _smooth(args):
    ctx = capi.Context(0)
    chains = synth.smooth_genome(300_000, seed=3)
    segs = []
    for ch in chains:
        a = np.nonzero(ch.fixed)[0]
        for l, r in zip(a[:-1], a[1:]):
            if r - l >= 2:
                sl = slice(l, r + 1)
                segs.append(capi.SmoothInput(ch.pos[sl], ch.dist_to_next[sl], ch.fixed[sl]))
    free = sum(int((x.fixed == 0).sum()) for x in segs)
    sweeps = args.moves or 20_000
    prm = capi.default_params(capi.LEVEL_SMOOTH, max_temp=5.0, dt_temp=0.9999,
                              milestone_steps=10**9, improvement=0.99,
                              schedule=capi.SCHEDULE_CPU, resync_every=1000)
    steps = []
    for x in segs:
        steps.append(0.5)
    times, total = [], 0
    for k in range(args.warmup + args.steps):
        ctx.set_seed(3)
        # each region: sweeps x its free beads
        out, res, ms = _smooth_run(ctx, segs, prm, sweeps)
        if k >= args.warmup:
            times.append(ms)
            total = sum(r.moves for r in res)
    ms = float(np.mean(times))
    line = {
        "metric": "MC moves/s", "value": total / (ms * 1e-3), "unit": "moves/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"genome_smoothing_{len(segs)}regions_{free}free_beads_"
                               f"{sweeps}sweeps", "moves_per_step": total},
        "final_energy_rel_error_max": max(r.rel_error for r in res),
    }
    print(json.dumps(line))


def _smooth_run(ctx, segs, prm, sweeps):
    # regions share one move cap per call: group them by free-bead count
    groups = {}
    for i, x in enumerate(segs):
        groups.setdefault(int((x.fixed == 0).sum()), []).append(i)
    res_all = [None] * len(segs)
    out_all = [None] * len(segs)
    ms_total = 0.0
    for nf, idx in sorted(groups.items()):
        prm.max_moves = sweeps * max(nf, 1)
        out, res, ms = capi.smooth_batch_anneal(ctx, [segs[i] for i in idx], prm,
                                                [0.5] * len(idx))
        ms_total += ms
        for j, i in enumerate(idx):
            res_all[i] = res[j]
            out_all[i] = out[j]
    return out_all, res_all, ms_total


def main(args):
    if args.workload == "heatmap":
        _heatmap(args, 1)
    elif args.workload == "heatmap-batch":
        _heatmap(args, args.maps or 152)
    else:
        _smooth(args)
