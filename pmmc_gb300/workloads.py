"""Workloads and GPU legs of bench.py's lines other than the default
ensemble (bench.py --workload NAME; bench.py adds each line's CPU baseline,
clocks and launch count).

heatmap        one chain on a 2048-bead map (contact map |i-j|^-1 x
               lognormal(0.5), 20 TADs x3, expected distance c^-1/3), T0 5,
               cooling 0.9999, milestones every 100k moves: moves/s.
heatmap-batch  one chain per distinct 2048-bead map (16 MB each; the
               generated map scaled by a per-map factor), two maps per SM by
               default: the form whose rows stream from HBM; reports HBM GB/s
               of the row traffic (4 bytes per row entry per move) and of the
               two FP64 full scores per map.
smooth         genome-scale smoothing: 23 chromosomes (~300k beads, anchors
               every Poisson(10) beads, fixed), split at the anchors into
               independent regions; 20k sweeps (moves = 20k x free beads).
plain          one arc-level region of 256 beads, 400 arcs (seed 42), T0 5,
               cooling 0.9999, milestones every 50k moves, threshold 0.99,
               through the plain drop-in call (host buffers, one call per
               step): one chain, and the reference GPU form's best of
               4 x SM-count chains.
distmap        expected-distance map of a 16384-bead contact map (1 GiB:
               |i-j|^-1 x lognormal(0.5), 10 % zeros, diagonal band 1),
               createDistanceHeatmap's transform and clamp; HBM GB/s.
equidistant    equidistant model of the largest chromosome of the genome
               workload (~24.8k clusters at 10 kb) resampled every 100 bp
               (~2.5M points); points/s.
targets        anchor-level expected distances of one chromosome: 4000
               anchors, 6000 arcs, 2M genomic-position long arcs (Hi-C style,
               seed 21), built as the annealer's CSR
               (calcAnchorExpectedDistancesHeatmap); arcs/s.
stress         stress refinement of one chromosome's anchors (4000 anchors,
               200k long arcs -> 70k pair targets, seed 51, reference spring
               and angle constants, step 0.01) for 2000 iterations (the run
               may converge earlier); iterations/s.
serve          request loop: 5000 arc-level regions, sizes round(exp U[ln 64,
               ln 8192]), 1.5625 arcs per bead (400 per 256 beads), Poisson
               arrivals at 200 requests/s (seed 11), 20k moves each, device
               budget 40 GiB.  Replayed open-loop at the trace's arrival times
               (latency p50/p99) and saturated (all requests at once:
               structures/s and moves/s).
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


def _traffic(kernel: str, workload: str):
    """DRAM bytes per launch from the committed ncu summary, if recorded."""
    p = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))),
                     "profiles", "traffic_per_launch.txt")
    if os.path.exists(p):
        for line in open(p):
            f = line.split()
            if len(f) >= 3 and f[0] == kernel and f[1] == workload:
                return float(f[2])
    return None


def smem_peak_gbs(sm_mhz: float = 2070.0, sms: int = 152) -> float:
    """Nominal shared-memory bandwidth of the device: 128 bytes per clock per
    SM (no measured figure exists for it)."""
    return 128.0 * sms * sm_mhz * 1e6 / 1e9


def fp32_peak_tflops(sm_mhz: float = 2070.0, sms: int = 152) -> float:
    """Nominal FP32 rate: 128 FMA lanes per SM, 2 FLOP per FMA."""
    return 2.0 * 128.0 * sms * sm_mhz * 1e6 / 1e12


def _smem_roofline(moves_per_s: float, bytes_per_move: float, flop_per_move: float,
                   sm_mhz: float = 2070.0) -> dict:
    """Shared-memory and FP32 roofline of an in-SMEM annealing kernel, on the
    algorithmic bytes and FLOP of one move, against nominal device peaks."""
    smem = moves_per_s * bytes_per_move / 1e9
    flops = moves_per_s * flop_per_move / 1e12
    return {"bound": "smem", "achieved": smem, "peak": smem_peak_gbs(sm_mhz), "unit": "GB/s",
            "frac": smem / smem_peak_gbs(sm_mhz), "traffic": None,
            "peak_source": "nominal (128 B/clk/SM, 152 SMs, 2070 MHz)",
            "algorithmic_bytes_per_move": bytes_per_move,
            "fp32": {"achieved": flops, "peak": fp32_peak_tflops(sm_mhz), "unit": "TFLOP/s",
                     "frac": flops / fp32_peak_tflops(sm_mhz),
                     "algorithmic_flop_per_move": flop_per_move,
                     "peak_source": "nominal (128 FMA/clk/SM)"}}


HEATMAP_ANNEAL = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=100_000, improvement=0.99)


def heatmap_maps(n_maps: int):
    """The 2048-bead heatmap region (20 TAD blocks, expected distance c^-1/3)
    and one scale factor per distinct map: the batch holds the generated map
    scaled by a per-map factor, so every chain streams its own rows."""
    base = synth.heatmap_region(2048, seed=7)
    rng = np.random.default_rng(11)
    scales = [1.0] + list(rng.uniform(0.8, 1.25, n_maps - 1))
    return base, scales


def heatmap(args, n_maps):
    import torch
    torch.cuda.init()
    ctx = capi.Context(0)
    if n_maps <= 0:          # two distinct maps per SM (two chains share an SM)
        n_maps = 2 * ctx.sm_count
    base, scales = heatmap_maps(n_maps)
    inputs = [capi.HeatmapInput(base.pos, (base.heat * np.float32(sc)).astype(np.float32),
                                base.diag, base.bounds) for sc in scales]
    moves = args.moves or (100_000 if n_maps == 1 else 20_000)
    prm = capi.default_params(capi.LEVEL_HEATMAP, schedule=capi.SCHEDULE_CPU, max_moves=moves,
                              **HEATMAP_ANNEAL)
    times, walls, total = [], [], 0
    for k in range(args.warmup + args.steps):
        ctx.set_seed(7)
        t0 = time.perf_counter()
        out, res, ms, _ = capi.heatmap_batch_anneal(ctx, inputs, prm, [1.0] * len(inputs))
        wall = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(ms)
            walls.append(wall)
            total = sum(r.moves for r in res)
    ms = float(np.mean(times))
    wall = float(np.median(walls))
    row_bytes = 4 * 2048
    # one launch reads each move's row once and each map twice in full (the
    # FP64 start and end scores)
    alg = total * row_bytes + 2 * n_maps * 2048 * 2048 * 4
    achieved = alg / (ms * 1e-3) / 1e9
    peak, kind = _peak()
    traffic = _traffic("heatmap_anneal_kernel", f"heatmap_{n_maps}x2048_moves{moves}")
    line = {
        "metric": "MC moves/s", "value": total / (ms * 1e-3), "unit": "moves/s",
        "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"heatmap_{n_maps}x2048_T0=5_cool0.9999_moves{moves}",
                   "maps": n_maps, "moves_per_step": total},
        "final_energy_rel_error_max": max(r.rel_error for r in res),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "peak_source": kind,
                     "algorithmic_bytes_per_move": row_bytes,
                     "algorithmic_bytes_per_launch": alg},
        # pmmc_heatmap_batch_anneal with host arrays: the reciprocal map is
        # packed and checked on the host, copied up, annealed, copied back
        "e2e": {"value": total / wall, "unit": "moves/s", "ms_per_step": wall * 1e3,
                "h2d_bytes_per_step": int(sum(4 * (x.n * x.n + 3 * x.n) for x in inputs)),
                "d2h_bytes_per_step": int(sum(12 * x.n + 56 for x in inputs))},
    }
    return line


SMOOTH_ANNEAL = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=10**9, improvement=0.99)


def smooth_segments():
    """The genome-smoothing workload's regions: about 300k beads over the 23
    chromosomes, cut at the fixed anchors into (pos, dist_to_next, fixed)
    segments of at least one free bead."""
    out = []
    for ch in synth.smooth_genome(300_000, seed=3):
        a = np.nonzero(ch.fixed)[0]
        for l, r in zip(a[:-1], a[1:]):
            if r - l >= 2:
                sl = slice(l, r + 1)
                out.append((ch.pos[sl], ch.dist_to_next[sl], ch.fixed[sl]))
    return out


def smooth_packed():
    """The genome-smoothing regions packed back to back: (bead_off, pos,
    dist_to_next, fixed)."""
    segs = smooth_segments()
    off = np.zeros(len(segs) + 1, np.int64)
    off[1:] = np.cumsum([len(p) for p, _, _ in segs])
    return (off, np.concatenate([p for p, _, _ in segs]).astype(np.float32),
            np.concatenate([d for _, d, _ in segs]).astype(np.float32),
            np.concatenate([f for _, _, f in segs]).astype(np.uint8))


def smooth(args):
    ctx = capi.Context(0)
    segs = [capi.SmoothInput(*x) for x in smooth_segments()]
    packed = smooth_packed()
    free = sum(int((x.fixed == 0).sum()) for x in segs)
    sweeps = args.moves or 20_000
    prm = capi.default_params(capi.LEVEL_SMOOTH, schedule=capi.SCHEDULE_CPU, resync_every=1000,
                              **SMOOTH_ANNEAL)
    prm.max_moves = -int(sweeps)
    steps = np.full(len(segs), 0.5, np.float32)
    times, walls, total = [], [], 0
    for k in range(args.warmup + args.steps):
        ctx.set_seed(3)
        # each region: sweeps x its free beads; host arrays in and out
        # through the packed entry point
        t0 = time.perf_counter()
        out, res, ms = capi.smooth_batch_anneal_packed(ctx, *packed, prm, steps)
        wall = time.perf_counter() - t0
        if k >= args.warmup:
            times.append(ms)
            walls.append(wall)
            total = sum(r.moves for r in res)
    ms = float(np.mean(times))
    wall = float(np.median(walls))
    beads = sum(x.n for x in segs)
    # kernel launches of a call: one per non-empty class under the library's
    # default windows (32 slots for regions with 20+ free beads, 8 for the
    # rest; a region whose chains overflow a 200 KB slice at that window
    # takes the one-move kernel)
    classes = set()
    for x in segs:
        w = 32 if int((x.fixed == 0).sum()) >= 20 else 8
        classes.add(w if (32 // w) * x.n * 28 <= 200 * 1024 else 0)
    # per move: two bonds and three angles read five beads (16 B each) and
    # take ~80 FLOP (the smoothing energy of a move)
    sm = _smem_roofline(total / (ms * 1e-3), 80.0, 80.0)
    line = {
        "metric": "MC moves/s", "value": total / (ms * 1e-3), "unit": "moves/s", "n_gpus": 1,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"genome_smoothing_{len(segs)}regions_{free}free_beads_"
                               f"{sweeps}sweeps", "moves_per_step": total},
        "final_energy_rel_error_max": max(r.rel_error for r in res),
        "kernel_launches_per_step": len(classes),
        "roofline": sm,
        "e2e": {"value": total / wall, "unit": "moves/s", "ms_per_step": wall * 1e3,
                "h2d_bytes_per_step": int(beads * (12 + 4 + 1) + len(segs) * 80),
                "d2h_bytes_per_step": int(beads * 12 + len(segs) * 56)},
    }
    return line


def _smooth_run(ctx, segs, prm, sweeps):
    # one launch: every region anneals `sweeps` proposals per free bead
    # (max_moves < 0 sets that cap per region)
    prm.max_moves = -int(sweeps)
    out, res, ms = capi.smooth_batch_anneal(ctx, segs, prm, [0.5] * len(segs))
    return out, res, ms


SERVE_ANNEAL = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=20_000, improvement=0.99,
                    max_moves=20_000, resync_every=1000)
SERVE_STEP = 0.5
SERVE_BUDGET = 40 << 30


def serve_trace(n_req: int = 5000, rate: float = 200.0, seed: int = 11,
                lo: int = 64, hi: int = 8192):
    """Region sizes and arrival times (s) of the serving trace."""
    rng = np.random.default_rng(seed)
    sizes = np.rint(np.exp(rng.uniform(np.log(lo), np.log(hi), n_req))).astype(int)
    gaps = rng.exponential(1.0 / rate, n_req)
    arrivals = np.cumsum(gaps) - gaps[0]
    return sizes, arrivals


def serve_region(k: int, n: int, seed: int = 11):
    return synth.arcs_region(int(n), int(round(1.5625 * n)), seed=seed * 100_000 + k)


def serve_seed(k: int) -> int:
    return 11_000 + k


def _serve_pass(ctx, prm, inputs, arrivals):
    """One pass through a fresh server; arrivals None = all at once.
    Returns (latencies ms, moves, wall s, stats, max rel error)."""
    import queue
    import threading
    sv = capi.Server(ctx, prm, budget_bytes=SERVE_BUDGET)
    q = queue.Queue()
    t0 = time.perf_counter()

    def produce():
        for k, inp in enumerate(inputs):
            if arrivals is not None:
                dt = t0 + arrivals[k] - time.perf_counter()
                if dt > 0:
                    time.sleep(dt)
            q.put(sv.submit(inp, SERVE_STEP, serve_seed(k)))
        q.put(None)

    th = threading.Thread(target=produce)
    th.start()
    lat, moves, err = [], 0, 0.0
    while True:
        t = q.get()
        if t is None:
            break
        _, res, ms = sv.wait(t)
        lat.append(ms)
        moves += res.moves
        err = max(err, res.rel_error)
    th.join()
    wall = time.perf_counter() - t0
    st = sv.stats()
    sv.close()
    return np.array(lat), moves, wall, st, err


def serve(args) -> dict:
    """The serving line (without the CPU baseline, which the caller adds)."""
    n_req = args.requests or 5000
    sizes, arrivals = serve_trace(n_req)
    t = time.perf_counter()
    inputs = []
    for k, n in enumerate(sizes):
        r = serve_region(k, n)
        rp, col, tgt = r.csr()
        inputs.append(capi.ArcsInput(r.pos, rp, col, tgt))
    gen_s = time.perf_counter() - t
    ctx = capi.Context(0)
    prm = capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_CPU, **SERVE_ANNEAL)
    # warm-up: module load, pinned staging, allocator pool
    for _ in range(max(1, args.warmup)):
        _serve_pass(ctx, prm, inputs[:64], None)
    sat_lat, sat_moves, sat_wall, sat_st, sat_err = _serve_pass(ctx, prm, inputs, None)
    ol_lat, ol_moves, ol_wall, ol_st, ol_err = _serve_pass(ctx, prm, inputs, arrivals)
    line = {
        "metric": "structures/s", "value": n_req / sat_wall, "unit": "structures/s",
        "n_gpus": 1, "steps": 1, "warmup": max(1, args.warmup),
        "ms_per_step": sat_wall * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"serve_{n_req}req_poisson200_sizes64-8192_"
                               f"1.5625arcs_per_bead_20k_moves_budget40GiB",
                   "requests": n_req, "beads_total": int(sizes.sum()),
                   "generation_s": gen_s},
        "saturated": {"structures_per_s": n_req / sat_wall, "moves_per_s": sat_moves / sat_wall,
                      "wall_s": sat_wall, "latency_ms_p50": float(np.percentile(sat_lat, 50)),
                      "latency_ms_p99": float(np.percentile(sat_lat, 99)),
                      "waves": sat_st["waves"], "running_peak": sat_st["running_peak"],
                      "bytes_peak": sat_st["bytes_peak"]},
        "open_loop_200rps": {"structures_per_s": n_req / ol_wall,
                             "moves_per_s": ol_moves / ol_wall, "wall_s": ol_wall,
                             "latency_ms_p50": float(np.percentile(ol_lat, 50)),
                             "latency_ms_p99": float(np.percentile(ol_lat, 99)),
                             "latency_ms_mean": float(ol_lat.mean()),
                             "waves": ol_st["waves"], "running_peak": ol_st["running_peak"]},
        "final_energy_rel_error_max": max(sat_err, ol_err),
        # per move as the plain region: 2 x deg pair terms, deg = 3.125
        "roofline": _smem_roofline(sat_moves / sat_wall, 2 * 3.125 * 24.0, 2 * 3.125 * 15.0),
        "e2e": {"value": n_req / sat_wall, "unit": "structures/s",
                "h2d_bytes_per_step": None, "d2h_bytes_per_step": None,
                "note": "host arrays in, host results out, through pmmc_server_*"},
    }
    return line


PLAIN_ANNEAL = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=50_000, improvement=0.99)


def plain_region():
    return synth.arcs_region(256, 400, seed=42)


def plain(args) -> dict:
    """One 256-bead region through pmmc_arcs_anneal (the drop-in call, host
    buffers in and out): moves/s of one chain and of the multi-chain form."""
    import time as _t
    r = plain_region()
    rp, col, tgt = r.csr()
    inp = capi.ArcsInput(r.pos, rp, col, tgt)
    ctx = capi.Context(0)
    prm = capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_CPU, **PLAIN_ANNEAL)
    out = {}
    for name, chains in (("one_chain", 1), ("best_of_chains", 0)):
        for _ in range(max(1, args.warmup)):
            capi.arcs_anneal(ctx, inp, prm, 0.5, chains)
        times, moves, tot, err = [], 0, 0, 0.0
        for k in range(args.steps):
            ctx.set_seed(42 + k)
            t = _t.perf_counter()
            pos, res = capi.arcs_anneal(ctx, inp, prm, 0.5, chains)
            times.append(_t.perf_counter() - t)
            moves, tot, err = res.moves, res.total_moves, max(err, res.rel_error)
        dt = float(np.median(times))
        out[name] = {"ms_per_call": dt * 1e3, "moves_per_chain": int(moves),
                     "moves_per_s": tot / dt, "chain_moves_per_s": moves / dt,
                     "rel_error": err}
    one = out["one_chain"]
    return {
        "metric": "MC moves/s", "value": one["chain_moves_per_s"], "unit": "moves/s",
        "n_gpus": 1, "steps": args.steps, "warmup": max(1, args.warmup),
        "ms_per_step": one["ms_per_call"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "arcs_plain_256beads_400arcs_seed42_T0=5_cool0.9999_"
                               "milestone50k_thr0.99", "call": "pmmc_arcs_anneal"},
        "forms": out,
        # per move: 2 x deg pair terms (deg = 800 / 256 arc-list entries per
        # bead), each a 16-byte position and an 8-byte arc entry, ~15 FLOP;
        # one serial chain runs on one SM of the device
        "roofline": dict(_smem_roofline(one["chain_moves_per_s"], 2 * 3.125 * 24.0,
                                        2 * 3.125 * 15.0),
                         note="one serial chain on one of 152 SMs: latency-bound"),
        "e2e": {"value": one["chain_moves_per_s"], "unit": "moves/s",
                "h2d_bytes_per_step": int(r.pos.nbytes + rp.nbytes + col.nbytes + tgt.nbytes),
                "d2h_bytes_per_step": int(r.pos.nbytes)},
        "final_energy_rel_error_max": max(v["rel_error"] for v in out.values()),
    }


def distmap_contact(n: int, seed: int = 5):
    rng = np.random.default_rng(seed)
    c = np.empty((n, n), np.float32)
    step = 1024
    for a in range(0, n, step):       # row blocks: bounded temporaries
        i = np.arange(a, min(n, a + step))[:, None]
        sep = np.abs(i - np.arange(n)[None, :]).astype(np.float32)
        blk = np.where(sep > 0, 1.0 / np.maximum(sep, 1.0), 2.0).astype(np.float32)
        blk *= rng.lognormal(0.0, 0.5, blk.shape).astype(np.float32)
        blk[rng.random(blk.shape) < 0.1] = 0.0
        c[a:a + step] = blk
    return c


def distmap(args) -> dict:
    """createDistanceHeatmap on the device: kernel time per call (device
    buffers) and the host-buffer call."""
    import time as _t
    n = args.n or 16384
    c = distmap_contact(n)
    ctx = capi.Context(0)
    ms_k, e2e = [], []
    for k in range(max(1, args.warmup) + args.steps):
        t = _t.perf_counter()
        d, avg, mx, ms = capi.distance_heatmap(ctx, c, 1, 100.0, -0.333, 2.0)
        dt = _t.perf_counter() - t
        if k >= max(1, args.warmup):
            ms_k.append(ms)
            e2e.append(dt)
    ms = float(np.median(ms_k))
    # contact upper triangle read, upper triangle written and read back, the
    # lower triangle written (clamped values rewrite a part of the upper one)
    alg = 4.0 * n * n * 2.0
    peak, kind = _peak()
    achieved = alg / (ms * 1e-3) / 1e9
    return {
        "metric": "matrix entries/s", "value": n * n / (ms * 1e-3), "unit": "entries/s",
        "n_gpus": 1, "steps": args.steps, "warmup": max(1, args.warmup), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"distance_heatmap_{n}x{n}_diag1_scale100_power-0.333_stretch2",
                   "n": n},
        "e2e": {"value": n * n / float(np.median(e2e)), "unit": "entries/s",
                "h2d_bytes_per_step": 4 * n * n, "d2h_bytes_per_step": 4 * n * n},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "peak_source": kind,
                     "algorithmic_bytes_per_launch": alg},
        "avg": avg, "clamp": mx,
    }


def equidistant_level(seed: int = 3):
    """The largest chromosome of the genome workload as a level: 10 kb
    clusters, positions from the smoothing chain."""
    ch = max(synth.smooth_genome(300_000, seed=seed), key=lambda c: c.n)
    n = ch.n
    start = (np.arange(n, dtype=np.int64) * 10_000 + 1).astype(np.int32)
    end = (start + 9_999).astype(np.int32)
    gpos = ((start.astype(np.int64) + end) // 2).astype(np.int32)
    return gpos, start, end, ch.pos


def equidistant(args) -> dict:
    import time as _t
    gpos, start, end, pos = equidistant_level()
    res = args.n or 100
    ctx = capi.Context(0)
    ms_k, e2e, m = [], [], 0
    for k in range(max(1, args.warmup) + args.steps):
        t = _t.perf_counter()
        pts, ms = capi.equidistant_model(ctx, gpos, pos, int(end[0]), int(start[-1]),
                                         int(gpos[0]), int(gpos[-1]), res)
        dt = _t.perf_counter() - t
        m = len(pts)
        if k >= max(1, args.warmup):
            ms_k.append(ms)
            e2e.append(dt)
    ms = float(np.median(ms_k))
    peak, kind = _peak()
    alg = 12.0 * m + 16.0 * len(gpos)   # points written, level read
    achieved = alg / (ms * 1e-3) / 1e9
    return {
        "metric": "points/s", "value": m / (ms * 1e-3), "unit": "points/s", "n_gpus": 1,
        "steps": args.steps, "warmup": max(1, args.warmup), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"equidistant_{len(gpos)}clusters_10kb_every{res}bp",
                   "points": m},
        "e2e": {"value": m / float(np.median(e2e)), "unit": "points/s",
                "h2d_bytes_per_step": int(gpos.nbytes + pos.nbytes),
                "d2h_bytes_per_step": 12 * m},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": None, "peak_source": kind,
                     "algorithmic_bytes_per_launch": alg},
    }


TARGETS_ANCHORS = 4000


def targets_problem(n_long: int = 2_000_000):
    return synth.anchor_targets_problem(n_anchors=TARGETS_ANCHORS, n_long=n_long, seed=21)


def targets(args) -> dict:
    """calcAnchorExpectedDistancesHeatmap on the device: device time per call
    (L2 flushed between calls) and the host-buffer call end to end."""
    import time as _t
    import torch
    n_long = args.n or 2_000_000
    t = targets_problem(n_long)
    ctx = capi.Context(0)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    ms_k, e2e, ph = [], [], []
    nnz = 0
    for k in range(max(3, args.warmup) + args.steps):
        flush.fill_(k & 0xff)
        torch.cuda.synchronize()
        t0 = _t.perf_counter()
        rp, col, tgt, st, ms = capi.anchor_targets(ctx, t)
        dt = _t.perf_counter() - t0
        nnz = len(col)
        if k >= max(3, args.warmup):
            ms_k.append(ms)
            e2e.append(dt)
            ph.append(capi.anchor_targets_phases())
    ms = float(np.median(ms_k))
    units = len(t["arc_start"]) + n_long
    phases = {key: float(np.median([p[key] for p in ph])) for key in ph[0]}
    # the larger of the two own kernels of the long-arc pass:
    #   long_map      8 bytes of positions read, 8 + 4 of key and index written
    #                 per long arc;
    #   long_resolve  8 + 4 bytes of sorted key and index read per entry, the
    #                 count of every written long arc (4), 8 + 4 per emitted pair
    n_items = n_long + len(t["arc_start"])
    n_emit = nnz // 2
    algs = {"map": ("long_map", 20.0 * n_long),
            "resolve": ("long_resolve", 12.0 * n_items + 4.0 * st["applied"] + 12.0 * n_emit)}
    dom = max(algs, key=lambda key: phases[key])
    kernel, alg = algs[dom]
    peak, kind = _peak()
    achieved = alg / (phases[dom] * 1e-3) / 1e9
    h2d = sum(int(np.asarray(t[key]).nbytes) for key in
              ("active", "arc_ptr", "arc_idx", "arc_start", "arc_end", "arc_score",
               "long_start", "long_end", "long_score", "anc_start", "anc_end", "memo"))
    return {
        "metric": "arcs/s", "value": units / (ms * 1e-3), "unit": "arcs/s", "n_gpus": 1,
        "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32",
        "data": "synthetic",
        "config": {"workload": f"anchor_targets_{TARGETS_ANCHORS}anchors_"
                               f"{len(t['arc_start'])}arcs_{n_long}long_arcs",
                   "l2": "256 MB buffer written between calls", "nnz": nnz,
                   "stats": st},
        "phases_ms": phases,
        "e2e": {"value": units / float(np.median(e2e)), "unit": "arcs/s",
                "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": int(4 * (len(rp) + 2 * nnz))},
        "roofline": {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak,
                     "traffic": _traffic(kernel, f"targets_{n_long}"),
                     "peak_source": kind, "algorithmic_bytes_per_launch": alg},
    }


STRESS_ANCHORS, STRESS_LONG, STRESS_LR = 4000, 200_000, 0.01


def stress_problem():
    return synth.stress_problem(n_anchors=STRESS_ANCHORS, n_long=STRESS_LONG, seed=51)


def stress(args) -> dict:
    """stressRefineAnchors on the device: one cooperative launch per call;
    device time of the descent and the host-buffer call end to end (pair
    list built on the host)."""
    import time as _t
    t = stress_problem()
    it = args.moves or 2000
    ctx = capi.Context(0)
    ms_k, e2e, res = [], [], None
    for k in range(max(3, args.warmup) + args.steps):
        t0 = _t.perf_counter()
        _, _, res = capi.stress_refine(ctx, t, it, STRESS_LR)
        dt = _t.perf_counter() - t0
        if k >= max(3, args.warmup):
            ms_k.append(res["kernel_ms"])
            e2e.append(dt)
    ms = float(np.median(ms_k))
    iters = res["iterations"]
    n, p = STRESS_ANCHORS, res["n_pairs"]
    # per iteration: each pair entry (8 bytes) and the partner's position
    # (16) read from both ends, each anchor's position, neighbours, target
    # and gradient (~80 bytes); the working set (1.2 MB) stays in L2
    alg = iters * (2.0 * p * 24.0 + 80.0 * n)
    peak, kind = _peak()
    achieved = alg / (ms * 1e-3) / 1e9
    return {
        "metric": "iterations/s", "value": iters / (ms * 1e-3), "unit": "iterations/s",
        "n_gpus": 1, "steps": args.steps, "warmup": max(3, args.warmup), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic",
        "config": {"workload": f"stress_refine_{n}anchors_{STRESS_LONG}long_arcs_"
                               f"{p}pairs_lr{STRESS_LR}_max{it}",
                   "iterations": iters, "stop": res["stop"], "final_energy": res["total"],
                   "pair_terms_per_s": iters * p / (ms * 1e-3)},
        "e2e": {"value": iters / float(np.median(e2e)), "unit": "iterations/s",
                "h2d_bytes_per_step": int(sum(np.asarray(t[key]).nbytes for key in
                                              capi.stress_arrays(t))),
                "d2h_bytes_per_step": 16 * n},
        "roofline": {"bound": "hbm", "kernel": "stress_kernel", "achieved": achieved,
                     "peak": peak, "unit": "GB/s", "frac": achieved / peak, "traffic": None,
                     "peak_source": kind, "algorithmic_bytes_per_launch": alg,
                     "note": "L2-resident working set; bound by the per-anchor gather "
                             "latency and two grid barriers per iteration"},
    }
