"""The oracle's restatement of the reference kernels' stopping schedule
(ORC_SCHEDULE_GPU) against a second restatement written here in Python,
move by move, from the kernel source:

* MonteCarloArcsKernel (src/ParallelMonteCarloArcs.cu:494-655): 256-move
  blocks while iterations < stop_condition_steps (:522,631); uphill test only
  when T > 0 and score_prev > 0 (:598-603); after each block the milestone
  predicate with its 1e-10 guard (:635-641), the miss counter (:643-646) and
  the stop on milestone_fails or a score below 1e-5 (:648-650);
* MonteCarloSmoothKernelMultiWarp (src/ParallelMonteCarloSmooth.cu:258-337):
  256-move blocks while iterations < stop_condition_steps; strict downhill
  acceptance, uphill with the ratio's denominator at least 1e-12 when T > 0
  (:289-296); the per-warp best score (:299-301).

The reference's GPU kernels cannot run on this host, and their RNG is
cuRAND; both restatements are driven by the Philox proposal stream the
kernels of this library draw from.  The Python loop also feeds a trace to
the oracle's replay, whose schedule bookkeeping must stop at the same move.
"""
import math

import numpy as np

from oracle import oracle as O
from pmmc_gb300 import synth

F32 = np.float32


def _u01(x):
    return F32(x >> 8) * F32(1.0 / 16777216.0)


def _draws(seed, chain, move, movable, step, use2d=False, smooth=False):
    """The kernels' draws of a move: block tag 0 gives the bead (high word of
    x * n_movable) and the displacement; the Metropolis uniform is block tag
    1's first word, or for smoothing the low word of x * n_movable."""
    key = (seed & 0xFFFFFFFF, seed >> 32)
    o = O.philox((move & 0xFFFFFFFF, move >> 32, chain, 0), key)
    prod = int(o[0]) * len(movable)
    b = movable[prod >> 32]
    d = np.array([(F32(2.0) * _u01(int(o[k])) - F32(1.0)) * F32(step) for k in (1, 2, 3)],
                 np.float32)
    if use2d:
        d[2] = 0.0
    if smooth:
        return b, d, _u01(prod & 0xFFFFFFFF)
    a = O.philox((move & 0xFFFFFFFF, move >> 32, chain, 1), key)
    return b, d, _u01(int(a[0]))


def _roundup256(k):
    return (k + 255) // 256 * 256 if k > 0 else 0


def py_arcs_gpu_schedule(pr, prm, step, seed, chain):
    movable = [i for i in range(pr.n) if pr.fixed is None or not pr.fixed[i]]
    pos = pr.pos.astype(np.float32).copy()
    E = O.arcs_full(pr, prm, pos=pos)
    T = float(F32(prm.max_temp))
    dt = float(F32(prm.dt_temp))
    impr = float(F32(prm.improvement))
    cap = _roundup256(prm.milestone_steps)
    E_ms, succ, misses, moves, acc = E, 0, 0, 0, 0
    trace = []
    while moves < cap:
        for _ in range(256):
            b, d, u = _draws(seed, chain, moves, movable, step)
            before = O.arcs_local(pr, prm, b, pos=pos)
            q = pos.copy()
            q[b] += d
            after = O.arcs_local(pr, prm, b, pos=q)
            En = E - before + after
            ok = En <= E
            if not ok and T > 0.0 and E > 0.0:
                tp = float(F32(prm.jump_scale)) * math.exp(
                    -float(F32(prm.jump_coef)) * (En / E) / T)
                ok = u < F32(tp)
            trace.append((b, int(ok), d))
            if ok:
                pos, E = q, En
                succ += 1
                acc += 1
            moves += 1
            T *= dt
        miss = ((E > impr * E_ms and succ < prm.min_successes) or E < 1e-5
                or (E_ms > 1e-10 and E / E_ms > 0.9999))
        misses = misses + 1 if miss else 0
        if misses >= prm.milestone_fails or E < 1e-5:
            break
        E_ms, succ = E, 0
    return pos, moves, acc, E, trace


def py_smooth_gpu_schedule(pr, prm, step, seed, chain):
    movable = [i for i in range(pr.n) if pr.fixed is None or not pr.fixed[i]]
    pos = pr.pos.astype(np.float32).copy()
    E = O.smooth_full(pr, prm, pos=pos)
    best = E
    T = float(F32(prm.max_temp))
    dt = float(F32(prm.dt_temp))
    cap = _roundup256(prm.milestone_steps)
    moves, acc = 0, 0
    trace = []
    while moves < cap:
        for _ in range(256):
            b, d, u = _draws(seed, chain, moves, movable, step, smooth=True)
            before = O.smooth_local(pr, prm, b, pos=pos)
            q = pos.copy()
            q[b] += d
            after = O.smooth_local(pr, prm, b, pos=q)
            En = E - before + after
            ok = En < E
            if not ok and T > 0.0:
                tp = float(F32(prm.jump_scale)) * math.exp(
                    -float(F32(prm.jump_coef)) * (En / max(E, 1e-12)) / T)
                ok = u < F32(tp)
            trace.append((b, int(ok), d))
            if ok:
                pos, E = q, En
                acc += 1
                best = min(best, E)
            moves += 1
            T *= dt
    return pos, moves, acc, E, best, trace


def _as_trace(rows):
    tr = np.zeros(len(rows), [("bead", "<i4"), ("accepted", "<i4"), ("before", "<f4"),
                              ("after", "<f4"), ("dx", "<f4"), ("dy", "<f4"), ("dz", "<f4"),
                              ("pad", "<f4")])
    for k, (b, ok, d) in enumerate(rows):
        tr[k]["bead"], tr[k]["accepted"] = b, ok
        tr[k]["dx"], tr[k]["dy"], tr[k]["dz"] = d
    return tr


def test_arcs_gpu_schedule_restatements_agree():
    for n, arcs, fails, steps, seed in [(40, 60, 3, 20000, 5), (48, 70, 1, 20000, 6),
                                        (40, 60, 1000, 3000, 7), (32, 40, 0, 20000, 8)]:
        r = synth.arcs_region(n, arcs, seed=seed)
        fixed = np.zeros(n, np.uint8)
        fixed[::6] = 1
        pr = O.ArcsProblem(r.pos, r.dense(), fixed)
        prm = O.Params(max_temp=5.0, dt_temp=0.9999, milestone_steps=steps, improvement=0.99,
                       schedule=O.SCHEDULE_GPU, milestone_fails=fails)
        pos, moves, acc, E, rows = py_arcs_gpu_schedule(pr, prm, 0.5, 900 + seed, 2)
        opos, ores = O.arcs_anneal(pr, prm, 0.5, 900 + seed, rng=O.RNG_PHILOX, chain=2)
        assert ores.moves == moves and ores.accepted == acc, (n, ores.moves, moves)
        np.testing.assert_array_equal(opos, pos)
        assert ores.score == E
        assert moves % 256 == 0 and moves <= _roundup256(steps)
        if fails <= 0:
            assert moves == 256
        if fails >= 1000:
            assert moves == _roundup256(steps)
        rep = O.arcs_replay(pr, prm, 0.5, 900 + seed, 2, _as_trace(rows))
        assert rep["proposal_mismatch"] == 0
        assert rep["stop_at"] == moves
        assert (rep["orc_acc"] == np.array([x[1] for x in rows])).all()


def test_smooth_gpu_schedule_restatements_agree():
    for n, steps, seed in [(30, 1500, 3), (50, 700, 4), (20, 1, 5)]:
        c = synth.smooth_chain(n, seed=seed)
        pr = O.SmoothProblem(c.pos, c.dist_to_next, c.fixed)
        prm = O.Params(max_temp=5.0, dt_temp=0.9999, milestone_steps=steps, improvement=0.99,
                       k_stretch=0.1, k_squeeze=0.1, k_angle=0.1, schedule=O.SCHEDULE_GPU)
        pos, moves, acc, E, best, rows = py_smooth_gpu_schedule(pr, prm, 0.5, 40 + seed, 1)
        opos, ores = O.smooth_anneal(pr, prm, 0.5, 40 + seed, rng=O.RNG_PHILOX, chain=1)
        assert moves == _roundup256(steps)
        assert ores.moves == moves and ores.accepted == acc
        np.testing.assert_array_equal(opos, pos)
        assert ores.score == E and ores.best == best
        rep = O.smooth_replay(pr, prm, 0.5, 40 + seed, 1, _as_trace(rows))
        assert rep["proposal_mismatch"] == 0 and rep["stop_at"] == moves


def test_gpu_schedule_zero_steps_makes_no_move():
    r = synth.arcs_region(24, 30, seed=2)
    pr = O.ArcsProblem(r.pos, r.dense())
    _, res = O.arcs_anneal(pr, O.Params(milestone_steps=0, schedule=O.SCHEDULE_GPU), 0.5, 1,
                           rng=O.RNG_PHILOX)
    assert res.moves == 0
    c = synth.smooth_chain(20, seed=2)
    sp = O.SmoothProblem(c.pos, c.dist_to_next, c.fixed)
    _, res = O.smooth_anneal(sp, O.Params(milestone_steps=-5, schedule=O.SCHEDULE_GPU), 0.5, 1,
                             rng=O.RNG_PHILOX)
    assert res.moves == 0


def test_cpu_schedule_unchanged_by_the_new_fields():
    """The CPU schedule (the default) still stops at the first milestone miss
    and never consults milestone_fails."""
    r = synth.arcs_region(40, 60, seed=9)
    pr = O.ArcsProblem(r.pos, r.dense())
    a = O.arcs_anneal(pr, O.Params(max_temp=5.0, dt_temp=0.9999, milestone_steps=1000,
                                   improvement=0.99, milestone_fails=1), 0.5, 3)
    b = O.arcs_anneal(pr, O.Params(max_temp=5.0, dt_temp=0.9999, milestone_steps=1000,
                                   improvement=0.99, milestone_fails=50), 0.5, 3)
    assert a[1].moves == b[1].moves and a[1].moves % 1000 == 0
    np.testing.assert_array_equal(a[0], b[0])
