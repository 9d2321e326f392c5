"""Subanchor smoothing on the GPU against the oracle, through the C ABI."""
import numpy as np
import pytest

from oracle import oracle as O
from pmmc_gb300 import capi, synth
from parity import check_replay, ks_2samp_p

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,sphere,w", [(40, 0.0, (1.0, 1.0)), (150, 9.0, (1.0, 1.0)),
                                        (90, 0.0, (0.7, 1.3))])
def test_smooth_trace_parity(ctx, n, sphere, w):
    c = synth.smooth_chain(n, seed=n)
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=2000, improvement=0.99,
                k_stretch=0.1, k_squeeze=0.1, k_angle=0.1, sphere_radius=sphere,
                w_dist=w[0], w_angle=w[1])
    prm = capi.default_params(capi.LEVEL_SMOOTH, schedule=capi.SCHEDULE_CPU, max_moves=8000, **base)
    ctx.set_seed(31)
    inp = capi.SmoothInput(c.pos, c.dist_to_next, c.fixed)
    out, res, ms, tr = capi.smooth_batch_anneal(ctx, [inp], prm, [0.5], chains=1, trace_cap=8000)
    m = int(res[0].moves)
    pr = O.SmoothProblem(c.pos, c.dist_to_next, c.fixed)
    rep = O.smooth_replay(pr, O.Params(**base), 0.5, 31, 0, tr[:m])
    check_replay(tr[:m], rep)
    np.testing.assert_array_equal(out[0][c.fixed == 1], c.pos[c.fixed == 1])
    if w == (1.0, 1.0):   # the running score is a function of state
        e64 = O.smooth_full(pr, O.Params(**base), pos=out[0])
        assert abs(res[0].energy_fp64 - e64) <= 1e-6 * abs(e64)
        assert abs(res[0].energy - e64) <= 1e-4 * abs(e64)


def test_smooth_segments_batch(ctx):
    chains = synth.smooth_genome(3000, seed=3)
    segs, probs = [], []
    for ch in chains:
        a = np.nonzero(ch.fixed)[0]
        for l, r in zip(a[:-1], a[1:]):
            if r - l >= 2:
                sl = slice(l, r + 1)
                segs.append(capi.SmoothInput(ch.pos[sl], ch.dist_to_next[sl], ch.fixed[sl]))
                probs.append(O.SmoothProblem(ch.pos[sl], ch.dist_to_next[sl], ch.fixed[sl]))
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=500, improvement=0.99,
                k_stretch=0.1, k_squeeze=0.1, k_angle=0.1)
    prm = capi.default_params(capi.LEVEL_SMOOTH, schedule=capi.SCHEDULE_CPU, max_moves=1500, **base)
    ctx.set_seed(5)
    out, res, ms = capi.smooth_batch_anneal(ctx, segs, prm, [0.5] * len(segs))
    assert ms > 0
    for u in range(0, len(segs), max(1, len(segs) // 12)):
        opos, ores = O.smooth_anneal(probs[u], O.Params(max_moves=1500, **base), 0.5, 5,
                                     rng=O.RNG_PHILOX, chain=u)
        assert abs(ores.score - res[u].energy) <= 1e-4 * max(abs(ores.score), 1e-6)
        assert np.isfinite(out[u]).all()


def test_smooth_dropin_keeps_fixed_beads(ctx):
    c = synth.smooth_chain(300, seed=9)
    prm = capi.default_params(capi.LEVEL_SMOOTH, max_temp=5.0, dt_temp=0.9999,
                              milestone_steps=2000, improvement=0.99)
    pos, res = capi.smooth_anneal(ctx, capi.SmoothInput(c.pos, c.dist_to_next, c.fixed), prm, 0.5)
    np.testing.assert_array_equal(pos[c.fixed == 1], c.pos[c.fixed == 1])
    assert res.total_moves >= res.moves > 0 and res.best_chain >= 0


def test_smooth_statistics_match_reference(ctx):
    c = synth.smooth_chain(60, seed=12)
    pr = O.SmoothProblem(c.pos, c.dist_to_next, c.fixed)
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=800, improvement=0.99,
                k_stretch=0.1, k_squeeze=0.1, k_angle=0.1)
    ref_e = [O.smooth_anneal(pr, O.Params(**base), 0.5, 700 + s)[1].score for s in range(16)]
    prm = capi.default_params(capi.LEVEL_SMOOTH, schedule=capi.SCHEDULE_CPU, **base)
    ctx.set_seed(77)
    inputs = [capi.SmoothInput(c.pos, c.dist_to_next, c.fixed) for _ in range(16)]
    out, res, ms = capi.smooth_batch_anneal(ctx, inputs, prm, [0.5] * 16)
    assert ks_2samp_p(ref_e, [r.energy for r in res]) > 0.05


def test_smooth_sweeps_cap_per_region(ctx):
    """max_moves < 0: every region anneals -max_moves sweeps of its own
    movable beads, all regions in one launch."""
    chains = [synth.smooth_chain(n, seed=40 + n) for n in (12, 30, 7, 55)]
    inputs = [capi.SmoothInput(c.pos, c.dist_to_next, c.fixed) for c in chains]
    prm = capi.default_params(capi.LEVEL_SMOOTH, max_temp=5.0, dt_temp=0.9999,
                              milestone_steps=10**9, improvement=0.99,
                              schedule=capi.SCHEDULE_CPU, max_moves=-50)
    out, res, ms = capi.smooth_batch_anneal(ctx, inputs, prm, [0.5] * len(inputs))
    for c, r in zip(chains, res):
        assert r.moves == 50 * int((c.fixed == 0).sum())
        assert r.rel_error < 1e-4   # FP32 deltas, no periodic recompute here


def test_smooth_structures_match_reference(ctx):
    """16 seeds on a 400-bead chromosome stretch with anchors every
    Poisson(10) beads held fixed (the genome-smoothing shape): final energy,
    RMSD to the start and distance-map Pearson against the start, GPU vs the
    reference's CPU MonteCarloArcsSmooth (the oracle in libc mode, bit-
    identical to it).  Two-sample KS and Welch tests, p > 0.01 each."""
    from parity import distmap_pearson, kabsch_rmsd, welch_p
    c = synth.smooth_chain(400, seed=31)
    pr = O.SmoothProblem(c.pos, c.dist_to_next, c.fixed)
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=4000, improvement=0.99,
                k_stretch=0.1, k_squeeze=0.1, k_angle=0.1)
    cap = 40_000
    outs = [O.smooth_anneal(pr, O.Params(max_moves=cap, **base), 0.5, 800 + s)
            for s in range(16)]
    prm = capi.default_params(capi.LEVEL_SMOOTH, schedule=capi.SCHEDULE_CPU, max_moves=cap,
                              **base)
    ctx.set_seed(8080)
    inp = capi.SmoothInput(c.pos, c.dist_to_next, c.fixed)
    gpos, gres, _ = capi.smooth_batch_anneal(ctx, [inp] * 16, prm, [0.5] * 16)
    ref_m = [[o[1].score for o in outs], [kabsch_rmsd(o[0], c.pos) for o in outs],
             [distmap_pearson(o[0], c.pos) for o in outs]]
    gpu_m = [[r.energy for r in gres], [kabsch_rmsd(p, c.pos) for p in gpos],
             [distmap_pearson(p, c.pos) for p in gpos]]
    for name, a, b in zip(("energy", "rmsd", "pearson"), ref_m, gpu_m):
        assert ks_2samp_p(a, b) > 0.01, name
        assert welch_p(a, b) > 0.01, name
