"""Windowed smoothing kernel (W proposals per chain scored at once, resolved
in order) against the one-move-at-a-time kernel and the oracle, through the
C ABI.  The two kernels make the same draws and walk the decisions in the
same order with the same float-float running score, so their traces,
energies and positions must agree exactly."""
import numpy as np
import pytest

from oracle import oracle as O
from pmmc_gb300 import capi, synth
from parity import check_replay

pytestmark = pytest.mark.gpu

WINDOWS = (0, 4, 8, 16, 32)


@pytest.fixture
def wctx(ctx):
    yield ctx
    ctx.set_smooth_window(8, 32, 20)   # the default


def _genome_segments(beads, seed):
    segs, probs = [], []
    for ch in synth.smooth_genome(beads, seed=seed):
        a = np.nonzero(ch.fixed)[0]
        for l, r in zip(a[:-1], a[1:]):
            if r - l >= 2:
                sl = slice(l, r + 1)
                segs.append(capi.SmoothInput(ch.pos[sl], ch.dist_to_next[sl], ch.fixed[sl]))
                probs.append(O.SmoothProblem(ch.pos[sl], ch.dist_to_next[sl], ch.fixed[sl]))
    return segs, probs


def _run(ctx, window, window_long, long_min_free, inputs, prm, steps, seed, **kw):
    ctx.set_smooth_window(window, window_long, long_min_free)
    ctx.set_seed(seed)
    return capi.smooth_batch_anneal(ctx, inputs, prm, steps, **kw)


def _same(a, b):
    (pa, ra) = a[0], a[1]
    (pb, rb) = b[0], b[1]
    for x, y in zip(pa, pb):
        np.testing.assert_array_equal(x, y)
    for x, y in zip(ra, rb):
        assert (x.moves, x.accepted, x.best_chain, x.status) == \
            (y.moves, y.accepted, y.best_chain, y.status)
        assert x.energy == y.energy and x.energy_fp64 == y.energy_fp64 and x.score == y.score


@pytest.mark.parametrize("window", WINDOWS)
def test_window_trace_parity(wctx, window):
    """Chain 0's move records replayed by the oracle, for every window size
    (0 = two lanes per chain, one move at a time)."""
    c = synth.smooth_chain(90, seed=90)
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=2000, improvement=0.99,
                k_stretch=0.1, k_squeeze=0.1, k_angle=0.1, sphere_radius=9.0)
    prm = capi.default_params(capi.LEVEL_SMOOTH, schedule=capi.SCHEDULE_CPU, max_moves=8000,
                              **base)
    inp = capi.SmoothInput(c.pos, c.dist_to_next, c.fixed)
    out, res, ms, tr = _run(wctx, window, window, 0, [inp], prm, [0.5], 31, chains=1,
                            trace_cap=8000)
    m = int(res[0].moves)
    assert m > 0
    pr = O.SmoothProblem(c.pos, c.dist_to_next, c.fixed)
    rep = O.smooth_replay(pr, O.Params(**base), 0.5, 31, 0, tr[:m])
    check_replay(tr[:m], rep)
    e64 = O.smooth_full(pr, O.Params(**base), pos=out[0])
    assert abs(res[0].energy_fp64 - e64) <= 1e-6 * abs(e64)


def test_window_trace_identical_to_one_move_kernel(wctx):
    c = synth.smooth_chain(150, seed=150)
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=2000, improvement=0.99,
                k_stretch=0.1, k_squeeze=0.1, k_angle=0.1, sphere_radius=9.0)
    prm = capi.default_params(capi.LEVEL_SMOOTH, schedule=capi.SCHEDULE_CPU, max_moves=20000,
                              resync_every=1000, **base)
    inp = capi.SmoothInput(c.pos, c.dist_to_next, c.fixed)
    ref = _run(wctx, 0, 0, 0, [inp], prm, [0.5], 7, chains=3, trace_cap=20000)
    for w in (4, 8, 16, 32):
        got = _run(wctx, w, w, 0, [inp], prm, [0.5], 7, chains=3, trace_cap=20000)
        _same(ref, got)
        m = int(ref[1][0].moves)
        for f in ("bead", "accepted", "before", "after", "dx", "dy", "dz"):
            np.testing.assert_array_equal(ref[3][f][:m], got[3][f][:m], err_msg=f"{w} {f}")


@pytest.mark.parametrize("window,window_long,long_min_free",
                         [(8, 8, 0), (4, 4, 0), (16, 16, 0), (8, 16, 10), (0, 8, 10),
                          (8, 0, 12), (4, 32, 6)])
def test_window_genome_segments_identical(wctx, window, window_long, long_min_free):
    """Genome-smoothing regions (sweeps of each region's free beads, FP64
    resync every 1000 moves), all windowed or split between kernels running
    side by side: the same result region by region."""
    segs, probs = _genome_segments(6000, 3)
    prm = capi.default_params(capi.LEVEL_SMOOTH, schedule=capi.SCHEDULE_CPU, max_temp=5.0,
                              dt_temp=0.9999, milestone_steps=10**9, improvement=0.99,
                              max_moves=-200, resync_every=1000)
    steps = [0.5] * len(segs)
    ref = _run(wctx, 0, 0, 0, segs, prm, steps, 3)
    got = _run(wctx, window, window_long, long_min_free, segs, prm, steps, 3)
    _same(ref, got)
    for u in range(0, len(segs), max(1, len(segs) // 8)):
        free = int((segs[u].fixed == 0).sum())
        assert got[1][u].moves == 200 * free


def test_window_gpu_schedule_identical(wctx):
    """The reference kernel's schedule (fixed cap, lowest score reached
    picks the chain): windowed and one-move kernels agree."""
    c = synth.smooth_chain(80, seed=23)
    prm = capi.default_params(capi.LEVEL_SMOOTH, schedule=capi.SCHEDULE_GPU, max_temp=5.0,
                              dt_temp=0.9999, milestone_steps=3000, improvement=0.99)
    inp = capi.SmoothInput(c.pos, c.dist_to_next, c.fixed)
    ref = _run(wctx, 0, 0, 0, [inp], prm, [0.5], 11, chains=8)
    got = _run(wctx, 8, 8, 0, [inp], prm, [0.5], 11, chains=8)
    _same(ref, got)
    assert ref[1][0].moves == 3072


def test_window_rejects_bad_size(wctx):
    with pytest.raises(RuntimeError):
        wctx.set_smooth_window(6)
    with pytest.raises(RuntimeError):
        wctx.set_smooth_window(8, 12)
    with pytest.raises(RuntimeError):
        wctx.set_smooth_window(8, 16, -1)


def test_packed_batch_matches_list_form(wctx):
    """pmmc_smooth_batch_anneal_packed (regions back to back in one set of
    arrays) gives the list form's results."""
    segs, _ = _genome_segments(3000, 5)
    prm = capi.default_params(capi.LEVEL_SMOOTH, schedule=capi.SCHEDULE_CPU, max_temp=5.0,
                              dt_temp=0.9999, milestone_steps=10**9, improvement=0.99,
                              max_moves=-100, resync_every=1000)
    steps = [0.5] * len(segs)
    ref = _run(wctx, 8, 32, 20, segs, prm, steps, 9)
    off = np.zeros(len(segs) + 1, np.int64)
    off[1:] = np.cumsum([s.n for s in segs])
    wctx.set_seed(9)
    pos, res, ms = capi.smooth_batch_anneal_packed(
        wctx, off, np.concatenate([s.pos for s in segs]), np.concatenate([s.dtn for s in segs]),
        np.concatenate([s.fixed for s in segs]), prm, steps)
    for u, s in enumerate(segs):
        np.testing.assert_array_equal(pos[off[u]:off[u + 1]], ref[0][u])
        assert res[u].energy == ref[1][u].energy and res[u].moves == ref[1][u].moves
