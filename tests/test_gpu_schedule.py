"""The reference kernels' stopping schedule (PMMC_SCHEDULE_GPU), the one the
drop-in calls run, against the oracle's restatement of it
(MonteCarloArcsKernel, ParallelMonteCarloArcs.cu:494-655;
MonteCarloSmoothKernelMultiWarp, ParallelMonteCarloSmooth.cu:258-337).

Every kernel move is replayed on the oracle: same Philox proposals, local
scores within 1e-5, decisions equal away from the Metropolis threshold, and
the move at which the oracle's schedule stops -- following the kernel's
decisions with its FP64 running energy -- equals the kernel's.  A stop may
differ only where a milestone comparison sat within 1e-6 of its threshold
(the kernel's running energy is a float-float pair, the oracle's a double).

One deliberate difference, kept in every form of this library: a proposal
draws its bead among the movable beads, where the reference kernels redraw
(at most 4n times at the arc level, n times when smoothing) until a free
bead comes up.  The proposal distribution is the same."""
import numpy as np
import pytest

from oracle import oracle as O
from pmmc_gb300 import capi, synth
from parity import check_replay

pytestmark = pytest.mark.gpu

STOP_TOL = 1e-6


def arcs_problem(n, arcs, seed, fixed_every=0, loops=False):
    r = synth.arcs_region(n, arcs, seed=seed)
    dense = r.dense()
    fixed = None
    if fixed_every:
        fixed = np.zeros(n, np.uint8)
        fixed[::fixed_every] = 1
    lp = None
    if loops:
        rng = np.random.default_rng(seed)
        lp = (rng.integers(0, n, 8).astype(np.int32), rng.integers(0, n, 8).astype(np.int32),
              rng.uniform(0.5, 2.0, 8).astype(np.float32),
              rng.uniform(1.0, 3.0, 8).astype(np.float32))
    pr = O.ArcsProblem(r.pos, dense, fixed, *(lp or ()))
    inp = capi.ArcsInput.from_dense(r.pos, dense, fixed, lp)
    return pr, inp


def roundup256(k):
    return (k + 255) // 256 * 256 if k > 0 else 0


def check_stop(moves, rep):
    assert rep["stop_at"] == moves or rep["stop_margin"] < STOP_TOL, \
        f"kernel stopped after {moves} moves, the oracle's schedule after {rep['stop_at']} " \
        f"(closest milestone comparison {rep['stop_margin']:.3g})"


@pytest.mark.parametrize("n,arcs,fails,steps,lanes,extra", [
    (96, 160, 3, 60000, 1, {}),          # stops by its milestone misses
    (96, 160, 2, 60000, 4, {}),
    (96, 160, 1, 60000, 2, {}),          # the first non-improving block stops it
    (128, 200, 3, 60000, 2, {"fixed_every": 5}),
    (96, 160, 3, 60000, 8, {"loops": True}),
    (96, 160, 1000, 5000, 1, {}),        # never misses enough: the cap, rounded up to 256
    (64, 100, 0, 60000, 1, {}),          # fails threshold 0: the first milestone stops it
])
def test_arcs_gpu_schedule_single_chain(ctx, n, arcs, fails, steps, lanes, extra):
    pr, inp = arcs_problem(n, arcs, seed=n + fails, **extra)
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=steps, improvement=0.99,
                min_successes=5)
    prm = capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_GPU,
                              milestone_fails=fails, **base)
    oprm = O.Params(schedule=O.SCHEDULE_GPU, milestone_fails=fails, **base)
    seed = 4100 + n + fails
    ctx.set_seed(seed)
    cap = roundup256(steps)
    b = capi.ArcsBatch(ctx, [inp], prm, [0.5], use_graph=False, trace_cap=cap, lanes=lanes)
    b.run()
    pos, res = b.results()
    m = int(res[0].moves)
    assert 0 < m <= cap and (m % 256 == 0 or m == cap)
    if fails >= 1000:
        assert m == cap
    if fails <= 0:
        assert m == 256
    tr = b.trace(m)
    rep = O.arcs_replay(pr, oprm, 0.5, seed, 0, tr)
    _, mism = check_replay(tr, rep)
    check_stop(m, rep)
    # with every decision equal, the oracle's own annealer under the same
    # schedule walks the same chain and stops at the same move
    if mism == 0:
        opos, ores = O.arcs_anneal(pr, oprm, 0.5, seed, rng=O.RNG_PHILOX, chain=0)
        assert ores.moves == m and ores.accepted == res[0].accepted
        np.testing.assert_allclose(opos, pos[0], rtol=0, atol=1e-4)
    b.close()


def test_arcs_gpu_schedule_stop_all(ctx):
    """Several chains of one region with the shared stop flag (the drop-in
    call): the chain that stops by its own milestone rule ends the others at
    their next milestone.  Every chain's moves replay on the oracle; each
    chain stopped either where its own schedule says or, earlier, at a
    milestone; at least one stopped by its own rule; the reported chain has
    the lowest running energy."""
    pr, inp = arcs_problem(96, 160, seed=17)
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=60000, improvement=0.99,
                min_successes=5)
    prm = capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_GPU, milestone_fails=3,
                              **base)
    oprm = O.Params(schedule=O.SCHEDULE_GPU, milestone_fails=3, **base)
    chains, seed = 8, 5151
    ctx.set_seed(seed)
    b = capi.ArcsBatch(ctx, [inp], prm, [0.5], chains=chains, use_graph=False, stop_all=True,
                       trace_cap=roundup256(60000), lanes=1, drawing_warp=True)
    b.run()
    pos, res = b.results()
    cr = b.chain_results()
    assert len(cr) == chains
    own = 0
    for c, r in enumerate(cr):
        m = int(r.moves)
        assert m > 0 and m % 256 == 0
        tr = b.trace(m, chain=c)
        rep = O.arcs_replay(pr, oprm, 0.5, seed, c, tr)
        check_replay(tr, rep)
        if rep["stop_at"] == m:
            own += 1
        else:   # ended by the flag: before its own stop, at a milestone
            assert rep["stop_at"] == -1 or rep["stop_at"] > m or rep["stop_margin"] < STOP_TOL
    assert own >= 1
    energies = [r.energy for r in cr]
    assert res[0].best_chain == int(np.argmin(energies))
    assert res[0].moves == cr[res[0].best_chain].moves
    assert res[0].total_moves == sum(r.moves for r in cr)
    b.close()


def test_arcs_dropin_call_runs_the_gpu_schedule(ctx):
    """pmmc_arcs_anneal with the default parameters (the schedule the shim
    passes): every chain's move count is a whole number of 256-move blocks
    and at most the cap."""
    pr, inp = arcs_problem(256, 400, seed=42)
    prm = capi.default_params(capi.LEVEL_ARCS, max_temp=5.0, dt_temp=0.9999,
                              milestone_steps=50000, improvement=0.99)
    assert prm.schedule == capi.SCHEDULE_GPU
    pos, res = capi.arcs_anneal(ctx, inp, prm, 0.5, 16)
    assert res.moves % 256 == 0 and 0 < res.moves <= roundup256(50000)
    assert res.total_moves % 256 == 0


def test_arcs_gpu_schedule_zero_cap_makes_no_move(ctx):
    """stop_condition_steps <= 0: the reference kernel's loop never runs."""
    pr, inp = arcs_problem(64, 100, seed=3)
    prm = capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_GPU, milestone_steps=0)
    pos, res = capi.arcs_anneal(ctx, inp, prm, 0.5, 4)
    assert res.moves == 0 and res.total_moves == 0
    np.testing.assert_array_equal(pos, pr.pos)
    oprm = O.Params(schedule=O.SCHEDULE_GPU, milestone_steps=0)
    _, ores = O.arcs_anneal(pr, oprm, 0.5, 1, rng=O.RNG_PHILOX)
    assert ores.moves == 0


@pytest.mark.parametrize("n,steps,w", [(40, 3000, (1.0, 1.0)), (150, 5000, (1.0, 1.0)),
                                       (90, 2000, (0.7, 1.3)), (60, 100, (1.0, 1.0))])
def test_smooth_gpu_schedule_trace(ctx, n, steps, w):
    """The smoothing kernel's schedule: exactly stop_condition_steps rounded
    up to 256 moves, whatever the energy does."""
    c = synth.smooth_chain(n, seed=n)
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=steps, improvement=0.99,
                k_stretch=0.1, k_squeeze=0.1, k_angle=0.1, w_dist=w[0], w_angle=w[1])
    prm = capi.default_params(capi.LEVEL_SMOOTH, schedule=capi.SCHEDULE_GPU, **base)
    oprm = O.Params(schedule=O.SCHEDULE_GPU, **base)
    ctx.set_seed(61)
    inp = capi.SmoothInput(c.pos, c.dist_to_next, c.fixed)
    cap = roundup256(steps)
    out, res, ms, tr = capi.smooth_batch_anneal(ctx, [inp], prm, [0.5], chains=1, trace_cap=cap)
    assert int(res[0].moves) == cap
    pr = O.SmoothProblem(c.pos, c.dist_to_next, c.fixed)
    rep = O.smooth_replay(pr, oprm, 0.5, 61, 0, tr[:cap])
    _, mism = check_replay(tr[:cap], rep)
    assert rep["stop_at"] == cap
    if mism == 0:
        opos, ores = O.smooth_anneal(pr, oprm, 0.5, 61, rng=O.RNG_PHILOX, chain=0)
        assert ores.moves == cap and ores.accepted == res[0].accepted
        np.testing.assert_allclose(opos, out[0], rtol=0, atol=1e-4)


def test_smooth_gpu_schedule_reports_lowest_reached_chain(ctx):
    """Several chains: the reference's host keeps the warp whose running
    score reached the lowest value during the run (ties to the lower index),
    not the lowest final score."""
    c = synth.smooth_chain(80, seed=23)
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=4000, improvement=0.99,
                k_stretch=0.1, k_squeeze=0.1, k_angle=0.1)
    prm = capi.default_params(capi.LEVEL_SMOOTH, schedule=capi.SCHEDULE_GPU, **base)
    oprm = O.Params(schedule=O.SCHEDULE_GPU, **base)
    chains = 12
    ctx.set_seed(707)
    pos, res = capi.smooth_anneal(ctx, capi.SmoothInput(c.pos, c.dist_to_next, c.fixed), prm,
                                  0.5, chains)
    pr = O.SmoothProblem(c.pos, c.dist_to_next, c.fixed)
    outs = [O.smooth_anneal(pr, oprm, 0.5, 707, rng=O.RNG_PHILOX, chain=k) for k in range(chains)]
    bests = np.array([o[1].best for o in outs])
    k = int(np.argmin(bests))
    assert res.moves == roundup256(4000) and res.total_moves == chains * roundup256(4000)
    near = np.abs(bests - bests[k]) <= 1e-9 * abs(bests[k])
    assert near[res.best_chain], (res.best_chain, k, bests)
    if near.sum() == 1:
        np.testing.assert_allclose(pos[c.fixed == 0], outs[k][0][c.fixed == 0], rtol=0,
                                   atol=1e-3)
    np.testing.assert_array_equal(pos[c.fixed == 1], c.pos[c.fixed == 1])
