"""Heatmap-level annealing on the GPU against the oracle, through the C ABI."""
import numpy as np
import pytest

from oracle import oracle as O
from pmmc_gb300 import capi, synth
from parity import check_replay, ks_2samp_p

pytestmark = pytest.mark.gpu


@pytest.fixture
def hctx(ctx):
    yield ctx
    ctx.set_heatmap_cluster(0)   # the default: chosen by the batch


@pytest.mark.parametrize("cl", [0, 4, 8])
@pytest.mark.parametrize("n,diag,bounds,sphere", [(128, 1, [], 0.0), (200, 2, [0, 90, 200], 0.0),
                                                  (96, 1, [], 6.0)])
def test_heatmap_trace_parity(hctx, n, diag, bounds, sphere, cl):
    """cl: CTAs of the cluster that runs the chain (0 = the default, one
    CTA at these sizes); in a cluster each CTA scores a slice of every row."""
    ctx = hctx
    ctx.set_heatmap_cluster(cl)
    h = synth.heatmap_region(n, seed=n, n_tads=4, tad_min=10, tad_max=30)
    fixed = np.zeros(n, np.uint8)
    fixed[[0, n // 2]] = 1
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=3000, improvement=0.99,
                sphere_radius=sphere)
    prm = capi.default_params(capi.LEVEL_HEATMAP, schedule=capi.SCHEDULE_CPU, max_moves=6000, **base)
    ctx.set_seed(17)
    inp = capi.HeatmapInput(h.pos, h.heat, diag, np.array(bounds, np.int32), fixed)
    out, res, ms, tr = capi.heatmap_batch_anneal(ctx, [inp], prm, [1.0], trace_cap=6000)
    m = int(res[0].moves)
    pr = O.HeatmapProblem(h.pos, h.heat, diag, np.array(bounds, np.int32), fixed)
    rep = O.heatmap_replay(pr, O.Params(**base), 1.0, 17, 0, tr[:m])
    check_replay(tr[:m], rep, scale_factor=2.0, delta_only=True)
    e64 = O.heatmap_score(pr, -1, pos=out[0])
    if sphere > 0:
        e64 += float(np.sum(np.maximum(np.linalg.norm(out[0], axis=1) - sphere, 0) ** 2))
    assert abs(res[0].energy - e64) <= 1e-4 * e64
    if sphere == 0:
        assert abs(res[0].energy_fp64 - e64) <= 1e-6 * e64
    np.testing.assert_array_equal(out[0][fixed == 1], h.pos[fixed == 1])


def test_heatmap_batch_distinct_maps(ctx):
    hs = [synth.heatmap_region(256, seed=s, n_tads=5, tad_min=10, tad_max=40) for s in range(4)]
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=2000, improvement=0.99)
    prm = capi.default_params(capi.LEVEL_HEATMAP, schedule=capi.SCHEDULE_CPU, max_moves=4000, **base)
    ctx.set_seed(3)
    out, res, ms, _ = capi.heatmap_batch_anneal(ctx, [capi.HeatmapInput(h.pos, h.heat) for h in hs],
                                                prm, [1.0] * 4)
    for u, h in enumerate(hs):
        pr = O.HeatmapProblem(h.pos, h.heat)
        opos, ores = O.heatmap_anneal(pr, O.Params(max_moves=4000, **base), 1.0, 3,
                                      rng=O.RNG_PHILOX, incremental=True, chain=u)
        assert abs(ores.score - res[u].energy) <= 1e-3 * ores.score


def test_heatmap_statistics_match_reference(ctx):
    h = synth.heatmap_region(48, seed=5, n_tads=2, tad_min=6, tad_max=10)
    pr = O.HeatmapProblem(h.pos, h.heat)
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=600, improvement=0.99)
    ref_e = [O.heatmap_anneal(pr, O.Params(**base), 1.0, 900 + s)[1].score for s in range(16)]
    prm = capi.default_params(capi.LEVEL_HEATMAP, schedule=capi.SCHEDULE_CPU, **base)
    ctx.set_seed(55)
    out, res, ms, _ = capi.heatmap_batch_anneal(ctx, [capi.HeatmapInput(h.pos, h.heat)] * 16,
                                                prm, [1.0] * 16)
    assert ks_2samp_p(ref_e, [r.energy for r in res]) > 0.05


def test_heatmap_two_chains_per_sm(ctx):
    """With at least two chains per SM the batch runs two 256-thread CTAs per
    SM; chains still follow the oracle (trace of chain 0, energies of a
    sample of the others)."""
    n_units = 2 * ctx.sm_count + 3
    hs = [synth.heatmap_region(96 + (u % 5) * 8, seed=1000 + u, n_tads=3, tad_min=8, tad_max=20)
          for u in range(n_units)]
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=1500, improvement=0.99)
    prm = capi.default_params(capi.LEVEL_HEATMAP, schedule=capi.SCHEDULE_CPU, max_moves=1500, **base)
    ctx.set_seed(21)
    out, res, ms, tr = capi.heatmap_batch_anneal(
        ctx, [capi.HeatmapInput(h.pos, h.heat) for h in hs], prm, [1.0] * n_units, trace_cap=1500)
    m = int(res[0].moves)
    pr0 = O.HeatmapProblem(hs[0].pos, hs[0].heat)
    rep = O.heatmap_replay(pr0, O.Params(**base), 1.0, 21, 0, tr[:m])
    check_replay(tr[:m], rep, scale_factor=2.0, delta_only=True)
    for u in range(0, n_units, 37):
        pr = O.HeatmapProblem(hs[u].pos, hs[u].heat)
        opos, ores = O.heatmap_anneal(pr, O.Params(max_moves=1500, **base), 1.0, 21,
                                      rng=O.RNG_PHILOX, incremental=True, chain=u)
        assert abs(ores.score - res[u].energy) <= 1e-3 * ores.score
        assert res[u].rel_error < 1e-6 and res[u].status == 0


def test_heatmap_refuses_asymmetric_map(ctx):
    """A move changes the full score by twice its local change only on a
    symmetric map (createDistanceHeatmap mirrors it): an asymmetric pair
    that the score reads is refused; pairs it never reads (the diagonal band,
    across chromosome blocks) may differ."""
    h = synth.heatmap_region(64, seed=3, n_tads=2, tad_min=6, tad_max=10)
    prm = capi.default_params(capi.LEVEL_HEATMAP, schedule=capi.SCHEDULE_CPU, max_moves=500,
                              max_temp=5.0, dt_temp=0.9999, milestone_steps=250)
    assert (h.heat == h.heat.T).all()
    bad_value = h.heat.copy()
    bad_value[3, 40] *= 1.5
    bad_skip = h.heat.copy()
    bad_skip[50, 5] = 0.0           # one side skipped (< 1e-6), the other not
    for heat, pair in ((bad_value, "(3, 40)"), (bad_skip, "(5, 50)")):
        with pytest.raises(capi.PmmcError) as e:
            capi.heatmap_anneal(ctx, capi.HeatmapInput(h.pos, heat), prm, 1.0)
        assert e.value.status == capi.PMMC_ERR_INVALID
        assert "not symmetric" in str(e.value) and pair in str(e.value)
    # in a batch: the region named is the asymmetric one; its lowest pair
    both = bad_value.copy()
    both[50, 5] = 0.0
    good = capi.HeatmapInput(h.pos, h.heat)
    with pytest.raises(capi.PmmcError) as e:
        capi.heatmap_batch_anneal(ctx, [good, good, capi.HeatmapInput(h.pos, both)], prm,
                                  [1.0] * 3)
    assert "region 2" in str(e.value) and "(3, 40)" in str(e.value)
    unread = h.heat.copy()
    unread[7, 8] = 9.0              # inside a diagonal band of width 2
    unread[3, 40] *= 1.5            # across the block boundary at 32
    pos, res = capi.heatmap_anneal(
        ctx, capi.HeatmapInput(h.pos, unread, 2, np.array([0, 32, 64], np.int32)), prm, 1.0)
    assert res.moves == 500 and np.isfinite(pos).all()


def _config1_region():
    # the 2048-bead heatmap workload: c_ij = |i-j|^-1 x lognormal(0.5), 20 TAD
    # blocks x3, expected distance c^-1/3, seed 7
    return synth.heatmap_region(2048, seed=7)


@pytest.mark.parametrize("cl", [0, 1, 8])
def test_heatmap_trace_parity_config1(hctx, cl):
    """Per-move parity on the 2048-bead map, one chain: the launch the
    single-chain workload takes (cl = 0: a cluster of 16 CTAs, each scoring
    128 beads of every row), one CTA of 512 threads with a 16-row ring, and
    a cluster of 8 CTAs."""
    ctx = hctx
    ctx.set_heatmap_cluster(cl)
    h = _config1_region()
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=100_000, improvement=0.99)
    moves = 20_000
    prm = capi.default_params(capi.LEVEL_HEATMAP, schedule=capi.SCHEDULE_CPU, max_moves=moves,
                              **base)
    ctx.set_seed(7)
    out, res, ms, tr = capi.heatmap_batch_anneal(ctx, [capi.HeatmapInput(h.pos, h.heat)], prm,
                                                 [1.0], trace_cap=moves)
    m = int(res[0].moves)
    assert m == moves and res[0].status == 0
    pr = O.HeatmapProblem(h.pos, h.heat)
    rep = O.heatmap_replay(pr, O.Params(**base), 1.0, 7, 0, tr[:m])
    check_replay(tr[:m], rep, scale_factor=2.0, delta_only=True)
    e64 = O.heatmap_score(pr, -1, pos=out[0])
    assert abs(res[0].energy_fp64 - e64) <= 1e-6 * e64
    assert abs(res[0].energy - e64) <= 1e-5 * e64
    assert abs(rep["final_energy"] - res[0].energy) <= 1e-5 * abs(res[0].energy)


def test_heatmap_two_chains_per_sm_config1(ctx):
    """The batch form at 2048 beads with two chains per SM (two 256-thread
    CTAs share an SM, 8-row rings): chain 0's moves replay on the oracle and
    a sample of the other chains ends where the oracle's annealer ends."""
    h = _config1_region()
    n_units = 2 * ctx.sm_count
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=100_000, improvement=0.99)
    moves = 3000
    prm = capi.default_params(capi.LEVEL_HEATMAP, schedule=capi.SCHEDULE_CPU, max_moves=moves,
                              **base)
    inp = capi.HeatmapInput(h.pos, h.heat)
    ctx.set_seed(19)
    out, res, ms, tr = capi.heatmap_batch_anneal(ctx, [inp] * n_units, prm, [1.0] * n_units,
                                                 trace_cap=moves)
    pr = O.HeatmapProblem(h.pos, h.heat)
    rep = O.heatmap_replay(pr, O.Params(**base), 1.0, 19, 0, tr[:moves])
    check_replay(tr[:moves], rep, scale_factor=2.0, delta_only=True)
    for u in range(0, n_units, 29):
        opos, ores = O.heatmap_anneal(pr, O.Params(max_moves=moves, **base), 1.0, 19,
                                      rng=O.RNG_PHILOX, incremental=True, chain=u)
        assert res[u].moves == moves and res[u].status == 0
        assert abs(ores.score - res[u].energy) <= 1e-4 * ores.score
        assert res[u].rel_error < 1e-6


def test_heatmap_structures_match_reference_config1(ctx):
    """16 seeds on the 2048-bead map: final energy, RMSD to the start and
    distance-map Pearson against the start, GPU vs the reference's CPU
    annealer (MonteCarloHeatmap: the oracle in libc mode with local scores,
    which anneals exactly as the reference's full re-score).  Two-sample KS
    and Welch tests, p > 0.01 each."""
    from concurrent.futures import ThreadPoolExecutor
    from parity import distmap_pearson, kabsch_rmsd, welch_p
    h = _config1_region()
    pr = O.HeatmapProblem(h.pos, h.heat)
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=5000, improvement=0.99)
    cap = 20_000

    def ref(s):   # ctypes releases the GIL: the seeds run on all host cores
        return O.heatmap_anneal(pr, O.Params(max_moves=cap, **base), 1.0, 300 + s,
                                incremental=True)

    with ThreadPoolExecutor(16) as ex:
        outs = list(ex.map(ref, range(16)))
    prm = capi.default_params(capi.LEVEL_HEATMAP, schedule=capi.SCHEDULE_CPU, max_moves=cap,
                              **base)
    ctx.set_seed(3030)
    gpos, gres, _, _ = capi.heatmap_batch_anneal(ctx, [capi.HeatmapInput(h.pos, h.heat)] * 16,
                                                 prm, [1.0] * 16)
    ref_m = [[o[1].score for o in outs], [kabsch_rmsd(o[0], h.pos) for o in outs],
             [distmap_pearson(o[0], h.pos) for o in outs]]
    gpu_m = [[r.energy for r in gres], [kabsch_rmsd(p, h.pos) for p in gpos],
             [distmap_pearson(p, h.pos) for p in gpos]]
    for name, a, b in zip(("energy", "rmsd", "pearson"), ref_m, gpu_m):
        assert ks_2samp_p(a, b) > 0.01, name
        assert welch_p(a, b) > 0.01, name


def test_heatmap_cluster_rejects_bad_size(hctx):
    with pytest.raises(RuntimeError):
        hctx.set_heatmap_cluster(3)
    with pytest.raises(RuntimeError):
        hctx.set_heatmap_cluster(32)
