"""Arc-level annealing on the GPU against the oracle, through the C ABI."""
import numpy as np
import pytest

from oracle import oracle as O
from pmmc_gb300 import capi, synth
from parity import check_replay, distmap_pearson, kabsch_rmsd, ks_2samp_p

pytestmark = pytest.mark.gpu


def problem(variant, n=96, arcs=160, seed=3):
    r = synth.arcs_region(n, arcs, seed=seed)
    dense = r.dense()
    fixed = None
    loops = None
    kw = {}
    if variant == "loops_sphere":
        rng = np.random.default_rng(seed)
        li = rng.integers(0, n, 12).astype(np.int32)
        lj = rng.integers(0, n, 12).astype(np.int32)
        lk = rng.uniform(0.5, 2.0, 12).astype(np.float32)
        lr = rng.uniform(1.0, 3.0, 12).astype(np.float32)
        loops = (li, lj, lk, lr)
        kw["sphere_radius"] = 7.0
    if variant == "fixed":
        fixed = np.zeros(n, np.uint8)
        fixed[::7] = 1
    if variant == "2d":
        kw["use2d"] = 1
    if variant == "inert_pairs":   # listed pairs with 0 <= target < 1e-6
        dense[1, 5] = dense[5, 1] = 0.0
        dense[10, 40] = dense[40, 10] = 0.0
    if variant == "hub":           # a bead with more than 32 arcs
        for j in range(2, n, 2):
            dense[0, j] = dense[j, 0] = 1.0 + 0.01 * j
    pr = O.ArcsProblem(r.pos, dense, fixed, *(loops or ()))
    inp = capi.ArcsInput.from_dense(r.pos, dense, fixed, loops)
    return pr, inp, kw


@pytest.mark.parametrize("variant,lanes", [("plain", 4), ("loops_sphere", 4), ("fixed", 4),
                                           ("2d", 4), ("inert_pairs", 4), ("hub", 4),
                                           ("plain", 2), ("plain", 8), ("plain", 32),
                                           ("hub", 2), ("loops_sphere", 8), ("plain", 1),
                                           ("loops_sphere", 1), ("hub", 1), ("fixed", 1)])
def test_arcs_trace_parity(ctx, variant, lanes):
    """Windows of 32/lanes proposals resolve to the one-move-at-a-time chain."""
    pr, inp, kw = problem(variant)
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=4000, improvement=0.99, **kw)
    prm = capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_CPU, max_moves=12000, **base)
    ctx.set_seed(777)
    b = capi.ArcsBatch(ctx, [inp], prm, [0.5], use_graph=False, trace_cap=12000, lanes=lanes)
    b.run()
    pos, res = b.results()
    m = int(res[0].moves)
    tr = b.trace(m)
    rep = O.arcs_replay(pr, O.Params(**base), 0.5, 777, 0, tr)
    check_replay(tr, rep)
    # the oracle, following the kernel's decisions, lands on the same structure
    # and the same running energy
    assert abs(rep["final_energy"] - res[0].energy) <= 1e-5 * abs(rep["final_energy"])


@pytest.mark.parametrize("lanes", [1, 2, 8])
def test_arcs_extended_energy_trace_parity(ctx, lanes):
    """Opt-in extended energy (bonds to the next bead, target 1.0, k 0.1; the
    stiffness angle term, k 0.1): per-move local scores and decisions follow
    the oracle, and the FP64 energy is arcs + loops + bonds + angles."""
    pr, inp, _ = problem("plain", n=256, arcs=400, seed=42)
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=4000, improvement=0.99)
    ext = dict(arcs_extended=1, bond_target=1.0, k_stretch_bond=0.1, k_squeeze_bond=0.1,
               k_angle_ext=0.1)
    prm = capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_CPU, max_moves=12000,
                              resync_every=1000, **base, **ext)
    ctx.set_seed(31)
    b = capi.ArcsBatch(ctx, [inp], prm, [0.5], use_graph=False, trace_cap=12000, lanes=lanes)
    b.run()
    pos, res = b.results()
    m = int(res[0].moves)
    tr = b.trace(m)
    ox = O.Ext(1.0, 0.1, 0.1, 0.1)
    rep = O.arcs_replay(pr, O.Params(**base), 0.5, 31, 0, tr, ext=ox)
    check_replay(tr, rep)
    e64 = (O.arcs_repulsion(pr) + O.arcs_full(pr, O.Params(**base), pos=pos[0], repulsion=False)
           + O.arcs_ext_score(pr.n, pos[0], ox, -1))
    assert abs(res[0].energy_fp64 - e64) <= 1e-6 * e64
    assert abs(res[0].energy - e64) <= 1e-4 * e64


def test_arcs_fp64_energy_and_resync(ctx):
    pr, inp, _ = problem("plain", n=256, arcs=400, seed=42)
    oprm = O.Params(max_temp=5.0, dt_temp=0.9999, milestone_steps=50000, improvement=0.99)
    r0 = O.arcs_repulsion(pr)
    for resync in (0, 1000):
        prm = capi.default_params(capi.LEVEL_ARCS, max_temp=5.0, dt_temp=0.9999,
                                  milestone_steps=50000, improvement=0.99,
                                  schedule=capi.SCHEDULE_CPU, resync_every=resync)
        pos, res = capi.arcs_anneal(ctx, inp, prm, 0.5, 1)
        e64 = r0 + O.arcs_full(pr, oprm, pos=pos, repulsion=False)
        assert abs(res.energy_fp64 - e64) <= 1e-6 * e64
        assert res.rel_error < (1e-6 if resync else 1e-4)
        assert abs(res.energy - e64) <= 0.01 * e64   # the 1% final-energy bar


def test_arcs_dropin_multichain(ctx):
    pr, inp, _ = problem("plain", n=256, arcs=400, seed=42)
    prm = capi.default_params(capi.LEVEL_ARCS, max_temp=5.0, dt_temp=0.9999,
                              milestone_steps=50000, improvement=0.99)
    pos, res = capi.arcs_anneal(ctx, inp, prm, 0.5, 64)
    assert np.isfinite(pos).all()
    assert 0 <= res.best_chain < 64 and res.total_moves >= res.moves > 0
    oprm = O.Params(max_temp=5.0, dt_temp=0.9999, milestone_steps=50000, improvement=0.99)
    e64 = O.arcs_repulsion(pr) + O.arcs_full(pr, oprm, pos=pos, repulsion=False)
    assert abs(res.energy_fp64 - e64) <= 1e-6 * e64


@pytest.mark.parametrize("lanes", [1, 2, 4, 8])
def test_arcs_batch_units_match_oracle(ctx, lanes):
    """Every unit of a batch follows the oracle's Philox-mode annealer."""
    regs = [synth.arcs_region(n, int(1.5 * n), seed=s) for s, n in enumerate([32, 57, 130, 300, 80, 41])]
    inputs = [capi.ArcsInput.from_dense(r.pos, r.dense()) for r in regs]
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=1000, improvement=0.99)
    prm = capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_CPU, max_moves=3000, **base)
    ctx.set_seed(99)
    b = capi.ArcsBatch(ctx, inputs, prm, [0.5] * len(inputs), lanes=lanes)
    b.run()
    pos, res = b.results()
    same = 0
    for u, r in enumerate(regs):
        pr = O.ArcsProblem(r.pos, r.dense())
        opos, ores = O.arcs_anneal(pr, O.Params(max_moves=3000, **base), 0.5, 99,
                                   rng=O.RNG_PHILOX, chain=u)
        assert abs(ores.score - res[u].energy) <= 1e-3 * abs(ores.score)
        same += int(ores.moves == res[u].moves and np.allclose(opos, pos[u], atol=1e-3))
    assert same >= len(regs) - 1


def test_arcs_batch_autotune(ctx, tmp_path, monkeypatch):
    """PMMC_LANES_AUTO: every class gets lanes and warps from timed trials,
    the choices land in the JSON cache, the batch still follows the oracle,
    and a second batch of the same shape reuses the cached choices."""
    import json
    path = tmp_path / "tune.json"
    monkeypatch.setenv("PMMC_AUTOTUNE_CACHE", str(path))
    sizes = [32, 57, 130, 300, 80, 41, 1500, 2048]
    regs = [synth.arcs_region(n, int(1.5 * n), seed=s) for s, n in enumerate(sizes)]
    inputs = [capi.ArcsInput.from_dense(r.pos, r.dense()) for r in regs]
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=1000, improvement=0.99)
    prm = capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_CPU, max_moves=3000, **base)
    ctx.set_seed(99)
    b = capi.ArcsBatch(ctx, inputs, prm, [0.5] * len(inputs), lanes=capi.LANES_AUTO)
    cls = b.classes()
    assert cls and all(la in (1, 2, 4, 8) and w in (1, 2, 4) for la, w, _, _, _ in cls)
    assert all(not dw or la in (1, 2) for la, _, _, _, dw in cls)
    assert sum(it for _, _, it, _, _ in cls) == len(inputs)
    data = json.load(open(path))
    assert len(data["entries"]) >= len(cls)
    # classes whose regions set the pass's length take the low-latency
    # configuration without trials; every other class was timed
    assert all(v["moves_per_s"] > 0 or k.endswith("_critical")
               for k, v in data["entries"].items())
    assert any(k.endswith("_critical") for k in data["entries"])
    b.run()
    pos, res = b.results()
    same = 0
    for u, r in enumerate(regs):
        pr = O.ArcsProblem(r.pos, r.dense())
        opos, ores = O.arcs_anneal(pr, O.Params(max_moves=3000, **base), 0.5, 99,
                                   rng=O.RNG_PHILOX, chain=u)
        assert abs(ores.score - res[u].energy) <= 1e-3 * abs(ores.score)
        same += int(ores.moves == res[u].moves and np.allclose(opos, pos[u], atol=1e-3))
    assert same >= len(regs) - 1
    b2 = capi.ArcsBatch(ctx, inputs, prm, [0.5] * len(inputs), lanes=capi.LANES_AUTO)
    assert b2.classes() == cls


def test_arcs_batch_graph_replay_is_deterministic(ctx):
    regs = [synth.arcs_region(n, int(1.5 * n), seed=s) for s, n in enumerate([64, 200, 700])]
    inputs = [capi.ArcsInput.from_dense(r.pos, r.dense()) for r in regs]
    prm = capi.default_params(capi.LEVEL_ARCS, max_temp=5.0, dt_temp=0.9999,
                              milestone_steps=5000, improvement=0.99, resync_every=1000)
    b = capi.ArcsBatch(ctx, inputs, prm, [0.5] * 3, use_graph=True)
    b.run()
    p1, r1 = b.results()
    b.run()
    p2, r2 = b.results()
    for a, c in zip(p1, p2):
        np.testing.assert_array_equal(a, c)
    assert [x.moves for x in r1] == [x.moves for x in r2]


def test_arcs_statistics_match_reference(ctx):
    """16 seeds: final energy, RMSD to the start and distance-map Pearson of
    the GPU annealer vs the reference's CPU MonteCarloArcs (the oracle in
    libc mode is bit-identical to it)."""
    r = synth.arcs_region(64, 100, seed=8)
    dense = r.dense()
    pr = O.ArcsProblem(r.pos, dense)
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=2000, improvement=0.99)
    ref_e, ref_rmsd, ref_p = [], [], []
    for s in range(16):
        p, res = O.arcs_anneal(pr, O.Params(**base), 0.5, 500 + s)
        ref_e.append(res.score)
        ref_rmsd.append(kabsch_rmsd(p, r.pos))
        ref_p.append(distmap_pearson(p, r.pos))
    inputs = [capi.ArcsInput.from_dense(r.pos, dense) for _ in range(16)]
    prm = capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_CPU, **base)
    ctx.set_seed(4242)
    b = capi.ArcsBatch(ctx, inputs, prm, [0.5] * 16)
    b.run()
    pos, res = b.results()
    gpu_e = [x.energy for x in res]
    gpu_rmsd = [kabsch_rmsd(p, r.pos) for p in pos]
    gpu_p = [distmap_pearson(p, r.pos) for p in pos]
    for a, c in ((ref_e, gpu_e), (ref_rmsd, gpu_rmsd), (ref_p, gpu_p)):
        assert ks_2samp_p(a, c) > 0.05


@pytest.mark.parametrize("lanes", [1, 2])
def test_arcs_drawing_warp_gives_the_same_chains(ctx, lanes):
    """A second warp per chain drawing the moves ahead changes nothing but
    the timing: every chain of a batch ends bit-identical (positions, energy,
    moves) to the single-warp form."""
    sizes = [40, 300, 1100, 2000, 75]
    regs = [synth.arcs_region(n, int(1.5 * n), seed=50 + s) for s, n in enumerate(sizes)]
    inputs = [capi.ArcsInput.from_dense(r.pos, r.dense()) for r in regs]
    inputs += [problem("fixed")[1], problem("loops_sphere")[1]]  # movable list, loops
    prm = capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_CPU, max_temp=5.0,
                              dt_temp=0.9999, milestone_steps=5000, improvement=0.99,
                              resync_every=1000)
    out = []
    for dw in (False, True):
        ctx.set_seed(321)
        b = capi.ArcsBatch(ctx, inputs, prm, [0.5] * len(inputs), lanes=lanes, drawing_warp=dw)
        assert all(c[4] == dw for c in b.classes())
        b.run()
        out.append(b.results())
        b.close()
    (p0, r0), (p1, r1) = out
    for a, c in zip(p0, p1):
        np.testing.assert_array_equal(a, c)
    assert [(x.moves, x.accepted, x.energy, x.status) for x in r0] == \
        [(x.moves, x.accepted, x.energy, x.status) for x in r1]
    assert all(x.status == 0 for x in r1)


def test_arcs_drawing_warp_trace_replays(ctx):
    """The trace of a chain with a drawing warp replays on the oracle."""
    r = synth.arcs_region(300, 450, seed=77)
    pr = O.ArcsProblem(r.pos, r.dense())
    base = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=2000, improvement=0.99)
    prm = capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_CPU, max_moves=6000,
                              **base)
    ctx.set_seed(777)
    b = capi.ArcsBatch(ctx, [capi.ArcsInput.from_dense(r.pos, r.dense())], prm, [0.5],
                       trace_cap=6000, lanes=1, drawing_warp=True)
    b.run()
    _, res = b.results()
    tr = b.trace(int(res[0].moves))
    rep = O.arcs_replay(pr, O.Params(max_moves=6000, **base), 0.5, 777, 0, tr)
    check_replay(tr, rep)


def test_plain_call_with_one_chain_matches_the_single_warp_batch(ctx):
    """The drop-in call with at most one chain per SM runs one lane per
    proposal with a drawing warp; a one-chain call equals the batch form
    with one lane and no drawing warp, move for move (same Philox key: the
    seed is reset before each call).  With several chains the first to
    converge stops the others at a time-dependent move, so only one chain
    compares exactly."""
    n_chains = 1
    r = synth.arcs_region(180, 270, seed=91)
    inp = capi.ArcsInput.from_dense(r.pos, r.dense())
    prm = capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_CPU, max_temp=5.0,
                              dt_temp=0.9999, milestone_steps=3000, improvement=0.99)
    ctx.set_seed(4242)
    pos, res = capi.arcs_anneal(ctx, inp, prm, 0.5, n_chains)
    ctx.set_seed(4242)
    b = capi.ArcsBatch(ctx, [inp], prm, [0.5], chains=n_chains, use_graph=False,
                       stop_all=True, lanes=1, drawing_warp=False)
    b.run()
    bpos, bres = b.results()
    b.close()
    assert res.status == 0 and bres[0].status == 0
    assert (res.moves, res.energy) == (bres[0].moves, bres[0].energy)
    np.testing.assert_array_equal(pos, bpos[0])


def test_arcs_drawing_warp_wait_runs_out(ctx, monkeypatch):
    """The chain's wait on its drawing warp is bounded: with the drawing warp
    told never to publish (a test-only switch), the chain gives up after its
    2 s limit with status 3 and no move, nothing faults or hangs, and the
    context runs the next batch normally."""
    import time
    r = synth.arcs_region(100, 150, seed=5)
    inp = capi.ArcsInput.from_dense(r.pos, r.dense())
    prm = capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_CPU, max_moves=5000,
                              max_temp=5.0, dt_temp=0.9999, milestone_steps=1000,
                              improvement=0.99)
    monkeypatch.setenv("PMMC_TEST_STALL_DRAWS", "1")
    b = capi.ArcsBatch(ctx, [inp], prm, [0.5], use_graph=False, lanes=1, drawing_warp=True)
    monkeypatch.delenv("PMMC_TEST_STALL_DRAWS")
    t0 = time.time()
    b.run()
    _, res = b.results()
    dt = time.time() - t0
    b.close()
    assert res[0].status == 3 and res[0].moves == 0
    assert 1.5 < dt < 20
    b2 = capi.ArcsBatch(ctx, [inp], prm, [0.5], use_graph=False, lanes=1, drawing_warp=True)
    b2.run()
    _, res2 = b2.results()
    b2.close()
    assert res2[0].status == 0 and res2[0].moves > 0
