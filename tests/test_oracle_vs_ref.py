"""The oracle against the live reference harness on fresh seeded inputs
(runs only where the reference sources exist; elsewhere the golden fixtures
carry the pin)."""
import numpy as np
import pytest

from oracle import oracle as O
from pmmc_gb300 import synth

pytestmark = pytest.mark.skipif(not O.ref_available(), reason="reference harness not built")


@pytest.mark.parametrize("seed", [11, 12, 13])
def test_arcs_anneal_bit_exact(seed):
    r = synth.arcs_region(80, 150, seed=seed)
    pr = O.ArcsProblem(r.pos, r.dense())
    prm = O.Params(max_temp=5.0, dt_temp=0.9999, milestone_steps=3000, improvement=0.99)
    p1, s1, m1 = O.ref_arcs_anneal(pr, prm, 0.5, seed)
    p2, res = O.arcs_anneal(pr, prm, 0.5, seed)
    assert (m1, s1) == (res.moves, res.score)
    np.testing.assert_array_equal(p1, p2)


def test_heatmap_anneal_bit_exact():
    h = synth.heatmap_region(48, seed=21, n_tads=2, tad_min=6, tad_max=10)
    pr = O.HeatmapProblem(h.pos, h.heat, 1, np.array([0, 20, 48], np.int32))
    prm = O.Params(max_temp=5.0, dt_temp=0.9999, milestone_steps=300, improvement=0.99)
    p1, s1, m1 = O.ref_heatmap_anneal(pr, prm, 1.0, 9)
    p2, res = O.heatmap_anneal(pr, prm, 1.0, 9)
    assert (m1, s1) == (res.moves, res.score)
    np.testing.assert_array_equal(p1, p2)


def test_smooth_anneal_bit_exact():
    c = synth.smooth_chain(70, seed=22)
    pr = O.SmoothProblem(c.pos, c.dist_to_next, c.fixed)
    prm = O.Params(max_temp=5.0, dt_temp=0.9999, milestone_steps=700, improvement=0.99,
                   k_stretch=0.1, k_squeeze=0.1, sphere_radius=9.0)
    p1, s1, m1 = O.ref_smooth_anneal(pr, prm, 0.5, 4)
    p2, res = O.smooth_anneal(pr, prm, 0.5, 4)
    assert (m1, s1) == (res.moves, res.score)
    np.testing.assert_array_equal(p1, p2)


def test_mark_arcs_random():
    rng = np.random.default_rng(5)
    starts = np.sort(rng.choice(20_000, 25, replace=False)) * 50
    anchors = np.stack([starts, starts + rng.integers(0, 6000, 25)], 1).astype(np.int32)
    raw = []
    for _ in range(400):
        i, j = rng.integers(0, 25, 2)
        raw.append([int(rng.integers(anchors[i, 0], anchors[i, 1] + 1)),
                    int(rng.integers(anchors[j, 0], anchors[j, 1] + 1)),
                    int(rng.integers(1, 9)), int(rng.integers(0, 4))])
    raw = np.array(raw, np.int32)
    np.testing.assert_array_equal(O.mark_arcs(anchors, raw), O.ref_mark_arcs(anchors, raw))


@pytest.mark.parametrize("kw", [
    dict(n_anchors=400, n_active=300, active_from=60, n_long=6000, seed=71, outside_arcs=20,
         duplicate_arcs=20),
    dict(n_anchors=250, n_long=4000, seed=72, heat=True, count=(-0.6, 4.0, 0.5, 0.2),
         influence=0.8),
    dict(n_anchors=150, n_long=3000, seed=73, count=(0.4, 15.0, 1.0, -0.01)),
])
def test_anchor_targets_random(kw):
    """calcAnchorExpectedDistancesHeatmap on fresh inputs: the dense matrix
    and the long-arc counters."""
    t = synth.anchor_targets_problem(**kw)
    d1, s1 = O.ref_anchor_targets(t)
    d2, s2 = O.anchor_targets(t)
    assert s1 == s2
    np.testing.assert_array_equal(d1.view(np.uint32), d2.view(np.uint32))


@pytest.mark.parametrize("kw,it,lr", [
    (dict(n_anchors=160, n_long=2500, seed=74, springs=(0.1, 0.1, 0.0)), 400, 0.05),
    (dict(n_anchors=120, n_long=2000, seed=75, springs=(0.2, 0.05, 0.1)), 150, 0.03),
    (dict(n_anchors=90, n_long=1500, seed=76, springs=(0.0, 0.0, 0.0)), 300, 0.1),
])
def test_stress_refine_random(kw, it, lr):
    """stressRefineAnchors on fresh inputs: sorted region and positions
    (this host's libm acosf on both sides)."""
    t = synth.stress_problem(**kw)
    o1, x1 = O.ref_stress_refine(t, it, lr)
    o2, x2, _ = O.stress_refine(t, it, lr)
    np.testing.assert_array_equal(o1, o2)
    np.testing.assert_array_equal(x1.view(np.uint32), x2.view(np.uint32))


def _walk(n: int, moves: int, step: float, seed: int, movable=None, in2d=False):
    """A scripted walk: uniform beads (among `movable`), uniform displacements
    in [-step, step) per axis, each move kept with probability 0.3."""
    rng = np.random.default_rng(seed)
    t = np.zeros(moves, np.dtype([("bead", np.int32), ("accepted", np.int32),
                                  ("dx", np.float32), ("dy", np.float32), ("dz", np.float32)]))
    beads = np.arange(n) if movable is None else np.asarray(movable)
    t["bead"] = rng.choice(beads, moves)
    for ax in ("dx", "dy", "dz"):
        t[ax] = rng.uniform(-step, step, moves).astype(np.float32)
    if in2d:
        t["dz"] = 0.0
    t["accepted"] = rng.random(moves) < 0.3
    return t


WALK_MOVES = 10_000


def test_arcs_local_energy_walk():
    """10^4 proposals on the plain drop-in's region shape (256 beads, 400 arcs)
    plus loop constraints and a sphere: the oracle's local arc energy before
    and after every move equals the reference's calcScoreDistancesActiveRegion(p)
    + calcScoreLoopEnergy(p) + boundaryPenalty bit for bit."""
    r = synth.arcs_region(256, 400, seed=31)
    rng = np.random.default_rng(32)
    li = rng.integers(0, 256, 8).astype(np.int32)
    lj = rng.integers(0, 256, 8).astype(np.int32)
    pr = O.ArcsProblem(r.pos, r.dense(), None, li, lj, rng.uniform(0.5, 2.0, 8).astype(np.float32),
                       rng.uniform(1.0, 3.0, 8).astype(np.float32))
    prm = O.Params(sphere_radius=6.0)
    t = _walk(256, WALK_MOVES, 0.5, 33)
    ref = O.ref_arcs_walk(pr, prm, t)
    orc = O.arcs_replay(pr, prm, 0.5, 0, 0, t)
    np.testing.assert_array_equal(orc["before"], ref["before"])
    np.testing.assert_array_equal(orc["after"], ref["after"])
    assert np.count_nonzero(ref["after"] != ref["before"]) > WALK_MOVES // 2


def test_heatmap_local_energy_walk():
    """10^4 proposals on a 256-bead map with a diagonal band of 2 and two
    chromosome blocks: calcScoreHeatmapActiveRegion(p) before and after."""
    h = synth.heatmap_region(256, seed=34, n_tads=4, tad_min=20, tad_max=60)
    pr = O.HeatmapProblem(h.pos, h.heat, 2, np.array([0, 100, 256], np.int32))
    prm = O.Params()
    t = _walk(256, WALK_MOVES, 0.5, 35)
    ref = O.ref_heatmap_walk(pr, prm, t)
    orc = O.heatmap_replay(pr, prm, 1.0, 0, 0, t)
    np.testing.assert_array_equal(orc["before"], ref["before"])
    np.testing.assert_array_equal(orc["after"], ref["after"])


def test_smooth_local_energy_walk():
    """10^4 proposals on a 200-bead subanchor chain (anchors fixed, weights
    0.7/1.3, a sphere): calcScoreStructureSmooth(p, true, true) +
    boundaryPenalty before and after, 2D moves included."""
    c = synth.smooth_chain(200, seed=36)
    pr = O.SmoothProblem(c.pos, c.dist_to_next, c.fixed)
    prm = O.Params(k_stretch=0.1, k_squeeze=0.1, k_angle=0.1, w_dist=0.7, w_angle=1.3,
                   sphere_radius=8.0)
    free = np.flatnonzero(c.fixed == 0)
    for k, in2d in enumerate((False, True)):
        t = _walk(200, WALK_MOVES // 2, 0.5, 37 + k, movable=free, in2d=in2d)
        ref = O.ref_smooth_walk(pr, prm, t)
        orc = O.smooth_replay(pr, prm, 0.5, 0, 0, t)
        np.testing.assert_array_equal(orc["before"], ref["before"])
        np.testing.assert_array_equal(orc["after"], ref["after"])


@pytest.mark.parametrize("seed", [41, 42, 43])
def test_distance_heatmap_random(seed):
    """createDistanceHeatmap on fresh contact maps: odd sizes, wide diagonal
    bands, many zeros, asymmetric inputs, both level constants."""
    rng = np.random.default_rng(seed)
    n = int(rng.integers(20, 150))
    diag = int(rng.integers(0, 4))
    level = int(rng.integers(0, 2))
    scale = float(rng.choice([1.0, 100.0]))
    power = float(rng.uniform(-1.2, -0.2))
    stretch = float(rng.uniform(1.1, 3.0))
    c = (rng.lognormal(0.0, 1.0, (n, n)) * (rng.random((n, n)) > 0.3)).astype(np.float32)
    if seed % 2:
        c = np.triu(c) + np.triu(c, 1).T
    d, _, _ = O.distance_heatmap(c, diag, scale, power, stretch)
    np.testing.assert_array_equal(d, O.ref_distance_heatmap(c, diag, level, scale, power, stretch))


@pytest.mark.parametrize("seed", [51, 52, 53])
def test_equidistant_random(seed):
    """The equidistant-model interpolation on fresh chromosome levels:
    uneven spacing, 2 to 200 clusters, resolutions from below the smallest
    gap to above the largest."""
    import os
    if not os.path.exists(os.path.join(os.path.dirname(O.__file__), "_ref", "libpmmc_ref_hc.so")):
        pytest.skip("the reference's equidistant harness is not built")
    rng = np.random.default_rng(seed)
    n = int(rng.integers(2, 200))
    width = rng.integers(50, 40000, n)
    start = np.concatenate([[5_000], 5_000 + np.cumsum(width)[:-1]]).astype(np.int32)
    end = (start + width - 1).astype(np.int32)
    gpos = ((start + end) // 2).astype(np.int32)
    pos = synth.random_walk(n, rng) * np.float32(1.5)
    res = int(rng.choice([37, 500, 5000, 60000]))
    lo, hi = int(gpos[0]), int(gpos[-1])
    pts = O.equidistant(gpos, pos, int(end[0]), int(start[-1]), lo, hi, res)
    ref = O.ref_equidistant(gpos, start, end, pos, lo, hi, res)
    np.testing.assert_array_equal(pts, ref)


@pytest.mark.parametrize("n,seed", [(16, 61), (256, 62), (700, 63)])
def test_parity_metrics_match_reference(n, seed):
    """The structural metrics of the 16-seed distribution tests equal the
    reference's own: Kabsch RMSD against Chromosome::calcRMSD (fast_rmsd,
    float result) and the pairwise-distance Pearson correlation against
    MetricsFramework::distanceCorrelation (float distances, double sums,
    float result)."""
    from parity import distmap_pearson, kabsch_rmsd
    rng = np.random.default_rng(seed)
    a = synth.random_walk(n, rng)
    # a rotated, shifted, perturbed copy (and a mirror image for one case)
    q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    if seed % 2 == 0 and np.linalg.det(q) > 0:
        q[:, 0] *= -1.0
    b = (a @ q.T + rng.normal(0.0, 0.3, (n, 3)) + 5.0).astype(np.float32)
    assert kabsch_rmsd(a, b) == pytest.approx(O.ref_rmsd(a, b), rel=1e-5, abs=1e-5)
    assert distmap_pearson(a, b) == pytest.approx(O.ref_distance_correlation(a, b), rel=1e-6)
