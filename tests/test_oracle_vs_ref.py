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
