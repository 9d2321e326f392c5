"""Arc marking on the GPU against the oracle (bit-exact)."""
import os

import numpy as np
import pytest

from oracle import oracle as O
from pmmc_gb300 import capi

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_mark_arcs_golden(ctx):
    g = dict(np.load(os.path.join(GOLD, "mark0.npz")))
    arcs, nm = capi.mark_arcs(ctx, g["anchors"], g["raw"])
    np.testing.assert_array_equal(arcs, g["arcs"])


@pytest.mark.parametrize("seed,overlap", [(1, False), (2, True), (3, True)])
def test_mark_arcs_random(ctx, seed, overlap):
    rng = np.random.default_rng(seed)
    A = 400
    starts = np.sort(rng.choice(10_000_000, A, replace=False))
    width = rng.integers(0, 20_000 if overlap else 500, A)
    anchors = np.stack([starts, starts + width], 1).astype(np.int32)
    anchors[rng.integers(0, A, 10), 1] = anchors[rng.integers(0, A, 10), 0]  # some length <= 1
    raw = []
    for _ in range(5000):
        i, j = rng.integers(0, A, 2)
        raw.append([int(rng.integers(anchors[i, 0], max(anchors[i, 0], anchors[i, 1]) + 1)),
                    int(rng.integers(anchors[j, 0], max(anchors[j, 0], anchors[j, 1]) + 1)),
                    int(rng.integers(1, 20)), int(rng.integers(0, 4))])
    raw = np.array(raw, np.int32)
    arcs, nm = capi.mark_arcs(ctx, anchors, raw)
    np.testing.assert_array_equal(arcs, O.mark_arcs(anchors, raw))


def test_mark_arcs_edges(ctx):
    a = np.array([[0, 0], [100, 200], [300, 400]], np.int32)   # first anchor has length 0
    assert capi.mark_arcs(ctx, a, np.zeros((0, 4), np.int32))[0].shape == (0, 7)
    raw = np.array([[0, 150, 3, 0], [150, 350, 2, 1], [150, 160, 1, 0]], np.int32)
    arcs, nm = capi.mark_arcs(ctx, a, raw)
    np.testing.assert_array_equal(arcs, O.mark_arcs(a, raw))
    assert nm == 1
    with pytest.raises(capi.PmmcError):
        capi.mark_arcs(ctx, a[::-1].copy(), raw)   # anchors must be sorted
