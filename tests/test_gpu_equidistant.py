"""Equidistant model on the GPU against the oracle (pinned to the
reference's own CPU path): bit for bit."""
import numpy as np
import pytest

from oracle import oracle as O
from pmmc_gb300 import capi, synth

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", ["equi0", "equi1", "equi2", "equi3"])
def test_equidistant_golden(ctx, case):
    g = np.load(f"tests/golden/{case}.npz")
    pts, _ = capi.equidistant_model(ctx, g["gpos"], g["pos"], int(g["end"][0]),
                                    int(g["start"][-1]), int(g["gpos"][0]), int(g["gpos"][-1]),
                                    int(g["res"][0]))
    np.testing.assert_array_equal(pts, g["points"])


@pytest.mark.parametrize("n,res,sort", [(1, 100, True), (5000, 997, True), (300, 10, False)])
def test_equidistant_random_levels(ctx, n, res, sort):
    rng = np.random.default_rng(n)
    width = rng.integers(200, 20000, n)
    start = np.concatenate([[5_000], 5_000 + np.cumsum(width)[:-1]]).astype(np.int32)
    end = (start + width - 1).astype(np.int32)
    gpos = ((start + end) // 2).astype(np.int32)
    if not sort and n > 3:           # an out-of-order level: the linear scan
        gpos[[1, 2]] = gpos[[2, 1]]
    pos = synth.random_walk(n, rng) * np.float32(1.5)
    args = (int(end[0]), int(start[-1]), int(gpos[0]) - 3 * res, int(gpos[-1]) + 2 * res, res)
    pts, _ = capi.equidistant_model(ctx, gpos, pos, *args)
    ref = O.equidistant(gpos, pos, *args)
    np.testing.assert_array_equal(pts, ref)
