"""Expected-distance heatmap (createDistanceHeatmap) on the GPU against the
oracle (itself pinned bit for bit to the reference's output)."""
import numpy as np
import pytest

from oracle import oracle as O
from pmmc_gb300 import capi

pytestmark = pytest.mark.gpu

# powf on the device and in libm may differ in the last bits
REL_TOL = 1e-6


def contact_map(n, seed, zeros=0.1, diag_val=2.0):
    rng = np.random.default_rng(seed)
    i = np.arange(n)
    sep = np.abs(i[:, None] - i[None, :]).astype(np.float64)
    c = np.where(sep > 0, 1.0 / np.maximum(sep, 1.0), diag_val) * rng.lognormal(0.0, 0.5, (n, n))
    c[rng.random((n, n)) < zeros] = 0.0
    c = np.triu(c) + np.triu(c, 1).T
    return c.astype(np.float32)


def check(d_gpu, avg_g, max_g, d_ref, avg_r, max_r):
    assert abs(avg_g - avg_r) <= 1e-4 * abs(avg_r)   # FP64 sum vs the reference's float sum
    lo, hi = min(max_g, max_r), max(max_g, max_r)
    # entries away from the clamp band: equal to the tolerance of powf
    band = (d_ref >= lo * (1 - 1e-6)) & (d_ref <= hi * (1 + 1e-6))
    band |= (d_gpu >= lo * (1 - 1e-6)) & (d_gpu <= hi * (1 + 1e-6))
    ok = ~band
    np.testing.assert_array_equal(d_gpu[d_ref == -1.0], -1.0)
    np.testing.assert_array_equal(d_gpu[d_ref == 0.0], 0.0)
    err = np.abs(d_gpu[ok] - d_ref[ok]) / np.maximum(np.abs(d_ref[ok]), 1e-30)
    assert err.max() <= REL_TOL
    # inside the band both are clamped to their own value
    assert np.all(d_gpu <= max_g + abs(max_g) * 1e-7)


@pytest.mark.parametrize("case", ["distmap0", "distmap1", "distmap2"])
def test_distance_heatmap_golden(ctx, case):
    g = np.load(f"tests/golden/{case}.npz")
    diag, sc, pw, st = g["params"]
    d, avg, mx, _ = capi.distance_heatmap(ctx, g["contact"], int(diag), sc, pw, st)
    _, avg_r, max_r = O.distance_heatmap(g["contact"], int(diag), sc, pw, st)
    check(d, avg, mx, g["dist"], avg_r, max_r)


@pytest.mark.parametrize("n,diag", [(1, 1), (31, 0), (33, 1), (257, 3), (1000, 2)])
def test_distance_heatmap_sizes(ctx, n, diag):
    c = contact_map(n, seed=n)
    d, avg, mx, _ = capi.distance_heatmap(ctx, c, diag, 100.0, -0.333, 2.0)
    dr, avg_r, max_r = O.distance_heatmap(c, diag, 100.0, -0.333, 2.0)
    check(d, avg, mx, dr, avg_r, max_r)
    np.testing.assert_array_equal(d, d.T)


def test_distance_heatmap_all_band(ctx):
    """No value outside the diagonal band: the average takes the band (-1)
    entries, as Heatmap::getAvg does with diagonal size 0."""
    n = 40
    c = np.zeros((n, n), np.float32)
    for k in range(3):
        c += np.diag(np.ones(n - k, np.float32), k) + np.diag(np.ones(n - k, np.float32), -k) * (k > 0)
    d, avg, mx, _ = capi.distance_heatmap(ctx, c, 3, 100.0, -0.333, 2.0)
    dr, avg_r, max_r = O.distance_heatmap(c, 3, 100.0, -0.333, 2.0)
    assert avg == pytest.approx(avg_r, rel=1e-6) and avg < 0
    np.testing.assert_array_equal(d, dr)
