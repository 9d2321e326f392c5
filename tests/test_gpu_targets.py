"""Anchor-level expected distances (calcAnchorExpectedDistancesHeatmap) on
the GPU against the oracle, which is pinned bit for bit to the reference.

The CSR the device builds must hold exactly the entries >= 0 off the
diagonal of the reference's dense matrix (entry (i, j) = dense[j, i]), with
the same values.  Values from the memo table and from the host are
bit-exact; a long arc's count above 100 goes through FP64 exp / pow on the
device (at most 1 ulp in FP64), so its float can differ from the host's in
the last bit after rounding: values are compared to 1 float ulp, structure
and counters exactly."""
import numpy as np
import pytest

from oracle import oracle as O
from pmmc_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def dense_csr(d):
    n = d.shape[0]
    m = (d.T >= 0) & ~np.eye(n, dtype=bool)
    rows, cols = np.nonzero(m)
    row_ptr = np.concatenate([[0], np.cumsum(m.sum(1))]).astype(np.int32)
    return row_ptr, cols.astype(np.int32), d.T[rows, cols].astype(np.float32)


def case(name):
    g = np.load(f"tests/golden/{name}.npz")
    t = {k: g[k] for k in ("active", "arc_ptr", "arc_idx", "arc_start", "arc_end", "arc_score",
                           "long_start", "long_end", "long_score", "anc_start", "anc_end",
                           "memo")}
    t["first_cluster"] = int(g["first_cluster"][0])
    t["count"] = tuple(float(x) for x in g["count"])
    t["heat"] = None if g["heat"].size == 0 else g["heat"]
    t["influence"] = float(g["influence"][0])
    return t, g


def check(got, dense, stats=None, want_stats=None):
    rp, col, tgt, st, _ = got
    erp, ecol, etgt = dense_csr(dense)
    np.testing.assert_array_equal(rp, erp)
    np.testing.assert_array_equal(col, ecol)
    np.testing.assert_array_max_ulp(tgt, etgt, maxulp=1)
    if want_stats is not None:
        assert [st["applied"], st["out_of_range"], st["inactive"], st["collision"]] == \
            list(want_stats)


@pytest.mark.parametrize("name", [f"targets{k}" for k in range(5)])
def test_anchor_targets_golden(ctx, name):
    t, g = case(name)
    check(capi.anchor_targets(ctx, t), g["dense"], want_stats=g["stats"])


@pytest.mark.parametrize("kw", [
    dict(n_anchors=1500, n_active=1000, active_from=200, n_long=200_000, seed=41,
         outside_arcs=40, duplicate_arcs=40),
    dict(n_anchors=800, n_long=50_000, seed=42, heat=True, count=(-0.4, 3.0, 0.5, 0.05)),
    dict(n_anchors=3, n_long=100, seed=43),
    # every distance >= 0 takes the first-writer kernel, a negative base the walk
    dict(n_anchors=600, n_long=80_000, seed=46, count=(0.5, 20.0, 1.0, -0.005),
         duplicate_arcs=30),
    dict(n_anchors=600, n_long=80_000, seed=47, count=(0.5, 0.0, 1.0, 0.0)),
    dict(n_anchors=400, n_long=0, seed=44),
])
def test_anchor_targets_random(ctx, kw):
    t = synth.anchor_targets_problem(**kw)
    dense, st = O.anchor_targets(t)
    check(capi.anchor_targets(ctx, t), dense,
          want_stats=[st["applied"], st["out_of_range"], st["inactive"], st["collision"]])


def test_anchor_targets_empty_region(ctx):
    t = synth.anchor_targets_problem(n_anchors=50, n_long=100, seed=45)
    for k in ("active", "arc_idx"):
        t[k] = t[k][:0]
    t["arc_ptr"] = np.zeros(1, np.int32)
    rp, col, tgt, st, _ = capi.anchor_targets(ctx, t)
    assert list(rp) == [0] and len(col) == 0
    assert st["inactive"] + st["out_of_range"] == 100 and st["applied"] == 0


def test_anchor_targets_full_size_properties(ctx):
    """The benchmark size (4000 anchors, 2M long arcs): every long arc is
    counted once, the CSR is symmetric with sorted rows, and a sample of
    rows equals the oracle's on the same arcs."""
    t = synth.anchor_targets_problem(n_anchors=4000, n_long=2_000_000, seed=21)
    rp, col, tgt, st, _ = capi.anchor_targets(ctx, t)
    assert sum(st.values()) == 2_000_000
    n = len(t["active"])
    assert rp[0] == 0 and rp[-1] == len(col) and np.all(np.diff(rp) >= 0)
    rows = np.repeat(np.arange(n), np.diff(rp))
    assert np.all(col != rows)
    for i in range(n):
        assert np.all(np.diff(col[rp[i]:rp[i + 1]]) > 0)
    fwd = dict(zip(zip(rows.tolist(), col.tolist()), tgt.tolist()))
    assert all(fwd[(c, r)] == v for (r, c), v in list(fwd.items())[:: max(1, len(fwd) // 5000)])
    # the oracle on the same inputs with a tenth of the long arcs, against the
    # device on the same tenth
    sub = dict(t)
    for k in ("long_start", "long_end", "long_score"):
        sub[k] = t[k][:200_000]
    dense, ost = O.anchor_targets(sub)
    check(capi.anchor_targets(ctx, sub), dense,
          want_stats=[ost["applied"], ost["out_of_range"], ost["inactive"], ost["collision"]])


def test_anchor_targets_clustered_anchors(ctx):
    """Sorted anchors with very uneven gaps (many anchors per bucket of the
    lookup table, long empty stretches) against the oracle's scan."""
    t = synth.anchor_targets_problem(n_anchors=500, n_long=40_000, seed=48)
    rng = np.random.default_rng(48)
    gaps = np.where(rng.random(500) < 0.05, rng.integers(200_000, 2_000_000, 500),
                    rng.integers(12, 40, 500))
    start = (np.cumsum(gaps) + 1000).astype(np.int64)
    t["anc_start"] = start.astype(np.int32)
    t["anc_end"] = (start + rng.integers(0, 10, 500)).astype(np.int32)
    lo, hi = int(start[0]) - 5000, int(start[-1]) + 5000
    pick = rng.integers(0, 500, (40_000, 2))
    t["long_start"] = np.where(rng.random(40_000) < 0.7, start[pick[:, 0]] + 3,
                               rng.integers(lo, hi, 40_000)).astype(np.int32)
    t["long_end"] = np.where(rng.random(40_000) < 0.7, start[pick[:, 1]] + 1,
                             rng.integers(lo, hi, 40_000)).astype(np.int32)
    dense, st = O.anchor_targets(t)
    assert st["applied"] > 1000
    check(capi.anchor_targets(ctx, t), dense,
          want_stats=[st["applied"], st["out_of_range"], st["inactive"], st["collision"]])
