"""Stress refinement (stressRefineAnchors) on the GPU against the oracle,
which equals the reference bit for bit.

Each anchor's gradient is summed on the device in the reference's order, so
without the angle term the sorted region, the positions, the iteration
count, the stop reason and the final step are exact (and the golden
positions the reference wrote are matched bit for bit on any host).

The angle term calls CUDA's acosf where the reference calls the host libm's
(and the x86-64 and aarch64 libms differ from each other).  acos is
ill-conditioned near straight angles and the forward difference
(Ep - E0) / h with h = 1e-3 magnifies a last-ulp difference, so the
descents drift apart: on the first golden case the reference's own x86-64
run and the oracle on aarch64 end 13.5 units apart (extent 52), converging
after 57 and 211 iterations.  With angles the device is therefore compared
with the oracle over the first 20 iterations, where the drift stays below
1e-3 of the structure's extent (measured: 3.6e-5 after one iteration,
8.7e-4 after 20) and the energy within 1e-4, and full runs must lower the
energy."""
import numpy as np
import pytest

from oracle import oracle as O
from pmmc_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def case(name):
    g = np.load(f"tests/golden/{name}.npz")
    t = {k: g[k] for k in ("active", "genomic_pos", "pos", "arc_start", "arc_end", "arc_score",
                           "long_start", "long_end", "long_score", "anc_start", "anc_end")}
    t["first_cluster"] = int(g["first_cluster"][0])
    t["count"] = tuple(float(x) for x in g["count"])
    t["glen"] = tuple(float(x) for x in g["glen"])
    t["springs"] = tuple(float(x) for x in g["springs"])
    return t, int(g["max_iter"][0]), float(g["lr"][0]), g


def compare(ctx, t, it, lr, want_order=None, want_pos=None):
    order, pos, res = capi.stress_refine(ctx, t, it, lr)
    oo, op, out = O.stress_refine(t, it, lr)
    np.testing.assert_array_equal(order, oo)
    if want_order is not None:
        np.testing.assert_array_equal(order, want_order)
        np.testing.assert_array_equal(op.view(np.uint32), want_pos.view(np.uint32))
    assert res["n_pairs"] == out["n_pairs"]
    if t["springs"][2] == 0.0:
        np.testing.assert_array_equal(pos.view(np.uint32), op.view(np.uint32))
        assert (res["iterations"], res["stop"], res["lr"]) == \
            (out["iterations"], out["stop"], out["lr"])
        assert abs(res["total"] - out["total"]) <= 1e-9 * abs(out["total"])
    else:
        assert it <= 20, "the angle term is compared over 20 iterations at most"
        ext = float(np.ptp(op, axis=0).max())
        dev = float(np.abs(pos - op).max())
        assert dev <= 1e-3 * ext, (dev, ext, res, out)
        assert abs(res["total"] - out["total"]) <= 1e-4 * abs(out["total"]), (res, out)
    return res, out


def compare_angles(ctx, t, it, lr):
    """With the angle term: 20 iterations against the oracle, then the full
    run lowers the energy of the first iteration and stops properly."""
    first, _ = compare(ctx, t, min(it, 20), lr)
    _, _, one = capi.stress_refine(ctx, t, 1, lr)
    _, _, full = capi.stress_refine(ctx, t, it, lr)
    assert full["total"] < one["total"]
    assert full["stop"] in (0, 1, 2) and 1 <= full["iterations"] <= it
    return first


@pytest.mark.parametrize("name", ["stress2", "stress4"])
def test_stress_golden_exact(ctx, name):
    t, it, lr, g = case(name)
    compare(ctx, t, it, lr, g["order"], g["out_pos"])


@pytest.mark.parametrize("name", ["stress0", "stress1", "stress3"])
def test_stress_golden_angles(ctx, name):
    t, it, lr, g = case(name)
    order, _, _ = capi.stress_refine(ctx, t, it, lr)
    np.testing.assert_array_equal(order, g["order"])
    compare_angles(ctx, t, it, lr)


@pytest.mark.parametrize("kw,it,lr", [
    (dict(n_anchors=1000, n_long=50_000, seed=61, springs=(0.1, 0.1, 0.0)), 400, 0.05),
    (dict(n_anchors=1000, n_long=50_000, seed=62), 400, 0.05),
    (dict(n_anchors=300, n_long=5000, seed=63, springs=(0.0, 0.0, 0.0)), 300, 0.02),
    (dict(n_anchors=2, n_long=10, seed=64), 50, 0.05),
])
def test_stress_random(ctx, kw, it, lr):
    t = synth.stress_problem(**kw)
    if t["springs"][2] == 0.0:
        compare(ctx, t, it, lr)
    else:
        compare_angles(ctx, t, it, lr)


def test_stress_nothing_to_do(ctx):
    t = synth.stress_problem(n_anchors=40, n_long=100, seed=65)
    for it, sub in ((0, None), (10, 1)):
        tt = dict(t)
        if sub:
            for k in ("active", "genomic_pos"):
                tt[k] = t[k][:sub]
            tt["pos"] = t["pos"][:sub]
        order, pos, res = capi.stress_refine(ctx, tt, it, 0.05)
        np.testing.assert_array_equal(order, tt["active"])      # not even sorted
        np.testing.assert_array_equal(pos, np.asarray(tt["pos"]).reshape(-1, 3))
        assert res["iterations"] == 0


def test_stress_full_size(ctx):
    """The benchmark chromosome (4000 anchors, 200k long arcs): exact over
    300 iterations without the angle term; with it, 20 iterations against
    the oracle and a long run that lowers the energy."""
    t = synth.stress_problem(n_anchors=4000, n_long=200_000, seed=51,
                             springs=(0.1, 0.1, 0.0))
    compare(ctx, t, 300, 0.01)
    compare_angles(ctx, synth.stress_problem(n_anchors=4000, n_long=200_000, seed=51),
                   3000, 0.01)
