"""Request loop (pmmc_server_*): continuous batching of arc-level regions.

Each region anneals with its own Philox key, so its result must be the same
bit for bit whether it runs alone (one region per launch, one launch at a
time) or mixed with others (many per launch, launches overlapping, submitted
from several threads); and it must follow the oracle's Philox-mode annealer.
"""
import threading

import numpy as np
import pytest

from oracle import oracle as O
from pmmc_gb300 import capi, synth

pytestmark = pytest.mark.gpu

BASE = dict(max_temp=5.0, dt_temp=0.9999, milestone_steps=1000, improvement=0.99)
SIZES = [64, 3000, 97, 410, 64, 1500, 230, 5200, 130, 800, 71, 2048]


def regions():
    regs = [synth.arcs_region(n, int(1.5625 * n), seed=100 + k) for k, n in enumerate(SIZES)]
    inputs = []
    for r in regs:
        rp, col, tgt = r.csr()
        inputs.append(capi.ArcsInput(r.pos, rp, col, tgt))
    return regs, inputs


def params():
    return capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_CPU, max_moves=3000, **BASE)


def test_server_alone_equals_mixed_and_oracle(ctx):
    regs, inputs = regions()
    seeds = [1000 + 7 * k for k in range(len(inputs))]
    # alone: one region per launch, one launch in flight
    sv = capi.Server(ctx, params(), max_waves=1, max_wave_requests=1)
    alone = []
    for inp, sd in zip(inputs, seeds):
        t = sv.submit(inp, 0.5, sd)
        alone.append(sv.wait(t))
    st = sv.stats()
    assert st["waves"] == len(inputs) and st["running_peak"] == 1
    sv.close()
    # mixed: everything submitted at once from four threads
    sv = capi.Server(ctx, params(), max_waves=4, max_wave_requests=5)
    tickets = [None] * len(inputs)

    def submit(ks):
        for k in ks:
            tickets[k] = sv.submit(inputs[k], 0.5, seeds[k])

    th = [threading.Thread(target=submit, args=(range(i, len(inputs), 4),)) for i in range(4)]
    for t in th:
        t.start()
    for t in th:
        t.join()
    mixed = [sv.wait(t) for t in tickets]
    st = sv.stats()
    assert st["completed"] == len(inputs) and st["failed"] == 0
    assert st["running_peak"] > 1
    sv.close()
    for (pa, ra, _), (pm, rm, _) in zip(alone, mixed):
        np.testing.assert_array_equal(pa, pm)
        assert ra.energy == rm.energy and ra.moves == rm.moves and ra.accepted == rm.accepted
    # the oracle's Philox-mode annealer with the region's own key, chain 0
    agree = 0
    for r, (p, res, _), sd in zip(regs, alone, seeds):
        pr = O.ArcsProblem(r.pos, r.dense())
        opos, ores = O.arcs_anneal(pr, O.Params(max_moves=3000, **BASE), 0.5, sd,
                                   rng=O.RNG_PHILOX, chain=0)
        assert abs(ores.score - res.energy) <= 1e-3 * abs(ores.score)
        assert res.rel_error < 1e-4
        agree += int(ores.moves == res.moves and np.allclose(opos, p, atol=1e-3))
    assert agree >= len(regs) - 1


def test_server_budget_admission(ctx):
    regs, inputs = regions()
    big = int(np.argmax(SIZES))
    # a budget below the largest region's footprint refuses it at submit
    sv = capi.Server(ctx, params(), budget_bytes=200_000)
    with pytest.raises(capi.PmmcError) as e:
        sv.submit(inputs[big], 0.5, 1)
    assert e.value.status == capi.PMMC_ERR_BUDGET
    sv.close()
    # a budget of about two mid-size regions: everything completes, never
    # more resident than the budget
    budget = 700_000
    sv = capi.Server(ctx, params(), budget_bytes=budget, max_waves=8)
    small = [k for k, n in enumerate(SIZES) if n <= 2048]
    ts = [sv.submit(inputs[k], 0.5, 5 + k) for k in small]
    lat = [sv.wait(t)[2] for t in ts]
    st = sv.stats()
    assert st["completed"] == len(small)
    assert 0 < st["bytes_peak"] <= budget
    assert all(x > 0 for x in lat)
    sv.close()


def test_server_wait_timeout_and_unknown_ticket(ctx):
    _, inputs = regions()
    sv = capi.Server(ctx, params())
    t = sv.submit(inputs[0], 0.5, 3)
    sv.wait(t)
    with pytest.raises(capi.PmmcError) as e:
        sv.wait(t)
    assert e.value.status == capi.PMMC_ERR_NOT_FOUND
    sv.close()


def test_server_cancel_queued_request(ctx):
    """A request withdrawn while queued comes back cancelled at once; the
    others run as they would have, and the withdrawn one leaves no trace.
    One wave of one region at a time keeps the later requests queued."""
    _, inputs = regions()
    prm = capi.default_params(capi.LEVEL_ARCS, schedule=capi.SCHEDULE_CPU, max_moves=200_000,
                              **BASE)
    sv = capi.Server(ctx, prm, max_waves=1, max_wave_requests=1)
    tickets = [sv.submit(inputs[k], 0.5, 50 + k) for k in (7, 1, 5, 3)]
    last = tickets[-1]
    assert sv.cancel(last) == 0            # still behind the first three
    assert sv.poll(last)
    with pytest.raises(capi.PmmcError) as e:
        sv.wait(last)
    assert e.value.status == capi.PMMC_ERR_CANCELLED
    assert sv.cancel(last) == capi.PMMC_ERR_NOT_FOUND   # already collected
    for t in tickets[:-1]:
        pos, res, _ = sv.wait(t)
        assert res.status == 0 and np.isfinite(pos).all()
        assert sv.cancel(t) == capi.PMMC_ERR_NOT_FOUND
    st = sv.stats()
    assert st["queued"] == 0
    sv.close()
