"""The allocation-free arc-level entry point (pmmc_arcs_anneal_noalloc).

It serves callers that may not allocate device memory: the test plays such a
caller, owning every device buffer itself (torch tensors stand in for the
caller's pool) and passing only their addresses through the C ABI.  Two calls
in a row must reproduce the regular batched entry point with one chain (same
key, chain, lanes and staging) bit for bit, the second call running on the
scratch array the first one left behind.  A region the fixed array cannot
hold, or malformed arc lists, are refused before anything is written to the
caller's output.  This file is named so that pytest collects it last.
"""
import numpy as np
import pytest

from pmmc_gb300 import capi, synth

pytestmark = pytest.mark.gpu


def _device_problem(torch, r, fixed, csr=None):
    rp, col, tgt = r.csr() if csr is None else csr
    bufs = {
        "pos": torch.from_numpy(np.ascontiguousarray(r.pos.reshape(-1))).cuda(),
        "fixed": torch.from_numpy(fixed).cuda(),
        "rp": torch.from_numpy(rp).cuda(),
        "col": torch.from_numpy(col).cuda(),
        "tgt": torch.from_numpy(tgt).cuda(),
    }
    prob = capi.ArcsProblem(r.n, bufs["pos"].data_ptr(), bufs["fixed"].data_ptr(),
                            bufs["rp"].data_ptr(), bufs["col"].data_ptr(),
                            bufs["tgt"].data_ptr(), 0, None, None, None, None)
    return prob, bufs


def test_noalloc_matches_batched_entry_point(ctx):
    torch = pytest.importorskip("torch")
    r = synth.arcs_region(256, 400, seed=42)
    fixed = np.zeros(r.n, np.uint8)
    fixed[::17] = 1
    prm = capi.default_params(capi.LEVEL_ARCS, max_temp=5.0, dt_temp=0.9999,
                              milestone_steps=50000, improvement=0.99,
                              schedule=capi.SCHEDULE_CPU, resync_every=1000)
    seed = 20261203
    # the existing entry point: one unit, one chain, key = seed, chain 0
    ctx.set_seed(seed)
    inp = capi.ArcsInput(r.pos, *r.csr(), fixed=fixed)
    b = capi.ArcsBatch(ctx, [inp], prm, [0.5], chains=1, use_graph=False, lanes=2)
    b.run()
    want_pos, want = b.results()
    b.close()

    prob, bufs = _device_problem(torch, r, fixed)
    out = torch.zeros(r.n * 3, dtype=torch.float32, device="cuda")
    for call in range(2):
        out.fill_(float("nan"))
        torch.cuda.synchronize()
        res = capi.arcs_anneal_noalloc(prob, prm, 0.5, seed, out.data_ptr())
        got = out.cpu().numpy().reshape(-1, 3)
        assert res.status == 0, call
        assert (res.moves, res.accepted) == (want[0].moves, want[0].accepted), call
        np.testing.assert_array_equal(got, want_pos[0])
        assert res.energy == want[0].energy and res.energy_fp64 == want[0].energy_fp64
        assert res.score == want[0].score
        np.testing.assert_array_equal(got[fixed == 1], r.pos[fixed == 1])


def test_noalloc_rejects_oversized_regions(ctx):
    torch = pytest.importorskip("torch")
    r = synth.arcs_region(5000, 6000, seed=1)   # more beads than the fixed scratch holds
    prob, bufs = _device_problem(torch, r, np.zeros(r.n, np.uint8))
    out = torch.zeros(r.n * 3, dtype=torch.float32, device="cuda")
    prm = capi.default_params(capi.LEVEL_ARCS)
    with pytest.raises(capi.PmmcError) as e:
        capi.arcs_anneal_noalloc(prob, prm, 0.5, 1, out.data_ptr())
    assert e.value.status == capi.PMMC_ERR_BUDGET


def test_noalloc_rejects_malformed_lists_without_writing(ctx):
    """A column out of range, or row pointers out of order, is refused with
    PMMC_ERR_INVALID by the device-side check, before anything reads
    through the lists; the caller's output buffer keeps its contents, and the
    next good call still matches the batched entry point."""
    torch = pytest.importorskip("torch")
    r = synth.arcs_region(128, 200, seed=5)
    rp, col, tgt = r.csr()
    prm = capi.default_params(capi.LEVEL_ARCS, max_temp=5.0, dt_temp=0.9999,
                              milestone_steps=20000, improvement=0.99,
                              schedule=capi.SCHEDULE_CPU, resync_every=1000)
    out = torch.full((r.n * 3,), 7.0, dtype=torch.float32, device="cuda")
    bad_col = col.copy()
    bad_col[len(col) // 2] = r.n              # one past the last bead
    bad_rp = rp.copy()
    bad_rp[10], bad_rp[11] = bad_rp[11], bad_rp[10] - 1   # a row that ends before it starts
    for c, p in ((bad_col, rp), (col, bad_rp)):
        prob, bufs = _device_problem(torch, r, np.zeros(r.n, np.uint8), csr=(p, c, tgt))
        with pytest.raises(capi.PmmcError) as e:
            capi.arcs_anneal_noalloc(prob, prm, 0.5, 3, out.data_ptr())
        assert e.value.status == capi.PMMC_ERR_INVALID
        assert (out.cpu().numpy() == 7.0).all()
    seed = 77
    ctx.set_seed(seed)
    b = capi.ArcsBatch(ctx, [capi.ArcsInput(r.pos, rp, col, tgt)], prm, [0.5], chains=1,
                       use_graph=False, lanes=2)
    b.run()
    want_pos, want = b.results()
    b.close()
    prob, bufs = _device_problem(torch, r, np.zeros(r.n, np.uint8))
    res = capi.arcs_anneal_noalloc(prob, prm, 0.5, seed, out.data_ptr())
    np.testing.assert_array_equal(out.cpu().numpy().reshape(-1, 3), want_pos[0])
    assert res.moves == want[0].moves and res.energy == want[0].energy


def test_noalloc_rejects_too_many_entries(ctx):
    """16385 arc-list entries (one more than the fixed array holds) on a
    region within the bead limit: PMMC_ERR_BUDGET, output untouched."""
    torch = pytest.importorskip("torch")
    n = 3000
    r = synth.arcs_region(n, 8400, seed=9)
    rp, col, tgt = r.csr()
    assert len(col) >= 16385
    k = next(i for i in range(n + 1) if rp[i] >= 16385)   # the first rows hold 16385 entries
    rp2 = np.minimum(rp, 16385).astype(np.int32)
    rp2[k:] = 16385
    prob, bufs = _device_problem(torch, r, np.zeros(n, np.uint8),
                                 csr=(rp2, col[:16385].copy(), tgt[:16385].copy()))
    out = torch.full((n * 3,), 7.0, dtype=torch.float32, device="cuda")
    prm = capi.default_params(capi.LEVEL_ARCS)
    with pytest.raises(capi.PmmcError) as e:
        capi.arcs_anneal_noalloc(prob, prm, 0.5, 1, out.data_ptr())
    assert e.value.status == capi.PMMC_ERR_BUDGET
    assert (out.cpu().numpy() == 7.0).all()
