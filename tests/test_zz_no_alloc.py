"""The allocation-free arc-level entry point (pmmc_arcs_anneal_noalloc).

It serves callers that may not allocate device memory: the test plays such a
caller, owning every device buffer itself (torch tensors stand in for the
caller's pool) and passing only their addresses through the C ABI.  Two calls
in a row must reproduce the regular batched entry point with one chain (same
key and chain), the second call running on the scratch array the first one
left behind.  This file is named so that pytest collects it last.
"""
import numpy as np
import pytest

from pmmc_gb300 import capi, synth

pytestmark = pytest.mark.gpu

TOL = 1e-5  # the per-move tolerance of the other parity tests


def _device_problem(torch, r, fixed):
    rp, col, tgt = r.csr()
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
        assert res.moves == want[0].moves and res.status == 0, call
        np.testing.assert_allclose(got, want_pos[0], rtol=0, atol=TOL)
        assert abs(res.energy - want[0].energy) <= TOL * abs(want[0].energy)
        assert abs(res.energy_fp64 - want[0].energy_fp64) <= TOL * abs(want[0].energy_fp64)
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
