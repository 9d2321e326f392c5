"""The seeded synthetic workloads have the shapes and value distributions the
benchmark lines state (they stand in for the reference's ChIA-PET / Hi-C
example data, which it does not ship)."""
import numpy as np

from pmmc_gb300 import synth, workloads


def test_random_walk_has_unit_steps():
    p = synth.random_walk(1000, np.random.default_rng(0))
    steps = np.linalg.norm(np.diff(p.astype(np.float64), axis=0), axis=1)
    assert p.dtype == np.float32 and p.shape == (1000, 3)
    np.testing.assert_allclose(steps, 1.0, atol=1e-5)


def test_plain_region_shape_and_distributions():
    """256 beads, 400 distinct arcs i<j with |i-j| = round(exp U[ln 3, ln 255]),
    PET counts geometric with mean 8, target count^-0.5 |i-j|^0.25."""
    r = workloads.plain_region()
    assert r.n == 256 and len(r.arcs) == 400
    i, j = r.arcs[:, 0], r.arcs[:, 1]
    assert (i < j).all() and len({(a, b) for a, b in r.arcs.tolist()}) == 400
    sep = (j - i).astype(np.float64)
    assert sep.min() >= 3 and sep.max() <= 255
    # log-uniform: ln(sep) spread over [ln 3, ln 255] with its mean near the middle
    assert abs(np.log(sep).mean() - 0.5 * (np.log(3) + np.log(255))) < 0.25
    assert 6.5 < r.count.mean() < 9.5 and r.count.min() >= 1
    want = (r.count.astype(np.float64) ** -0.5 * sep ** 0.25).astype(np.float32)
    np.testing.assert_array_equal(r.target, want)
    d = r.dense()
    assert d.shape == (256, 256) and (np.diag(d) == 0).all()
    assert (d[i, j] == r.target).all() and (d[j, i] == r.target).all()
    assert ((d >= 0).sum() - 256) == 2 * 400


def test_heatmap_region_shape():
    """2048 beads; symmetric expected distances c^-1/3 >= 0 with a zero
    diagonal; 20 non-overlapping TAD blocks boost contacts x3."""
    h = synth.heatmap_region(2048, seed=7)
    assert h.heat.shape == (2048, 2048) and h.heat.dtype == np.float32
    np.testing.assert_array_equal(h.heat, h.heat.T)
    assert (np.diag(h.heat) == 0).all() and (h.heat >= 0).all()
    # away from TADs the expected distance of separation s is (s^-1 * noise)^-1/3:
    # its median over a diagonal is close to s^(1/3)
    for s in (10, 100, 1000):
        med = np.median(np.diagonal(h.heat, s))
        assert 0.7 * s ** (1 / 3) < med < 1.3 * s ** (1 / 3)


def test_genome_smoothing_shape():
    """~300k beads over 23 chromosomes in proportion to the human lengths,
    anchors every Poisson(10) beads (>= 1) fixed, both ends fixed, unit
    bond targets."""
    chains = synth.smooth_genome(300_000, seed=3)
    sizes = np.array([c.n for c in chains])
    assert len(chains) == 23 and abs(sizes.sum() - 300_000) < 100
    mb = np.array(synth.HUMAN_CHR_MB, np.float64)
    np.testing.assert_allclose(sizes / sizes.sum(), mb / mb.sum(), atol=1e-4)
    gaps = np.concatenate([np.diff(np.nonzero(c.fixed)[0]) for c in chains])
    assert gaps.min() >= 1 and 9.0 < gaps.mean() < 11.0
    assert all(c.fixed[0] and c.fixed[-1] for c in chains)
    assert all((c.dist_to_next == 1.0).all() for c in chains)


def test_ensemble_shape():
    """64 structures x 24 blocks, sizes round(exp U[ln 32, ln 2048]) (mean
    about 485 beads), 1.5 arcs per bead."""
    ens = synth.arcs_ensemble(64, 24)
    sizes = np.array([b.n for s in ens for b in s])
    assert len(ens) == 64 and all(len(s) == 24 for s in ens)
    assert sizes.min() >= 32 and sizes.max() <= 2048
    assert 0.85 * 485 < sizes.mean() < 1.15 * 485
    arcs = np.array([len(b.arcs) for s in ens for b in s])
    np.testing.assert_array_equal(arcs, np.rint(1.5 * sizes).astype(int))


def test_inputs_are_seeded():
    a = synth.arcs_region(300, seed=5)
    b = synth.arcs_region(300, seed=5)
    np.testing.assert_array_equal(a.pos, b.pos)
    np.testing.assert_array_equal(a.arcs, b.arcs)
    assert not np.array_equal(a.arcs, synth.arcs_region(300, seed=6).arcs)
