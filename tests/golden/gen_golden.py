"""Writes the golden fixtures of the parity tests from the REFERENCE itself.

Runs where the reference sources exist: oracle/Makefile builds
oracle/_ref/libpmmc_ref.so from them (the reference's own LooperSolver /
InteractionArcs CPU code behind a C harness) and this script records its
outputs on small seeded inputs into tests/golden/*.npz.  The tests then pin
the plain-C oracle against these files on any machine, including ones without
the reference tree.

    python tests/golden/gen_golden.py            # every group
    python tests/golden/gen_golden.py ext        # only the named groups
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402
from pmmc_gb300 import synth  # noqa: E402


def params_array(p: O.Params) -> np.ndarray:
    return np.array([getattr(p, f) for f, _ in O.OrcParams._fields_], np.float64)


def arcs_cases():
    out = {}
    # 1: config-0 shape scaled down; 2: loops + sphere + a fixed-free region;
    # 3: 2D moves
    specs = [
        dict(n=64, arcs=100, seed=1, loops=0, sphere=0.0, use2d=0, steps=2000),
        dict(n=48, arcs=60, seed=2, loops=6, sphere=6.0, use2d=0, steps=1500),
        dict(n=40, arcs=50, seed=3, loops=0, sphere=0.0, use2d=1, steps=1000),
    ]
    for k, sp in enumerate(specs):
        r = synth.arcs_region(sp["n"], sp["arcs"], seed=sp["seed"])
        dense = r.dense()
        rng = np.random.default_rng(100 + k)
        li = rng.integers(0, sp["n"], sp["loops"]).astype(np.int32)
        lj = rng.integers(0, sp["n"], sp["loops"]).astype(np.int32)
        lk = rng.uniform(0.5, 2.0, sp["loops"]).astype(np.float32)
        lr = rng.uniform(1.0, 3.0, sp["loops"]).astype(np.float32)
        pr = O.ArcsProblem(r.pos, dense, None, li, lj, lk, lr)
        prm = O.Params(max_temp=5.0, dt_temp=0.9999, milestone_steps=sp["steps"],
                       improvement=0.99, sphere_radius=sp["sphere"], use2d=sp["use2d"])
        beads = np.array([0, 1, sp["n"] // 2, sp["n"] - 1], np.int32)
        local = np.array([O.ref_arcs_score(pr, prm, int(b)) for b in beads])
        full = O.ref_arcs_score(pr, prm, -1)
        pos, score, moves = O.ref_arcs_anneal(pr, prm, 0.5, 1000 + k)
        out[f"arcs{k}"] = dict(pos=r.pos, dense=dense, li=li, lj=lj, lk=lk, lr=lr,
                               params=params_array(prm), beads=beads, local=local,
                               full=np.array([full]), step=np.array([0.5]),
                               seed=np.array([1000 + k]), out_pos=pos,
                               out_score=np.array([score]), out_moves=np.array([moves]))
    return out


def ext_cases():
    """The extended arc energy's two terms from the reference's own
    functions: calcScoreStructureActiveRegionLengths (bonds) and
    calcScoreStructureSmooth (bonds + angles, weights 1)."""
    out = {}
    for k, (n, t, ks, kq, ka) in enumerate([(64, 1.0, 0.1, 0.1, 0.1), (33, 0.7, 0.3, 0.05, 0.4)]):
        rng = np.random.default_rng(500 + k)
        pos = (synth.random_walk(n, rng) * 1.1 +
               rng.normal(0.0, 0.25, (n, 3))).astype(np.float32)
        dtn = np.full(n, t, np.float64)
        lp = O.Params(k_stretch=ks, k_squeeze=kq, k_angle=0.0, w_dist=1.0, w_angle=1.0)
        sp = O.Params(k_stretch=ks, k_squeeze=kq, k_angle=ka, w_dist=1.0, w_angle=1.0)
        beads = np.array([0, 1, 2, n // 2, n - 2, n - 1], np.int32)
        sm = O.SmoothProblem(pos, dtn)
        out[f"ext{k}"] = dict(
            pos=pos, ext=np.array([t, ks, kq, ka], np.float64), beads=beads,
            len_full=np.array([O.ref_lengths_score(n, pos, dtn, lp, -1)]),
            len_local=np.array([O.ref_lengths_score(n, pos, dtn, lp, int(b)) for b in beads]),
            all_full=np.array([O.ref_smooth_score(sm, sp, -1)]),
            all_local=np.array([O.ref_smooth_score(sm, sp, int(b)) for b in beads]))
    return out


def distmap_cases():
    """createDistanceHeatmap of the reference on seeded contact maps: |i-j|^-1
    decay with lognormal noise, zeros, a band of diag diagonals."""
    out = {}
    for k, (n, diag, level, scale, power, stretch) in enumerate(
            [(64, 1, 1, 100.0, -0.333, 2.0), (97, 2, 0, 100.0, -1.0, 2.0),
             (80, 1, 1, 1.0, -1.0 / 3.0, 1.5)]):
        rng = np.random.default_rng(700 + k)
        i = np.arange(n)
        sep = np.abs(i[:, None] - i[None, :]).astype(np.float64)
        c = np.where(sep > 0, 1.0 / np.maximum(sep, 1.0), 2.0) * rng.lognormal(0.0, 0.5, (n, n))
        c[rng.random((n, n)) < 0.1] = 0.0           # missing contacts
        c = np.triu(c) + np.triu(c, 1).T            # symmetric input
        c = c.astype(np.float32)
        d = O.ref_distance_heatmap(c, diag, level, scale, power, stretch)
        out[f"distmap{k}"] = dict(contact=c, params=np.array([diag, scale, power, stretch]),
                                  dist=d)
    return out


def equi_cases():
    """The reference's equidistant-model interpolation (gpuHelper, CPU path)
    on seeded chromosome levels: uneven cluster spacing, a 2-cluster level,
    resolutions that do and do not divide the span."""
    out = {}
    for k, (n, res) in enumerate([(40, 1000), (2, 333), (300, 7919), (17, 50)]):
        rng = np.random.default_rng(800 + k)
        width = rng.integers(500, 30000, n)
        start = np.concatenate([[10_000], 10_000 + np.cumsum(width)[:-1]]).astype(np.int32)
        end = (start + width - 1).astype(np.int32)
        gpos = ((start + end) // 2).astype(np.int32)
        pos = synth.random_walk(n, rng) * np.float32(2.0)
        pts = O.ref_equidistant(gpos, start, end, pos, int(gpos[0]), int(gpos[-1]), res)
        out[f"equi{k}"] = dict(gpos=gpos, start=start, end=end, pos=pos,
                               res=np.array([res]), points=pts)
    return out


def heatmap_cases():
    out = {}
    specs = [dict(n=64, diag=1, bounds=[], sphere=0.0, seed=4),
             dict(n=72, diag=2, bounds=[0, 30, 72], sphere=5.0, seed=5)]
    for k, sp in enumerate(specs):
        h = synth.heatmap_region(sp["n"], seed=sp["seed"], n_tads=3, tad_min=8, tad_max=16)
        fixed = np.zeros(sp["n"], np.uint8)
        fixed[0] = 1
        pr = O.HeatmapProblem(h.pos, h.heat, sp["diag"], np.array(sp["bounds"], np.int32), fixed)
        prm = O.Params(max_temp=5.0, dt_temp=0.9999, milestone_steps=400, improvement=0.99,
                       sphere_radius=sp["sphere"])
        beads = np.array([0, 5, sp["n"] - 1], np.int32)
        local = np.array([O.ref_heatmap_score(pr, int(b)) for b in beads])
        full = O.ref_heatmap_score(pr, -1)
        pos, score, moves = O.ref_heatmap_anneal(pr, prm, 1.0, 2000 + k)
        out[f"heatmap{k}"] = dict(pos=h.pos, heat=h.heat, diag=np.array([sp["diag"]]),
                                  bounds=np.array(sp["bounds"], np.int32), fixed=fixed,
                                  params=params_array(prm), beads=beads, local=local,
                                  full=np.array([full]), step=np.array([1.0]),
                                  seed=np.array([2000 + k]), out_pos=pos,
                                  out_score=np.array([score]), out_moves=np.array([moves]))
    return out


def smooth_cases():
    out = {}
    specs = [dict(n=60, seed=6, w=(1.0, 1.0), sphere=0.0),
             dict(n=50, seed=7, w=(0.7, 1.3), sphere=8.0)]
    for k, sp in enumerate(specs):
        c = synth.smooth_chain(sp["n"], seed=sp["seed"])
        dtn = c.dist_to_next.copy()
        dtn[3] = 0.0  # exercises the 1e-6 clamp
        pr = O.SmoothProblem(c.pos, dtn, c.fixed)
        prm = O.Params(max_temp=5.0, dt_temp=0.9999, milestone_steps=800, improvement=0.99,
                       k_stretch=0.1, k_squeeze=0.1, k_angle=0.1, w_dist=sp["w"][0],
                       w_angle=sp["w"][1], sphere_radius=sp["sphere"])
        beads = np.array([0, 1, 2, sp["n"] // 2, sp["n"] - 2, sp["n"] - 1], np.int32)
        local = np.array([O.ref_smooth_score(pr, prm, int(b)) for b in beads])
        full = O.ref_smooth_score(pr, prm, -1)
        pos, score, moves = O.ref_smooth_anneal(pr, prm, 0.5, 3000 + k)
        out[f"smooth{k}"] = dict(pos=c.pos, dtn=dtn, fixed=c.fixed, params=params_array(prm),
                                 beads=beads, local=local, full=np.array([full]),
                                 step=np.array([0.5]), seed=np.array([3000 + k]),
                                 out_pos=pos, out_score=np.array([score]),
                                 out_moves=np.array([moves]))
    return out


def mark_cases():
    out = {}
    rng = np.random.default_rng(8)
    starts = np.sort(rng.choice(50_000, 30, replace=False)) * 20
    anchors = np.stack([starts, starts + rng.integers(0, 4000, 30)], 1).astype(np.int32)
    anchors[3] = [anchors[3, 0], anchors[3, 0]]       # length 1: never matches
    anchors[5, 1] = anchors[6, 1] + 10               # overlaps the next anchor
    raw = []
    for _ in range(250):  # arcs between anchors (duplicates, factors, self loops)
        i, j = rng.integers(0, 30, 2)
        raw.append([int(rng.integers(anchors[i, 0], anchors[i, 1] + 1)),
                    int(rng.integers(anchors[j, 0], anchors[j, 1] + 1)),
                    int(rng.integers(1, 12)), int(rng.integers(0, 3))])
    for _ in range(40):   # arcs outside every anchor
        a, b = sorted(rng.integers(0, 1_000_000, 2))
        raw.append([int(a), int(b), int(rng.integers(1, 5)), 0])
    raw += raw[:10]       # exact duplicates
    raw = np.array(raw, np.int32)
    ref = O.ref_mark_arcs(anchors, raw)
    out["mark0"] = dict(anchors=anchors, raw=raw, arcs=ref)
    return out


def hcm_cases():
    lines = [O.hcm_cluster_line(10, 20, "N", (1.5, -2.25, 3.125), [4, 5], use_ref=True),
             O.hcm_cluster_line(0, 0, "L", (1e-7, 123456.789, -0.5), [], use_ref=True),
             O.hcm_arc_line([1, 2, 300, 400, 5, 6, -1], use_ref=True),
             O.hcm_arc_line([7, 9, -1, -1, 0, 12, 2], use_ref=True)]
    return {"hcm": dict(lines=np.array(lines))}


TARGET_KEYS = ("active", "arc_ptr", "arc_idx", "arc_start", "arc_end", "arc_score",
               "long_start", "long_end", "long_score", "anc_start", "anc_end", "memo")


def target_specs():
    """The anchor-target cases: problem dicts for synth.anchor_targets_problem
    plus edits that reach the reference's corner cases."""
    out = []
    # arcs leaving the active region (slot 0 through std::map insertion),
    # repeated pairs (the last write wins), collisions with long arcs
    out.append(synth.anchor_targets_problem(n_anchors=300, n_active=200, active_from=50,
                                            n_long=3000, seed=31, outside_arcs=12,
                                            duplicate_arcs=12))
    # power-law counts (countToDistA < 0) and the anchor heatmap's influence
    out.append(synth.anchor_targets_problem(n_anchors=300, n_active=200, active_from=50,
                                            n_long=3000, seed=32, heat=True,
                                            count=(-0.5, 2.0, 0.0, 0.1), influence=3.0))
    # overlapping, unsorted anchors: the first anchor holding a position wins
    t = synth.anchor_targets_problem(n_anchors=120, n_active=120, n_long=2000, seed=33)
    t["anc_end"] = t["anc_end"].copy()
    t["anc_end"][10] = t["anc_start"][12] + 100
    t["anc_start"] = t["anc_start"].copy()
    t["anc_start"][40], t["anc_start"][41] = t["anc_start"][41], t["anc_start"][40]
    t["anc_end"][40], t["anc_end"][41] = t["anc_end"][41], t["anc_end"][40]
    out.append(t)
    # negative distances (countToDistBaseLevel < 0): long arcs overwrite them
    out.append(synth.anchor_targets_problem(n_anchors=200, n_active=150, active_from=20,
                                            n_long=3000, seed=34,
                                            count=(0.5, 20.0, 1.0, -0.005)))
    # no anchor list: long arcs unused; a tiny region
    t = synth.anchor_targets_problem(n_anchors=12, n_active=12, n_long=50, seed=35)
    t["anc_start"] = t["anc_start"][:0]
    t["anc_end"] = t["anc_end"][:0]
    out.append(t)
    return out


def target_cases():
    out = {}
    for k, t in enumerate(target_specs()):
        dense, st = O.ref_anchor_targets(t)
        d = {key: np.asarray(t[key]) for key in TARGET_KEYS}
        d["first_cluster"] = np.array([t["first_cluster"]], np.int32)
        d["count"] = np.array(t["count"], np.float32)
        d["heat"] = np.zeros((0, 0), np.float32) if t["heat"] is None else t["heat"]
        d["influence"] = np.array([t["influence"]], np.float32)
        d["dense"] = dense
        d["stats"] = np.array([st["applied"], st["out_of_range"], st["inactive"],
                               st["collision"]], np.int64)
        out[f"targets{k}"] = d
    return out


STRESS_KEYS = ("active", "genomic_pos", "pos", "arc_start", "arc_end", "arc_score",
               "long_start", "long_end", "long_score", "anc_start", "anc_end")


def stress_specs():
    """(problem, max_iter, lr) of the stress-refinement cases."""
    return [
        # defaults: converges after the step was halved once
        (synth.stress_problem(n_anchors=120, n_long=2000, seed=51), 300, 0.05),
        # no backbone: consecutive anchors stay in the pair list
        (synth.stress_problem(n_anchors=200, n_long=3000, seed=52, springs=(0.0, 0.0, 0.1)),
         200, 0.05),
        # no angle term, squeeze stiffer than stretch
        (synth.stress_problem(n_anchors=150, n_long=2000, seed=53, springs=(0.1, 0.2, 0.0)),
         500, 0.05),
        # a large step: repeated halving, then convergence
        (synth.stress_problem(n_anchors=80, n_long=1000, seed=54), 400, 5.0),
        # no angle term, a long run to max_iter
        (synth.stress_problem(n_anchors=80, n_long=1000, seed=55, springs=(0.1, 0.1, 0.0)),
         3000, 0.05),
    ]


def stress_cases():
    out = {}
    for k, (t, it, lr) in enumerate(stress_specs()):
        order, pos = O.ref_stress_refine(t, it, lr)
        d = {key: np.asarray(t[key]) for key in STRESS_KEYS}
        d["first_cluster"] = np.array([t["first_cluster"]], np.int32)
        d["count"] = np.array(t["count"], np.float32)
        d["glen"] = np.array(t["glen"], np.float32)
        d["springs"] = np.array(t["springs"], np.float32)
        d["max_iter"] = np.array([it], np.int32)
        d["lr"] = np.array([lr], np.float32)
        d["order"] = order
        d["out_pos"] = pos
        out[f"stress{k}"] = d
    return out


def edge_cases():
    """The smallest and degenerate regions the reference's CPU annealers
    still finish on: a 2-bead region with one arc, a 3-bead region, a region
    without arcs (repulsion only), heatmap regions with one to five free
    beads and a diagonal band wider than most of the map, and smoothing
    chains of three and four beads (ends fixed).  Regions whose beads are all
    fixed are left out: the reference's heatmap and smoothing annealers
    redraw a bead until a free one comes up and never return on them, its
    arc annealer stops the program."""
    out = {}
    for k, (n, arcs, seed) in enumerate([(2, 1, 9), (3, 2, 9), (16, 0, 9), (5, 3, 9)]):
        r = synth.arcs_region(n, max(arcs, 1), seed=seed)
        dense = r.dense()
        if arcs == 0:
            dense[:] = -1.0
        z = np.zeros(0, np.int32)
        zf = np.zeros(0, np.float32)
        pr = O.ArcsProblem(r.pos, dense, None, z, z, zf, zf)
        prm = O.Params(max_temp=5.0, dt_temp=0.9999, milestone_steps=500, improvement=0.99)
        beads = np.arange(n, dtype=np.int32)
        pos, score, moves = O.ref_arcs_anneal(pr, prm, 0.5, 77 + k)
        out[f"edge_arcs{k}"] = dict(
            pos=r.pos, dense=dense, li=z, lj=z, lk=zf, lr=zf, params=params_array(prm),
            beads=beads, local=np.array([O.ref_arcs_score(pr, prm, int(b)) for b in beads]),
            full=np.array([O.ref_arcs_score(pr, prm, -1)]), step=np.array([0.5]),
            seed=np.array([77 + k]), out_pos=pos, out_score=np.array([score]),
            out_moves=np.array([moves]))
    for k, (n, diag, n_free) in enumerate([(4, 1, 3), (8, 3, 2), (6, 1, 5)]):
        h = synth.heatmap_region(n, seed=11, n_tads=1, tad_min=2, tad_max=3)
        fixed = np.ones(n, np.uint8)
        fixed[1:1 + n_free] = 0
        pr = O.HeatmapProblem(h.pos, h.heat, diag, np.zeros(0, np.int32), fixed)
        prm = O.Params(max_temp=5.0, dt_temp=0.9999, milestone_steps=300, improvement=0.99)
        beads = np.arange(n, dtype=np.int32)
        pos, score, moves = O.ref_heatmap_anneal(pr, prm, 1.0, 5 + k)
        out[f"edge_heatmap{k}"] = dict(
            pos=h.pos, heat=h.heat, diag=np.array([diag]), bounds=np.zeros(0, np.int32),
            fixed=fixed, params=params_array(prm), beads=beads,
            local=np.array([O.ref_heatmap_score(pr, int(b)) for b in beads]),
            full=np.array([O.ref_heatmap_score(pr, -1)]), step=np.array([1.0]),
            seed=np.array([5 + k]), out_pos=pos, out_score=np.array([score]),
            out_moves=np.array([moves]))
    for k, (n, sphere) in enumerate([(3, 0.0), (4, 2.0)]):
        c = synth.smooth_chain(n, seed=12)
        dtn = c.dist_to_next.copy()
        pr = O.SmoothProblem(c.pos, dtn, c.fixed)
        prm = O.Params(max_temp=5.0, dt_temp=0.9999, milestone_steps=300, improvement=0.99,
                       k_stretch=0.1, k_squeeze=0.1, k_angle=0.1, w_dist=1.0, w_angle=1.0,
                       sphere_radius=sphere)
        beads = np.arange(n, dtype=np.int32)
        pos, score, moves = O.ref_smooth_anneal(pr, prm, 0.5, 6 + k)
        out[f"edge_smooth{k}"] = dict(
            pos=c.pos, dtn=dtn, fixed=c.fixed, params=params_array(prm), beads=beads,
            local=np.array([O.ref_smooth_score(pr, prm, int(b)) for b in beads]),
            full=np.array([O.ref_smooth_score(pr, prm, -1)]), step=np.array([0.5]),
            seed=np.array([6 + k]), out_pos=pos, out_score=np.array([score]),
            out_moves=np.array([moves]))
    return out


def main():
    if not O.ref_available():
        O.build()
    if not O.ref_available():
        raise SystemExit("the reference harness could not be built (no reference tree)")
    # optional arguments name the groups to write (default: all of them)
    groups = {"arcs": arcs_cases, "ext": ext_cases, "distmap": distmap_cases,
              "equi": equi_cases,
              "heatmap": heatmap_cases,
              "smooth": smooth_cases, "mark": mark_cases, "hcm": hcm_cases,
              "targets": target_cases, "stress": stress_cases, "edge": edge_cases}
    want = sys.argv[1:] or list(groups) + ["rng"]
    fixtures = {}
    for g in want:
        if g in groups:
            fixtures.update(groups[g]())
    if "rng" in want:
        fixtures["rng"] = dict(random_vectors=O.ref_random_vectors(5, 4, 1.0, False),
                               random_vectors_2d=O.ref_random_vectors(6, 4, 1.0, True))
    for name, d in fixtures.items():
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), **d)
    print("wrote", len(fixtures), "fixtures")


if __name__ == "__main__":
    main()
