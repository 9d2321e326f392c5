"""Seeded synthetic inputs with the shapes of the benchmark workloads.

The reference's example inputs (ChIA-PET / Hi-C files) are not available, so
every workload is generated here from a seed:

* ``arcs_region``      -- one anchor-level active region: a 3D random walk
  with unit steps, arcs between beads i<j with |i-j| log-uniform in
  [3, n-1], PET counts geometric with mean 8, target distance
  count^-0.5 * |i-j|^0.25.  Returned both as the reference's dense n x n
  matrix (-1 = no arc, 0 on the diagonal, LooperSolver.hpp:5498-5538) and as
  per-bead arc lists (CSR) that the CUDA kernels consume.
* ``heatmap_region``   -- symmetric contact map c_ij = |i-j|^-1 x
  lognormal(0, 0.5), 20 TAD diagonal blocks boosted x3, expected distance
  c^-1/3 (createDistanceHeatmap with freq_dist_scale 1, power -1/3).
* ``smooth_genome``    -- 23 chromosomes with lengths proportional to human
  chr1..22,X at 10 kb per bead, anchors every Poisson(10) beads fixed.
* ``arcs_ensemble``    -- structures x blocks of arc regions with
  log-uniform block sizes.
* ``anchor_targets_problem`` -- one chromosome's anchors (genomic intervals
  of 2-6 kb every ~50 kb), its arcs (1.5 per anchor, spans log-uniform in
  [1, 200] anchors, PET counts geometric with mean 12) and long arcs at
  genomic positions (Hi-C style: spans log-uniform up to the chromosome,
  counts geometric with mean 3), with an active region of consecutive
  anchors: the inputs of calcAnchorExpectedDistancesHeatmap.
* ``stress_problem``   -- the same chromosome as the input of
  stressRefineAnchors: every anchor active in registration order (shuffled
  against the genomic order), positions a random walk with steps of the
  backbone target, power-law count-to-distance constants.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

# Human chromosome lengths in Mb (chr1..chr22, chrX), used only for the
# relative sizes of the genome-scale smoothing workload.
HUMAN_CHR_MB = [248, 242, 198, 190, 181, 171, 159, 145, 138, 134, 135, 133,
                114, 107, 102, 90, 83, 80, 59, 64, 47, 51, 156]


def random_walk(n: int, rng: np.random.Generator, step: float = 1.0) -> np.ndarray:
    """3D random walk with steps of fixed length `step` (float32, (n,3))."""
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    d[0] = 0.0
    return (np.cumsum(d * step, axis=0)).astype(np.float32)


@dataclass
class ArcsRegion:
    pos: np.ndarray          # (n,3) float32
    arcs: np.ndarray         # (m,2) int32, i<j
    target: np.ndarray       # (m,) float32 expected distance
    count: np.ndarray        # (m,) int32 PET counts

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])

    def csr(self):
        """Per-bead arc lists over both directions, columns sorted: the layout
        pmmc_arcs_dense_to_csr produces from dense(), built directly."""
        n = self.n
        i = np.concatenate([self.arcs[:, 0], self.arcs[:, 1]])
        j = np.concatenate([self.arcs[:, 1], self.arcs[:, 0]])
        t = np.concatenate([self.target, self.target])
        order = np.lexsort((j, i))
        i, j, t = i[order], j[order], t[order]
        row_ptr = np.zeros(n + 1, np.int32)
        np.add.at(row_ptr, i + 1, 1)
        row_ptr = np.cumsum(row_ptr).astype(np.int32)
        return row_ptr, j.astype(np.int32), t.astype(np.float32)

    def dense(self) -> np.ndarray:
        """The reference layout: -1 everywhere, 0 on the diagonal, targets on
        arc pairs (both triangles)."""
        n = self.n
        m = np.full((n, n), -1.0, np.float32)
        np.fill_diagonal(m, 0.0)
        m[self.arcs[:, 0], self.arcs[:, 1]] = self.target
        m[self.arcs[:, 1], self.arcs[:, 0]] = self.target
        return m


def arcs_region(n: int = 256, n_arcs: int = 400, seed: int = 42,
                mean_count: float = 8.0, arcs_per_bead: float | None = None) -> ArcsRegion:
    """Arcs i<j with |i-j| = round(exp U[ln 3, ln(n-1)]), i uniform, PET
    counts geometric with the given mean; distinct pairs in draw order."""
    rng = np.random.default_rng(seed)
    pos = random_walk(n, rng)
    if arcs_per_bead is not None:
        n_arcs = int(round(arcs_per_bead * n))
    max_sep = n - 1
    n_arcs = max(0, min(n_arcs, n * (n - 1) // 2 - (n - 1) * 2))
    keys = np.zeros(0, np.int64)
    counts = np.zeros(0, np.int64)
    lo = np.log(3.0)
    hi = np.log(max(max_sep, 3))
    for _ in range(64):
        need = n_arcs - len(keys)
        if need <= 0:
            break
        m = 2 * need + 16
        sep = np.rint(np.exp(rng.uniform(lo, hi, m))).astype(np.int64)
        sep = np.clip(sep, min(3, max_sep), max_sep)
        i = (rng.random(m) * (n - sep)).astype(np.int64)
        cnt = rng.geometric(1.0 / mean_count, m)
        keys = np.concatenate([keys, i * n + i + sep])
        counts = np.concatenate([counts, cnt])
        _, first = np.unique(keys, return_index=True)
        first = np.sort(first)
        keys, counts = keys[first], counts[first]
    keys, counts = keys[:n_arcs], counts[:n_arcs]
    order = np.argsort(keys)
    keys, counts = keys[order], counts[order]
    arcs = np.stack([keys // n, keys % n], 1).astype(np.int32).reshape(-1, 2)
    count = counts.astype(np.int32)
    sepf = (arcs[:, 1] - arcs[:, 0]).astype(np.float64)
    target = (count.astype(np.float64) ** -0.5 * sepf ** 0.25).astype(np.float32)
    return ArcsRegion(pos, arcs, target, count)


@dataclass
class HeatmapRegion:
    pos: np.ndarray      # (n,3) float32
    heat: np.ndarray     # (n,n) float32 expected distances (0 = ignore)
    diag: int
    bounds: np.ndarray   # chromosome boundaries ([] = one block)

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])


def heatmap_region(n: int = 2048, seed: int = 7, n_tads: int = 20,
                   tad_min: int = 40, tad_max: int = 200, sigma: float = 0.5,
                   diag: int = 1) -> HeatmapRegion:
    rng = np.random.default_rng(seed)
    pos = random_walk(n, rng)
    i = np.arange(n)
    sep = np.abs(i[:, None] - i[None, :]).astype(np.float64)
    noise = rng.lognormal(0.0, sigma, size=(n, n))
    noise = np.triu(noise, 1)
    noise = noise + noise.T
    with np.errstate(divide="ignore"):
        c = np.where(sep > 0, 1.0 / np.maximum(sep, 1.0), 0.0) * noise
    # TAD blocks: non-overlapping diagonal blocks boosted x3
    placed = []
    tries = 0
    while len(placed) < n_tads and tries < 10000:
        tries += 1
        size = int(rng.integers(tad_min, tad_max + 1))
        if size >= n:
            continue
        s = int(rng.integers(0, n - size))
        if any(not (s + size <= a or b <= s) for a, b in placed):
            continue
        placed.append((s, s + size))
    for a, b in placed:
        c[a:b, a:b] *= 3.0
    with np.errstate(divide="ignore"):
        h = np.where(c > 0, c ** (-1.0 / 3.0), 0.0)
    h = h.astype(np.float32)
    np.fill_diagonal(h, 0.0)
    return HeatmapRegion(pos, h, diag, np.zeros(0, np.int32))


@dataclass
class SmoothChain:
    pos: np.ndarray          # (n,3) float32
    fixed: np.ndarray        # (n,) uint8
    dist_to_next: np.ndarray # (n,) float64
    chrom_start: np.ndarray  # chromosome first-bead offsets (+ total at end)

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])


def smooth_chain(n: int, seed: int = 3, gap_mean: float = 10.0,
                 bond: float = 1.0) -> SmoothChain:
    """One chromosome: anchors every Poisson(gap_mean) (>=1) beads held fixed
    at random-walk positions; free beads start on the straight line between
    anchors plus noise."""
    rng = np.random.default_rng(seed)
    walk = random_walk(n, rng, step=bond)
    fixed = np.zeros(n, np.uint8)
    k = 0
    while k < n:
        fixed[k] = 1
        k += max(1, int(rng.poisson(gap_mean)))
    fixed[n - 1] = 1
    pos = walk.copy()
    anchors = np.nonzero(fixed)[0]
    for a, b in zip(anchors[:-1], anchors[1:]):
        if b - a > 1:
            t = (np.arange(a + 1, b) - a) / (b - a)
            pos[a + 1:b] = walk[a] + (walk[b] - walk[a]) * t[:, None]
    pos += (rng.normal(size=pos.shape) * 0.25 * (1 - fixed[:, None])).astype(np.float32)
    dtn = np.full(n, bond, np.float64)
    return SmoothChain(pos.astype(np.float32), fixed, dtn, np.array([0, n], np.int64))


def smooth_genome(total_beads: int = 300_000, seed: int = 3) -> list[SmoothChain]:
    """23 chromosomes with lengths proportional to HUMAN_CHR_MB summing to
    about total_beads."""
    mb = np.array(HUMAN_CHR_MB, np.float64)
    sizes = np.maximum(16, np.round(mb / mb.sum() * total_beads)).astype(int)
    return [smooth_chain(int(s), seed=seed * 1000 + c) for c, s in enumerate(sizes)]


def ensemble_block_specs(n_structures: int = 64, n_blocks: int = 24, min_size: int = 32,
                         max_size: int = 2048, seeds=None) -> list[list[tuple[int, int]]]:
    """(beads, region seed) of every block: structures x blocks, block sizes
    log-uniform in [min_size, max_size], structure s drawn from seed s."""
    out = []
    seeds = list(range(n_structures)) if seeds is None else list(seeds)
    for s in seeds:
        rng = np.random.default_rng(10_000 + s)
        out.append([(int(round(np.exp(rng.uniform(np.log(min_size), np.log(max_size))))),
                     s * 1000 + b) for b in range(n_blocks)])
    return out


def arcs_ensemble(n_structures: int = 64, n_blocks: int = 24, min_size: int = 32,
                  max_size: int = 2048, arcs_per_bead: float = 1.5,
                  seeds=None) -> list[list[ArcsRegion]]:
    """structures x blocks arc regions (ensemble_block_specs); block (s, b)
    is arcs_region(size, seed=1000 s + b)."""
    return [[arcs_region(n, seed=seed, arcs_per_bead=arcs_per_bead) for n, seed in blocks]
            for blocks in ensemble_block_specs(n_structures, n_blocks, min_size, max_size, seeds)]


def freq_memo(count_a: float, count_scale: float, count_shift: float,
              count_base: float) -> np.ndarray:
    """The reference's freq_to_distance table (LooperSolver.hpp:950-951 fills
    2..100 with freqToDistance(i, false)); entry 1 is filled the same way
    here, entry 0 is 0."""
    m = np.zeros(101, np.float32)
    for i in range(1, 101):
        fs = np.float32(np.float32(i) + np.float32(count_shift))
        if count_a < 0:
            fi = max(int(fs), 1)
            v = float(np.float32(count_base)) + float(np.float32(count_scale)) * \
                float(fi) ** float(np.float32(count_a))
        else:
            v = float(np.float32(count_base)) + float(np.float32(count_scale)) / \
                np.exp(float(np.float32(count_a)) * float(fs))
        m[i] = np.float32(v)
    return m


def anchor_targets_problem(n_anchors: int = 4000, n_active: int | None = None,
                           active_from: int = 0, arcs_per_anchor: float = 1.5,
                           n_long: int = 100_000, seed: int = 21, first_cluster: int = 7,
                           count=(0.5, 20.0, 1.0, 0.01), heat: bool = False,
                           influence: float = 0.5, outside_arcs: int = 0,
                           duplicate_arcs: int = 0) -> dict:
    """Inputs of calcAnchorExpectedDistancesHeatmap for one chromosome as a
    dict (the keys of capi.anchor_targets_arrays).  The active region is
    anchors [active_from, active_from + n_active) as cluster indices
    first_cluster + anchor; `outside_arcs` arcs reach from the region to
    anchors outside it, `duplicate_arcs` repeat an existing pair with
    another count."""
    rng = np.random.default_rng(seed)
    n_active = n_anchors if n_active is None else n_active
    gap = rng.integers(40_000, 60_000, n_anchors).astype(np.int64)
    start = np.cumsum(gap) + 10_000
    length = rng.integers(2_000, 6_000, n_anchors)
    anc_start = start.astype(np.int32)
    anc_end = (start + length).astype(np.int32)
    lo, hi = active_from, active_from + n_active
    n_arcs = int(round(arcs_per_anchor * n_active))
    a = rng.integers(lo, hi - 1, n_arcs)
    span = np.exp(rng.uniform(0.0, np.log(200.0), n_arcs)).astype(np.int64)
    b = np.minimum(a + np.maximum(span, 1), hi - 1)
    keep = b > a
    a, b = a[keep], b[keep]
    score = rng.geometric(1.0 / 12.0, len(a)).astype(np.int64)
    pairs = [(int(x), int(y), int(z)) for x, y, z in zip(a, b, score)]
    for _ in range(outside_arcs):
        x = int(rng.integers(lo, hi))
        y = int(rng.integers(0, n_anchors))
        if y < lo or y >= hi:
            pairs.append((min(x, y), max(x, y), int(rng.geometric(1.0 / 12.0))))
    for _ in range(duplicate_arcs):
        if pairs:
            x, y, _s = pairs[int(rng.integers(0, len(pairs)))]
            pairs.append((x, y, int(rng.geometric(1.0 / 12.0))))
    pairs.sort()
    arc_start = np.array([first_cluster + x for x, _, _ in pairs], np.int32)
    arc_end = np.array([first_cluster + y for _, y, _ in pairs], np.int32)
    arc_score = np.array([z for _, _, z in pairs], np.int32)
    active = np.arange(first_cluster + lo, first_cluster + hi, dtype=np.int32)
    per = [[] for _ in range(n_active)]
    for k, (x, y, _) in enumerate(pairs):
        for c in (x, y):
            if lo <= c < hi:
                per[c - lo].append(k)
    arc_ptr = np.zeros(n_active + 1, np.int32)
    arc_ptr[1:] = np.cumsum([len(p) for p in per])
    arc_idx = np.array([k for p in per for k in p], np.int32)
    # long arcs: one end inside an anchor of the chromosome most of the time
    chrom_end = int(anc_end[-1]) + 20_000
    i0 = rng.integers(0, n_anchors, n_long)
    p0 = anc_start[i0] + rng.integers(-500, 6_500, n_long)
    sp = np.exp(rng.uniform(np.log(5e4), np.log(chrom_end), n_long)).astype(np.int64)
    p1 = p0 + sp
    miss = rng.random(n_long) < 0.3        # land between anchors
    nxt = np.searchsorted(anc_start, p1)   # beyond the last anchor: stays outside
    p1 = np.where(miss | (nxt >= n_anchors), p1,
                  anc_start[np.minimum(nxt, n_anchors - 1)] + 100)
    long_start = np.minimum(p0, chrom_end).astype(np.int32)
    long_end = np.minimum(p1, chrom_end).astype(np.int32)
    long_score = rng.geometric(1.0 / 3.0, n_long).astype(np.int32)
    long_score[rng.random(n_long) < 0.01] += 100   # counts above the memo table
    t = {"active": active, "arc_ptr": arc_ptr, "arc_idx": arc_idx, "arc_start": arc_start,
         "arc_end": arc_end, "arc_score": arc_score, "long_start": long_start,
         "long_end": long_end, "long_score": long_score, "anc_start": anc_start,
         "anc_end": anc_end, "first_cluster": first_cluster,
         "memo": freq_memo(*count), "count": tuple(count), "heat": None,
         "influence": influence}
    if heat:
        n = n_active
        i = np.arange(n)
        sep = np.abs(i[:, None] - i[None, :]).astype(np.float32)
        h = np.where(sep >= 2, 1.0 / np.maximum(sep, 1.0), 0.0).astype(np.float32)
        h *= rng.lognormal(0.0, 0.5, (n, n)).astype(np.float32)
        t["heat"] = h
    return t


def stress_problem(n_anchors: int = 4000, n_long: int = 200_000, seed: int = 51,
                   count=(-0.5, 10.0, 0.0, 0.5), glen=(0.0, 1.0, 0.5),
                   springs=(0.1, 0.1, 0.1), shuffle: bool = True,
                   arcs_per_anchor: float = 1.5, first_cluster: int = 7) -> dict:
    """Inputs of stressRefineAnchors for one chromosome (the keys of
    capi.stress_arrays)."""
    t = anchor_targets_problem(n_anchors=n_anchors, n_long=n_long, seed=seed,
                               arcs_per_anchor=arcs_per_anchor, first_cluster=first_cluster)
    rng = np.random.default_rng(seed + 1)
    center = ((t["anc_start"].astype(np.int64) + t["anc_end"]) // 2).astype(np.int32)
    order = rng.permutation(n_anchors) if shuffle else np.arange(n_anchors)
    step = float(np.sqrt(50.0)) * float(glen[1])
    pos = random_walk(n_anchors, rng, step)
    return {"active": (first_cluster + order).astype(np.int32),
            "genomic_pos": center[order], "pos": pos[order],
            "arc_start": t["arc_start"], "arc_end": t["arc_end"], "arc_score": t["arc_score"],
            "long_start": t["long_start"], "long_end": t["long_end"],
            "long_score": t["long_score"], "anc_start": t["anc_start"],
            "anc_end": t["anc_end"], "first_cluster": first_cluster, "count": tuple(count),
            "glen": tuple(glen), "springs": tuple(springs)}
