/*
 * ref_harness.cpp -- drives the REFERENCE's own CPU code (SFGLab/pMMC,
 * header-only LooperSolver / InteractionArcs) through a C ABI.
 *
 * TEST INFRASTRUCTURE ONLY.  oracle/Makefile compiles this file together with
 * the reference's sources where they lie (its src/include headers and
 * src/thirdparty/*.cpp) into oracle/_ref/libpmmc_ref.so.  Tests use it to pin
 * the plain-C oracle (pmmc_oracle.c) bit for bit, and
 * tests/golden/gen_golden.py uses it to write the golden fixtures that travel
 * with the repository.  No reference source is copied here: this file only
 * fills the reference's data structures and calls its functions.
 *
 * The header-only classes keep their state private; the harness opens them
 * with `#define private public` after including every standard header first
 * (the reference's common.h defines `epsilon`, which would break <random>).
 */
#include <algorithm>
#include <array>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <numeric>
#include <queue>
#include <random>
#include <set>
#include <sstream>
#include <unordered_map>
#include <vector>

#include <fcntl.h>
#include <unistd.h>

#define private public
#define protected public
#include <AppCommon.hpp>
#include <Static.hpp>
#include <LooperSolver.hpp>
#include <MetricsFramework.hpp>
#undef private
#undef protected

#include "pmmc_oracle.h"

/* The CPU-only harness holds no device resources; LooperSolver's destructor
 * still references this member of its GPU cache. */
void GpuResourceCache::cleanup() {}

namespace {

/* Silence the reference's progress printing for the duration of a call. */
struct Quiet {
  int saved = -1;
  Quiet() {
    fflush(stdout);
    std::cout.flush();
    saved = dup(1);
    int dn = open("/dev/null", O_WRONLY);
    if (dn >= 0) {
      dup2(dn, 1);
      close(dn);
    }
  }
  ~Quiet() {
    fflush(stdout);
    std::cout.flush();
    if (saved >= 0) {
      dup2(saved, 1);
      close(saved);
    }
  }
};

std::string segments_file() {
  static std::string path;
  if (path.empty()) {
    char tmpl[] = "/tmp/pmmc_ref_segXXXXXX";
    int fd = mkstemp(tmpl);
    if (fd >= 0) {
      const char *line = "chr1\t0\t1000000\n";
      if (write(fd, line, strlen(line)) < 0) {
      }
      close(fd);
    }
    path = tmpl;
  }
  return path;
}

void apply_settings(const orc_params *p, int level) {
  static Settings st;
  static bool inited = false;
  if (!inited) {
    st.init();
    inited = true;
  }
  Settings::dataSegmentsSplit = segments_file();
  Settings::outputLevel = 0;
  Settings::energyTraceEnabled = false;
  Settings::use2D = p->use2d != 0;
  Settings::sphere_radius = p->sphere_radius;
  Settings::springAngularConstant = p->k_angle;
  Settings::weightDistSmooth = p->w_dist;
  Settings::weightAngleSmooth = p->w_angle;
  if (level == 0) { /* arcs */
    Settings::maxTemp = p->max_temp;
    Settings::dtTemp = p->dt_temp;
    Settings::tempJumpScale = p->jump_scale;
    Settings::tempJumpCoef = p->jump_coef;
    Settings::MCstopConditionImprovement = p->improvement;
    Settings::MCstopConditionMinSuccesses = p->min_successes;
    Settings::MCstopConditionSteps = p->milestone_steps;
    Settings::springConstantStretchArcs = p->k_stretch;
    Settings::springConstantSqueezeArcs = p->k_squeeze;
  } else if (level == 1) { /* heatmap */
    Settings::maxTempHeatmap = p->max_temp;
    Settings::dtTempHeatmap = p->dt_temp;
    Settings::tempJumpScaleHeatmap = p->jump_scale;
    Settings::tempJumpCoefHeatmap = p->jump_coef;
    Settings::MCstopConditionImprovementHeatmap = p->improvement;
    Settings::MCstopConditionMinSuccessesHeatmap = p->min_successes;
    Settings::MCstopConditionStepsHeatmap = p->milestone_steps;
  } else { /* smooth */
    Settings::maxTempSmooth = p->max_temp;
    Settings::dtTempSmooth = p->dt_temp;
    Settings::tempJumpScaleSmooth = p->jump_scale;
    Settings::tempJumpCoefSmooth = p->jump_coef;
    Settings::MCstopConditionImprovementSmooth = p->improvement;
    Settings::MCstopConditionMinSuccessesSmooth = p->min_successes;
    Settings::MCstopConditionStepsSmooth = p->milestone_steps;
    Settings::springConstantStretch = p->k_stretch;
    Settings::springConstantSqueeze = p->k_squeeze;
  }
}

void load_clusters(LooperSolver &s, int n, const float *pos,
                   const unsigned char *fixed, const double *dtn) {
  s.clusters.assign(n, Cluster());
  s.active_region.clear();
  for (int i = 0; i < n; ++i) {
    s.clusters[i].pos.set(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    s.clusters[i].is_fixed = fixed ? fixed[i] != 0 : false;
    s.clusters[i].dist_to_next = dtn ? dtn[i] : 0.0;
    s.active_region.push_back(i);
  }
}

void store_positions(const LooperSolver &s, int n, float *pos) {
  for (int i = 0; i < n; ++i) {
    pos[3 * i] = s.clusters[i].pos.x;
    pos[3 * i + 1] = s.clusters[i].pos.y;
    pos[3 * i + 2] = s.clusters[i].pos.z;
  }
}

void load_dense(Heatmap &h, int n, const float *m) {
  h.init(n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j)
      h.v[i][j] = m[(size_t)i * n + j];
}

void load_loops(LooperSolver &s, int n_loops, const int *li, const int *lj,
                const float *lk, const float *lr0) {
  s.loop_constraints.clear();
  for (int c = 0; c < n_loops; ++c) {
    LooperSolver::LoopConstraint lc;
    lc.cluster_i = li[c];
    lc.cluster_j = lj[c];
    lc.stiffness = lk[c];
    lc.eq_distance = lr0[c];
    s.loop_constraints.push_back(lc);
  }
  s.rebuildActiveLoopMap();
}

} // namespace

extern "C" {

/* LooperSolver::MonteCarloArcs (src/include/LooperSolver.hpp:4670-4796). */
void ref_arcs_anneal(int n, float *pos, const unsigned char *fixed,
                     const float *exp_dist, int n_loops, const int *li,
                     const int *lj, const float *lk, const float *lr0,
                     const orc_params *p, float step, unsigned seed,
                     double *score, long long *moves) {
  Quiet q;
  apply_settings(p, 0);
  LooperSolver s("ref", "/tmp/");
  load_clusters(s, n, pos, fixed, nullptr);
  load_dense(s.heatmap_exp_dist_anchor, n, exp_dist);
  load_loops(s, n_loops, li, lj, lk, lr0);
  srand(seed);
  *score = s.MonteCarloArcs(step);
  *moves = s.total_mc_steps;
  store_positions(s, n, pos);
}

/* moved < 0: calcScoreDistancesActiveRegion() + calcScoreLoopEnergy() +
 * sphere over all beads; moved >= 0: the local score MonteCarloArcs uses. */
double ref_arcs_score(int n, const float *pos, const float *exp_dist,
                      int n_loops, const int *li, const int *lj,
                      const float *lk, const float *lr0, const orc_params *p,
                      int moved) {
  Quiet q;
  apply_settings(p, 0);
  LooperSolver s("ref", "/tmp/");
  load_clusters(s, n, pos, nullptr, nullptr);
  load_dense(s.heatmap_exp_dist_anchor, n, exp_dist);
  load_loops(s, n_loops, li, lj, lk, lr0);
  double sc;
  if (moved < 0) {
    sc = s.calcScoreDistancesActiveRegion() + s.calcScoreLoopEnergy();
    if (s.spherical_container)
      for (int k = 0; k < n; k++)
        sc += s.spherical_container->boundaryPenalty(s.clusters[k].pos);
  } else {
    sc = s.calcScoreDistancesActiveRegion(moved) + s.calcScoreLoopEnergy(moved);
    if (s.spherical_container)
      sc += s.spherical_container->boundaryPenalty(s.clusters[moved].pos);
  }
  return sc;
}

/* LooperSolver::MonteCarloHeatmap (:1424-1565). */
void ref_heatmap_anneal(int n, float *pos, const unsigned char *fixed,
                        const float *heat, int diag, int n_bounds,
                        const int *bounds, const orc_params *p, float step,
                        unsigned seed, double *score, long long *moves) {
  Quiet q;
  apply_settings(p, 1);
  LooperSolver s("ref", "/tmp/");
  load_clusters(s, n, pos, fixed, nullptr);
  load_dense(s.heatmap_dist, n, heat);
  s.heatmap_dist.diagonal_size = diag;
  s.heatmap_chromosome_boundaries.assign(bounds, bounds + n_bounds);
  srand(seed);
  *score = s.MonteCarloHeatmap(step);
  *moves = s.total_mc_steps;
  store_positions(s, n, pos);
}

/* calcScoreHeatmapActiveRegion(moved) (:3583-3617). */
double ref_heatmap_score(int n, const float *pos, const float *heat, int diag,
                         int n_bounds, const int *bounds, int moved) {
  Quiet q;
  orc_params p{};
  apply_settings(&p, 1);
  LooperSolver s("ref", "/tmp/");
  load_clusters(s, n, pos, nullptr, nullptr);
  load_dense(s.heatmap_dist, n, heat);
  s.heatmap_dist.diagonal_size = diag;
  s.heatmap_chromosome_boundaries.assign(bounds, bounds + n_bounds);
  return s.calcScoreHeatmapActiveRegion(moved);
}

/* LooperSolver::MonteCarloArcsSmooth(step, false) (:4798-5047). */
void ref_smooth_anneal(int n, float *pos, const unsigned char *fixed,
                       const double *dtn, const orc_params *p, float step,
                       unsigned seed, double *score, long long *moves) {
  Quiet q;
  apply_settings(p, 2);
  LooperSolver s("ref", "/tmp/");
  load_clusters(s, n, pos, fixed, dtn);
  srand(seed);
  *score = s.MonteCarloArcsSmooth(step, false);
  *moves = s.total_mc_steps;
  store_positions(s, n, pos);
}

/* moved < 0: calcScoreStructureSmooth(true,true) + sphere over all beads (the
 * initial score of MonteCarloArcsSmooth, :4880-4884); moved >= 0: the local
 * score calcScoreStructureSmooth(moved,true,true) + sphere of that bead. */
double ref_smooth_score(int n, const float *pos, const double *dtn,
                        const orc_params *p, int moved) {
  Quiet q;
  apply_settings(p, 2);
  LooperSolver s("ref", "/tmp/");
  load_clusters(s, n, pos, nullptr, dtn);
  double sc;
  if (moved < 0) {
    sc = s.calcScoreStructureSmooth(true, true);
    if (s.spherical_container)
      for (int k = 0; k < n; k++)
        sc += s.spherical_container->boundaryPenalty(s.clusters[k].pos);
  } else {
    sc = s.calcScoreStructureSmooth(moved, true, true);
    if (s.spherical_container)
      sc += s.spherical_container->boundaryPenalty(s.clusters[moved].pos);
  }
  return sc;
}

/* Scores a scripted walk with the reference's local energy functions, the
 * ones its annealers evaluate per proposal.  Move k: before[k] = local score
 * of bead[k]; the bead moves by disp[3k..3k+2] (vector3 float addition, as
 * in the annealers); after[k] = local score again; the move stays when
 * acc[k] != 0, else the saved position comes back.  One solver is set up per
 * call, so a walk of 10^4 moves costs O(10^4 n).
 *   level 0: calcScoreDistancesActiveRegion(p) + calcScoreLoopEnergy(p)
 *            + boundaryPenalty(p)  (MonteCarloArcs, LooperSolver.hpp:4721-4731)
 *   level 1: calcScoreHeatmapActiveRegion(p) (:3583-3617; MonteCarloHeatmap
 *            re-scores the whole map per move, :1488, whose change is twice
 *            the local one)
 *   level 2: calcScoreStructureSmooth(p, true, true) + boundaryPenalty(p)
 *                                  (MonteCarloArcsSmooth, :4939-4949)
 * matrix is the arc-target map (level 0) or the heatmap (level 1). */
void ref_local_walk(int level, int n, const float *pos, const float *matrix, int diag,
                    int n_bounds, const int *bounds, const double *dtn, int n_loops,
                    const int *li, const int *lj, const float *lk, const float *lr0,
                    const orc_params *p, int n_moves, const int *bead, const float *disp,
                    const int *acc, double *before, double *after) {
  Quiet q;
  apply_settings(p, level);
  LooperSolver s("ref", "/tmp/");
  load_clusters(s, n, pos, nullptr, level == 2 ? dtn : nullptr);
  if (level == 0) {
    load_dense(s.heatmap_exp_dist_anchor, n, matrix);
    load_loops(s, n_loops, li, lj, lk, lr0);
  } else if (level == 1) {
    load_dense(s.heatmap_dist, n, matrix);
    s.heatmap_dist.diagonal_size = diag;
    s.heatmap_chromosome_boundaries.assign(bounds, bounds + n_bounds);
  }
  auto local = [&](int b) -> double {
    double sc;
    if (level == 0)
      sc = s.calcScoreDistancesActiveRegion(b) + s.calcScoreLoopEnergy(b);
    else if (level == 1)
      return s.calcScoreHeatmapActiveRegion(b);
    else
      sc = s.calcScoreStructureSmooth(b, true, true);
    if (s.spherical_container) sc += s.spherical_container->boundaryPenalty(s.clusters[b].pos);
    return sc;
  };
  for (int k = 0; k < n_moves; ++k) {
    const int b = bead[k];
    vector3 &x = s.clusters[b].pos;
    const vector3 saved = x;
    before[k] = local(b);
    x += vector3(disp[3 * k], disp[3 * k + 1], disp[3 * k + 2]);
    after[k] = local(b);
    if (!acc[k]) x = saved;
  }
}

/* The structural metrics the distribution tests compare: RMSD after optimal
 * superposition (Chromosome::calcRMSD -> fast_rmsd, Chromosome.hpp:613-634)
 * and the Pearson correlation of all pairwise distances
 * (MetricsFramework::distanceCorrelation, MetricsFramework.hpp:238-286). */
static void load_chromosome(Chromosome &c, int n, const float *pos) {
  c.points.clear();
  for (int i = 0; i < n; ++i)
    c.points.push_back(vector3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]));
  c.size = n;
}

double ref_rmsd(int n, const float *a, const float *b) {
  Chromosome ca, cb;
  load_chromosome(ca, n, a);
  load_chromosome(cb, n, b);
  return ca.calcRMSD(cb);
}

double ref_distance_correlation(int n, const float *a, const float *b) {
  Chromosome ca, cb;
  load_chromosome(ca, n, a);
  load_chromosome(cb, n, b);
  MetricsFramework m;
  return m.distanceCorrelation(ca, cb, 1);
}

/* calcScoreStructureActiveRegionLengths() (moved < 0) or
 * calcScoreStructureActiveRegionLengths(moved) (LooperSolver.hpp:3375-3412):
 * the bond term the extended arc energy uses. */
double ref_lengths_score(int n, const float *pos, const double *dtn,
                         const orc_params *p, int moved) {
  Quiet q;
  apply_settings(p, 2);
  LooperSolver s("ref", "/tmp/");
  load_clusters(s, n, pos, nullptr, dtn);
  return moved < 0 ? s.calcScoreStructureActiveRegionLengths()
                   : s.calcScoreStructureActiveRegionLengths(moved);
}

/* createDistanceHeatmap(level) (LooperSolver.hpp:3042-3085) on one n x n
 * contact map (level 0: the inter-chromosomal constants); writes the
 * expected-distance map into dist_out (n*n). */
int ref_distance_heatmap(int n, const float *contact, int diag, int level, float scale,
                         float power, float stretching, float *dist_out) {
  Quiet q;
  orc_params p;
  memset(&p, 0, sizeof(p));
  apply_settings(&p, 1);
  if (level == 0) {
    Settings::freqToDistHeatmapScaleInter = scale;
    Settings::freqToDistHeatmapPowerInter = power;
  } else {
    Settings::freqToDistHeatmapScale = scale;
    Settings::freqToDistHeatmapPower = power;
  }
  Settings::heatmapDistanceHeatmapStretching = stretching;
  LooperSolver s("ref", "/tmp/");
  s.heatmap.resize(2);
  load_dense(s.heatmap[level], n, contact);
  s.heatmap[level].diagonal_size = diag;
  s.createDistanceHeatmap(level);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) dist_out[(size_t)i * n + j] = s.heatmap_dist.v[i][j];
  return 0;
}

/* LooperSolver::calcAnchorExpectedDistancesHeatmap (src/include/
 * LooperSolver.hpp:5494-5627) on chromosome "chr1": clusters[active[i]].arcs
 * = arc_idx[arc_ptr[i]..], the chromosome's arcs, long arcs and anchors as
 * given, freq_to_distance = memo.  dense (n*n) receives
 * heatmap_exp_dist_anchor; stats4 the applied / oor / inactive / collision
 * counts the reference prints (read back from its output).  Returns 0, or -1
 * when the reference did not finish (it exits on an arc that does not touch
 * its cluster, so callers pass only well-formed arcs). */
int ref_anchor_targets(int n, const int *active, const int *arc_ptr, const int *arc_idx,
                       int n_arcs, const int *arc_start, const int *arc_end,
                       const int *arc_score, int n_long, const int *long_start,
                       const int *long_end, const int *long_score, int n_anc,
                       const int *anc_start, const int *anc_end, int first_cluster,
                       const float *memo, float count_a, float count_scale,
                       float count_shift, float count_base, const float *heat,
                       float influence, float *dense, long long *stats4) {
  char tmpl[] = "/tmp/pmmc_ref_outXXXXXX";
  int fd = mkstemp(tmpl);
  if (fd < 0)
    return -1;
  orc_params p;
  memset(&p, 0, sizeof(p));
  apply_settings(&p, 0);
  Settings::outputLevel = 0;
  Settings::countToDistA = count_a;
  Settings::countToDistScale = count_scale;
  Settings::countToDistShift = count_shift;
  Settings::countToDistBaseLevel = count_base;
  Settings::useAnchorHeatmap = heat != nullptr;
  Settings::anchorHeatmapInfluence = influence;
  fflush(stdout);
  std::cout.flush();
  int saved = dup(1);
  dup2(fd, 1);
  {
    LooperSolver s("ref", "/tmp/");
    int max_cluster = first_cluster + n_anc;
    for (int i = 0; i < n; ++i) max_cluster = std::max(max_cluster, active[i] + 1);
    for (int k = 0; k < n_arcs; ++k)
      max_cluster = std::max(max_cluster, std::max(arc_start[k], arc_end[k]) + 1);
    s.clusters.assign(max_cluster, Cluster());
    s.active_region.assign(active, active + n);
    for (int i = 0; i < n; ++i)
      s.clusters[active[i]].arcs.assign(arc_idx + arc_ptr[i], arc_idx + arc_ptr[i + 1]);
    const std::string chr = "chr1";
    s.current_chr = chr;
    s.chr_first_cluster[chr] = first_cluster;
    std::vector<InteractionArc> &av = s.arcs.arcs[chr];
    for (int k = 0; k < n_arcs; ++k) av.push_back(InteractionArc(arc_start[k], arc_end[k], arc_score[k]));
    std::vector<InteractionArc> &lv = s.arcs.long_arcs[chr];
    for (int k = 0; k < n_long; ++k)
      lv.push_back(InteractionArc(long_start[k], long_end[k], long_score[k]));
    if (n_anc > 0) {
      std::vector<Anchor> &anc = s.arcs.anchors[chr];
      for (int i = 0; i < n_anc; ++i) anc.push_back(Anchor(chr, anc_start[i], anc_end[i], 'N'));
    }
    for (int i = 0; i <= 100; ++i) s.freq_to_distance[i] = memo[i];
    if (heat) load_dense(s.heatmap_anchor, n, heat);
    s.calcAnchorExpectedDistancesHeatmap();
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) dense[(size_t)i * n + j] = s.heatmap_exp_dist_anchor.v[i][j];
  }
  fflush(stdout);
  std::cout.flush();
  dup2(saved, 1);
  close(saved);
  for (int k = 0; k < 4; ++k) stats4[k] = 0;
  FILE *f = fdopen(fd, "r");
  if (f) {
    rewind(f);
    char line[512];
    while (fgets(line, sizeof(line), f)) {
      int a, b, c, d;
      if (sscanf(line, "long_arcs->anchor: applied=%d oor=%d inactive=%d collision=%d", &a, &b,
                 &c, &d) == 4) {
        stats4[0] = a;
        stats4[1] = b;
        stats4[2] = c;
        stats4[3] = d;
      }
    }
    fclose(f);
  } else {
    close(fd);
  }
  unlink(tmpl);
  return 0;
}

/* LooperSolver::stressRefineAnchors("chr1", max_iter, lr)
 * (src/include/LooperSolver.hpp:5638-5913): clusters[active[i]] at pos[i]
 * with genomic_pos[i]; on return order_out = active_region (sorted by the
 * reference) and pos_out the positions of those clusters. */
void ref_stress_refine(int n, const int *active, const int *genomic_pos, const float *pos,
                       int n_arcs, const int *arc_start, const int *arc_end,
                       const int *arc_score, int n_long, const int *long_start,
                       const int *long_end, const int *long_score, int n_anc,
                       const int *anc_start, const int *anc_end, int first_cluster,
                       const orc_stress_params *p, int max_iter, float lr, int *order_out,
                       float *pos_out) {
  Quiet q;
  orc_params op;
  memset(&op, 0, sizeof(op));
  apply_settings(&op, 0);
  Settings::countToDistA = p->count_a;
  Settings::countToDistScale = p->count_scale;
  Settings::countToDistShift = p->count_shift;
  Settings::countToDistBaseLevel = p->count_base;
  Settings::genomicLengthToDistBase = p->glen_base;
  Settings::genomicLengthToDistScale = p->glen_scale;
  Settings::genomicLengthToDistPower = p->glen_power;
  Settings::springConstantStretch = p->k_stretch;
  Settings::springConstantSqueeze = p->k_squeeze;
  Settings::springAngularConstant = p->k_angular;
  LooperSolver s("ref", "/tmp/");
  int max_cluster = first_cluster + n_anc;
  for (int i = 0; i < n; ++i) max_cluster = std::max(max_cluster, active[i] + 1);
  s.clusters.assign(max_cluster, Cluster());
  s.active_region.assign(active, active + n);
  for (int i = 0; i < n; ++i) {
    s.clusters[active[i]].genomic_pos = genomic_pos[i];
    s.clusters[active[i]].pos.set(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
  }
  const std::string chr = "chr1";
  s.current_chr = chr;
  s.chr_first_cluster[chr] = first_cluster;
  std::vector<InteractionArc> &av = s.arcs.arcs[chr];
  for (int k = 0; k < n_arcs; ++k) av.push_back(InteractionArc(arc_start[k], arc_end[k], arc_score[k]));
  std::vector<InteractionArc> &lv = s.arcs.long_arcs[chr];
  for (int k = 0; k < n_long; ++k)
    lv.push_back(InteractionArc(long_start[k], long_end[k], long_score[k]));
  std::vector<Anchor> &anc = s.arcs.anchors[chr];
  for (int i = 0; i < n_anc; ++i) anc.push_back(Anchor(chr, anc_start[i], anc_end[i], 'N'));
  s.stressRefineAnchors(chr, max_iter, lr);
  for (int i = 0; i < n; ++i) {
    order_out[i] = s.active_region[i];
    const vector3 &v = s.clusters[s.active_region[i]].pos;
    pos_out[3 * i] = v.x;
    pos_out[3 * i + 1] = v.y;
    pos_out[3 * i + 2] = v.z;
  }
}

/* InteractionArcs::markArcs (src/include/InteractionArcs.hpp:207-336) on a
 * single chromosome "chr1".  Output layout as orc_mark_arcs. */
int ref_mark_arcs(int n_anchors, const int *a_start, const int *a_end,
                  int n_raw, const int *r_start, const int *r_end,
                  const int *r_score, const int *r_factor, int *out, int cap,
                  int *non_matching) {
  Quiet q;
  InteractionArcs ia;
  std::string chr = "chr1";
  ia.chrs.push_back(chr);
  for (int i = 0; i < n_anchors; ++i)
    ia.anchors[chr].push_back(Anchor(chr, a_start[i], a_end[i], 'N'));
  ia.anchors_cnt[chr] = n_anchors;
  for (int i = 0; i < n_raw; ++i) {
    InteractionArc a(r_start[i], r_end[i], r_score[i], r_factor[i]);
    ia.raw_arcs[chr].push_back(a);
  }
  ia.markArcs(false);
  const std::vector<InteractionArc> &v = ia.arcs[chr];
  *non_matching = 0; /* printed, not stored, by the reference */
  int cnt = (int)v.size();
  if (cnt > cap)
    return -cnt - 1;
  for (int i = 0; i < cnt; ++i) {
    int *o = out + 7 * i;
    o[0] = v[i].start;
    o[1] = v[i].end;
    o[2] = v[i].genomic_start;
    o[3] = v[i].genomic_end;
    o[4] = v[i].score;
    o[5] = v[i].eff_score;
    o[6] = v[i].factor;
  }
  return cnt;
}

/* Cluster::toFile (src/include/Cluster.hpp:175-181) into a buffer. */
int ref_hcm_cluster_line(char *buf, int cap, int start, int end, char orient,
                         float x, float y, float z, int n_children,
                         const int *children) {
  Cluster c(start, end);
  c.orientation = orient;
  c.pos.set(x, y, z);
  c.children.assign(children, children + n_children);
  char *mem = nullptr;
  size_t sz = 0;
  FILE *f = open_memstream(&mem, &sz);
  c.toFile(f);
  fclose(f);
  int w = (int)sz < cap - 1 ? (int)sz : cap - 1;
  memcpy(buf, mem, w);
  buf[w] = 0;
  free(mem);
  return (int)sz;
}

/* InteractionArc::toFile (src/include/InteractionArc.hpp:122-125). */
int ref_hcm_arc_line(char *buf, int cap, const int *a7) {
  InteractionArc a(a7[0], a7[1], a7[4], a7[6]);
  a.genomic_start = a7[2];
  a.genomic_end = a7[3];
  a.eff_score = a7[5];
  char *mem = nullptr;
  size_t sz = 0;
  FILE *f = open_memstream(&mem, &sz);
  a.toFile(f);
  fclose(f);
  int w = (int)sz < cap - 1 ? (int)sz : cap - 1;
  memcpy(buf, mem, w);
  buf[w] = 0;
  free(mem);
  return (int)sz;
}

/* random_vector (src/thirdparty/common.cpp:20-25) after srand(seed): records
 * which of the three rand() draws lands in x, y and z with this compiler. */
void ref_random_vectors(unsigned seed, int count, float max_size, int in2d,
                        float *out) {
  srand(seed);
  for (int i = 0; i < count; ++i) {
    vector3 v = random_vector(max_size, in2d != 0);
    out[3 * i] = v.x;
    out[3 * i + 1] = v.y;
    out[3 * i + 2] = v.z;
  }
}

} /* extern "C" */
