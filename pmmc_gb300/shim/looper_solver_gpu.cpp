// looper_solver_gpu.cpp -- drop-in definitions of the reference's GPU entry
// points on top of the GB300 C ABI (include/pmmc_gb300.h).
//
// SFGLab/pMMC declares its GPU hot path as member functions of LooperSolver
// and InteractionArcs and defines them in five .cu files.  This translation
// unit defines the same symbols instead, so that the reference's pipeline
// (pMMC-reconstruct, runLooper, reconstructClusterArcsDistances ...) runs on
// this library unchanged: build the reference library with this file in
// place of ParallelMonteCarlo{Arcs,Heatmap,Smooth}.cu and ParallelMarkArcs.cu
// and link libpmmc_gb300.so.
//
// Data contract kept from the reference: inputs are read from the solver's
// active region, outputs written back into clusters[active_region[i]].pos
// (smoothing writes free beads only), the return value is the score the
// reference returns, total_mc_steps and the acceptance log are updated.
// Error behaviour: the reference prints and exits on any CUDA error
// (gpuErrchk, ParallelMonteCarloArcs.cu:60-70); so does this file, with the
// library's status message.  There is no CPU fallback.
#include <cstdio>
#include <cstdlib>
#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include <LooperSolver.hpp>

#include "pmmc_gb300.h"

namespace {

pmmc_ctx *g_ctx = nullptr;
std::mutex g_mutex;
uint64_t g_seed = 0;
bool g_seed_set = false;

void check(pmmc_status s, const char *what) {
  if (s == PMMC_OK) return;
  fprintf(stderr, "GPUassert (pmmc_gb300): %s: %s: %s\n", what, pmmc_status_string(s),
          g_ctx ? pmmc_last_error(g_ctx) : "");
  exit((int)s);
}

pmmc_ctx *ctx() {
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_ctx) {
    check(pmmc_ctx_create(&g_ctx, 0), "context");
    // the reference seeds from -j / [main] seed, else time(NULL)
    pmmc_set_seed(g_ctx, g_seed_set ? g_seed
                                    : (Settings::gpuSeed ? Settings::gpuSeed
                                                         : (uint64_t)time(nullptr)));
  }
  return g_ctx;
}

pmmc_anneal_params arcs_params() {
  pmmc_anneal_params p;
  pmmc_default_params(PMMC_LEVEL_ARCS, &p);
  p.max_temp = Settings::maxTemp;
  p.dt_temp = Settings::dtTemp;
  p.jump_scale = Settings::tempJumpScale;
  p.jump_coef = Settings::tempJumpCoef;
  p.improvement = Settings::MCstopConditionImprovement;
  p.min_successes = Settings::MCstopConditionMinSuccesses;
  p.milestone_steps = Settings::MCstopConditionSteps;
  p.k_stretch = Settings::springConstantStretchArcs;
  p.k_squeeze = Settings::springConstantSqueezeArcs;
  p.sphere_radius = Settings::sphere_radius;
  p.use2d = Settings::use2D ? 1 : 0;
  p.milestone_fails = Settings::milestoneFailsThreshold;
  p.schedule = PMMC_SCHEDULE_GPU;  // the reference kernel's schedule
  return p;
}

}  // namespace

// setGpuSeed (platform.h:106, ParallelMonteCarloHeatmap.cu:37-39)
void setGpuSeed(unsigned int seed) {
  g_seed = seed;
  g_seed_set = true;
  if (g_ctx) pmmc_set_seed(g_ctx, seed);
}

// LooperSolver_setArcsGpuSeed (ParallelMonteCarloArcs.cu:950-952)
void LooperSolver_setArcsGpuSeed(unsigned int seed) { setGpuSeed(seed); }

// GpuResourceCache (LooperSolver.hpp:54-106): the library context owns the
// device buffers; the cache only records that a device is there.
void GpuResourceCache::init() {
  if (initialized) return;
  pmmc_ctx *c = ctx();
  sm_count = pmmc_sm_count(c);
  initialized = true;
}
void GpuResourceCache::initArcsBuffers(int, int, int) {}
void GpuResourceCache::initSmoothBuffers(int) {}
void GpuResourceCache::cleanup() { initialized = false; }

// LooperSolver::parallelMonteCarloArcs (LooperSolver.hpp:682,
// ParallelMonteCarloArcs.cu:680-944)
float LooperSolver::parallelMonteCarloArcs(float step_size) {
  const int n = static_cast<int>(active_region.size());
  if (n <= 1) return 0.0f;
  rebuildActiveLoopMap();
  // host staging kept across calls (the reference caches its device buffers
  // in gpu_cache the same way); the drop-in is called from one thread
  static std::vector<float> pos, out, target;
  static std::vector<unsigned char> fixed;
  static std::vector<int> row_ptr, col;
  static std::vector<const float *> rows;
  pos.resize(3 * n);
  out.resize(3 * n);
  fixed.resize(n);
  for (int i = 0; i < n; ++i) {
    const Cluster &c = clusters[active_region[i]];
    pos[3 * i] = c.pos.x;
    pos[3 * i + 1] = c.pos.y;
    pos[3 * i + 2] = c.pos.z;
    fixed[i] = c.is_fixed ? 1 : 0;
  }
  // the arc lists straight from the rows of heatmap_exp_dist_anchor (no
  // n x n copy); without a matrix of the region's size every pair repels
  row_ptr.resize(n + 1);
  if (col.empty()) {  // non-null buffers: a short capacity reports the count
    col.resize(1);
    target.resize(1);
  }
  int64_t nnz = 0;
  if ((int)heatmap_exp_dist_anchor.size == n) {
    rows.assign(heatmap_exp_dist_anchor.v, heatmap_exp_dist_anchor.v + n);
    pmmc_status st = pmmc_arcs_rows_to_csr(n, rows.data(), row_ptr.data(), col.data(),
                                           target.data(), (int64_t)col.size(), &nnz);
    if (st != PMMC_OK && nnz > (int64_t)col.size()) {  // grow to the count, once
      col.resize(nnz);
      target.resize(nnz);
      st = pmmc_arcs_rows_to_csr(n, rows.data(), row_ptr.data(), col.data(), target.data(),
                                 (int64_t)col.size(), &nnz);
    }
    check(st, "arc lists");
  } else {
    std::fill(row_ptr.begin(), row_ptr.end(), 0);
  }
  std::vector<int> li, lj;
  std::vector<float> lk, lr;
  for (const auto &entry : active_loop_map) {
    li.push_back(entry.first.first);
    lj.push_back(entry.first.second);
    lk.push_back(loop_constraints[entry.second].stiffness);
    lr.push_back(loop_constraints[entry.second].eq_distance);
  }
  pmmc_arcs_problem pr{n, pos.data(), fixed.data(), row_ptr.data(), col.data(), target.data(),
                       (int)li.size(), li.data(), lj.data(), lk.data(), lr.data()};
  pmmc_anneal_params p = arcs_params();
  pmmc_result r;
  check(pmmc_arcs_anneal(ctx(), &pr, &p, step_size, 0, out.data(), &r), "parallelMonteCarloArcs");
  for (int i = 0; i < n; ++i)
    clusters[active_region[i]].pos.set(out[3 * i], out[3 * i + 1], out[3 * i + 2]);
  total_mc_steps += r.moves;
  if (sim_logger) sim_logger->logAcceptanceRatio("arcs_gpu", (int)r.moves, (int)r.accepted);
  return r.score;
}

// LooperSolver::ParallelMonteCarloSmooth (LooperSolver.hpp:482-483,
// ParallelMonteCarloSmooth.cu:357-506)
float LooperSolver::ParallelMonteCarloSmooth(float step_size, unsigned long long seed) {
  const int n = static_cast<int>(active_region.size());
  if (n <= 2) return 0.0f;
  std::vector<float> pos(3 * n), out(3 * n), dtn(n);
  std::vector<unsigned char> fixed(n);
  for (int i = 0; i < n; ++i) {
    const Cluster &c = clusters[active_region[i]];
    pos[3 * i] = c.pos.x;
    pos[3 * i + 1] = c.pos.y;
    pos[3 * i + 2] = c.pos.z;
    fixed[i] = c.is_fixed ? 1 : 0;
    dtn[i] = static_cast<float>(c.dist_to_next);
  }
  pmmc_anneal_params p;
  pmmc_default_params(PMMC_LEVEL_SMOOTH, &p);
  p.max_temp = Settings::maxTempSmooth;
  p.dt_temp = Settings::dtTempSmooth;
  p.jump_scale = Settings::tempJumpScaleSmooth;
  p.jump_coef = Settings::tempJumpCoefSmooth;
  p.improvement = Settings::MCstopConditionImprovementSmooth;
  p.min_successes = Settings::MCstopConditionMinSuccessesSmooth;
  p.milestone_steps = Settings::MCstopConditionStepsSmooth;
  p.k_stretch = Settings::springConstantStretch;
  p.k_squeeze = Settings::springConstantSqueeze;
  p.k_angle = Settings::springAngularConstant;
  p.w_dist = Settings::weightDistSmooth;
  p.w_angle = Settings::weightAngleSmooth;
  p.sphere_radius = Settings::sphere_radius;
  p.use2d = Settings::use2D ? 1 : 0;
  p.milestone_fails = Settings::milestoneFailsThreshold;
  p.schedule = PMMC_SCHEDULE_GPU;
  pmmc_ctx *c = ctx();
  if (seed) pmmc_set_seed(c, seed);
  pmmc_smooth_problem pr{n, pos.data(), fixed.data(), dtn.data()};
  pmmc_result r;
  check(pmmc_smooth_anneal(c, &pr, &p, step_size, 0, out.data(), &r), "ParallelMonteCarloSmooth");
  for (int i = 0; i < n; ++i)
    if (!fixed[i]) clusters[active_region[i]].pos.set(out[3 * i], out[3 * i + 1], out[3 * i + 2]);
  total_mc_steps += r.moves;
  if (sim_logger) sim_logger->logAcceptanceRatio("smooth_gpu", (int)r.moves, (int)r.accepted);
  // the reference returns the CPU FP64 re-score (ParallelMonteCarloSmooth.cu:503)
  return static_cast<float>(calcScoreStructureSmooth(true, true));
}

// LooperSolver::ParallelMonteCarloHeatmap (LooperSolver.hpp:469,
// ParallelMonteCarloHeatmap.cu:365-511), with the semantics of the CPU
// MonteCarloHeatmap (the reference kernel only ever moves bead 0 when a seed
// is set).
float LooperSolver::ParallelMonteCarloHeatmap(float step_size) {
  const int n = static_cast<int>(active_region.size());
  if (n <= 1) return 0.0f;
  std::vector<float> pos(3 * n), out(3 * n), heat((size_t)n * n);
  std::vector<unsigned char> fixed(n);
  for (int i = 0; i < n; ++i) {
    const Cluster &c = clusters[active_region[i]];
    pos[3 * i] = c.pos.x;
    pos[3 * i + 1] = c.pos.y;
    pos[3 * i + 2] = c.pos.z;
    fixed[i] = c.is_fixed ? 1 : 0;
    for (int j = 0; j < n; ++j) heat[(size_t)i * n + j] = heatmap_dist.v[i][j];
  }
  pmmc_anneal_params p;
  pmmc_default_params(PMMC_LEVEL_HEATMAP, &p);
  p.max_temp = Settings::maxTempHeatmap;
  p.dt_temp = Settings::dtTempHeatmap;
  p.jump_scale = Settings::tempJumpScaleHeatmap;
  p.jump_coef = Settings::tempJumpCoefHeatmap;
  p.improvement = Settings::MCstopConditionImprovementHeatmap;
  p.min_successes = Settings::MCstopConditionMinSuccessesHeatmap;
  p.milestone_steps = Settings::MCstopConditionStepsHeatmap;
  p.sphere_radius = Settings::sphere_radius;
  p.use2d = Settings::use2D ? 1 : 0;
  p.schedule = PMMC_SCHEDULE_CPU;
  pmmc_heatmap_problem pr{n, pos.data(), fixed.data(), heat.data(), heatmap_dist.diagonal_size,
                          (int)heatmap_chromosome_boundaries.size(),
                          heatmap_chromosome_boundaries.data()};
  pmmc_result r;
  check(pmmc_heatmap_anneal(ctx(), &pr, &p, step_size, out.data(), &r), "ParallelMonteCarloHeatmap");
  for (int i = 0; i < n; ++i)
    clusters[active_region[i]].pos.set(out[3 * i], out[3 * i + 1], out[3 * i + 2]);
  total_mc_steps += r.moves;
  return static_cast<float>(calcScoreHeatmapActiveRegion());
}

// InteractionArcs::parallelMarkArcs (ParallelMarkArcs.cu:69-244); output in
// the order of the CPU markArcs (InteractionArcs.hpp:207-336).
void InteractionArcs::parallelMarkArcs(bool ignore_missing) {
  (void)ignore_missing;
  for (const std::string &chr : chrs) {
    printf(" %s...\n", chr.c_str());
    arcs[chr].clear();
    std::sort(raw_arcs[chr].begin(), raw_arcs[chr].end());
    const std::vector<Anchor> &an = anchors[chr];
    const std::vector<InteractionArc> &raw = raw_arcs[chr];
    const int A = anchors_cnt[chr], R = (int)raw.size();
    std::vector<int> as(A), ae(A), rs(R), re(R), rsc(R), rf(R);
    for (int i = 0; i < A; ++i) {
      as[i] = an[i].start;
      ae[i] = an[i].end;
    }
    for (int i = 0; i < R; ++i) {
      rs[i] = raw[i].start;
      re[i] = raw[i].end;
      rsc[i] = raw[i].score;
      rf[i] = raw[i].factor;
    }
    std::vector<int> out(7 * (2 * R + 8));
    int n_out = 0, nm = 0;
    check(pmmc_mark_arcs(ctx(), A, as.data(), ae.data(), R, rs.data(), re.data(), rsc.data(),
                         rf.data(), out.data(), 2 * R + 8, &n_out, &nm),
          "parallelMarkArcs");
    for (int k = 0; k < n_out; ++k) {
      const int *o = &out[7 * k];
      InteractionArc a(o[0], o[1], o[4], o[6]);
      a.genomic_start = o[2];
      a.genomic_end = o[3];
      a.eff_score = o[5];
      arcs[chr].push_back(a);
    }
    if (nm > 0) printf("  %d non-matching arcs skipped\n", nm);
    arcs_cnt[chr] = static_cast<int>(arcs[chr].size());
  }
}
