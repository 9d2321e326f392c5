/*
 * pmmc_oracle.h -- CPU oracle for the pMMC simulated-annealing hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the pmmc_gb300 package,
 * its CUDA library or its C ABI) links, loads or calls this code.  It is the
 * checker: a plain-C restatement of the reference's CPU algorithms, used by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU-baseline leg.
 *
 * Every function cites the reference file:line it restates (paths relative to
 * the SFGLab/pMMC source tree).  The restatement keeps the reference's
 * floating-point types and operation order (float vs double per expression)
 * so that, driven by the same libc rand() stream, it reproduces the
 * reference's CPU annealers bit for bit; tests pin it against the reference
 * itself (oracle/_ref, built from the reference sources by oracle/Makefile)
 * and against committed golden vectors generated from it.
 *
 * Build flags matter: compile with -ffp-contract=off so that no platform
 * fuses a*b+c into an FMA that the reference's x86-64 build does not use.
 */
#ifndef PMMC_ORACLE_H_
#define PMMC_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Annealing parameters; every field mirrors a reference Settings:: static
 * (src/include/Settings.hpp:242-328) and keeps its C type (float / int). */
typedef struct orc_params {
  float max_temp;      /* maxTemp / maxTempHeatmap / maxTempSmooth          */
  float dt_temp;       /* dtTemp* : T *= dt after every counted move        */
  float jump_scale;    /* tempJumpScale*                                    */
  float jump_coef;     /* tempJumpCoef*                                     */
  float improvement;   /* MCstopConditionImprovement*                       */
  int min_successes;   /* MCstopConditionMinSuccesses*                      */
  int milestone_steps; /* MCstopConditionSteps*                             */
  float k_stretch;     /* springConstantStretch(Arcs)                       */
  float k_squeeze;     /* springConstantSqueeze(Arcs)                       */
  float k_angle;       /* springAngularConstant                             */
  float w_dist;        /* weightDistSmooth                                  */
  float w_angle;       /* weightAngleSmooth                                 */
  float sphere_radius; /* sphere_radius (0 = no container)                  */
  int use2d;           /* use2D                                             */
  int64_t max_moves;   /* oracle-only safety cap on counted moves (0: none) */
  int schedule;        /* ORC_SCHEDULE_CPU (0) or ORC_SCHEDULE_GPU (1)       */
  int milestone_fails; /* milestoneFailsThreshold ([cuda] milestone_fails)   */
} orc_params;

/* Stopping schedule of an annealer.
 *  ORC_SCHEDULE_CPU : the reference's CPU loops (MonteCarloArcs,
 *                     MonteCarloHeatmap, MonteCarloArcsSmooth): a milestone
 *                     every milestone_steps moves, stop at the first miss.
 *  ORC_SCHEDULE_GPU : the reference's CUDA kernels, restated from their
 *                     source (src/ParallelMonteCarloArcs.cu:494-655,
 *                     src/ParallelMonteCarloSmooth.cu:258-337): moves in
 *                     blocks of 256, milestone_steps caps the moves; the arc
 *                     kernel tests a milestone after every block and stops
 *                     after milestone_fails consecutive misses, the
 *                     smoothing kernel runs every block of its cap.  The
 *                     heatmap annealer has only the CPU schedule. */
enum { ORC_SCHEDULE_CPU = 0, ORC_SCHEDULE_GPU = 1 };

/* Random-number source of an oracle annealer.
 *  ORC_RNG_LIBC   : the reference's own stream -- libc rand() after
 *                   srand(seed) (src/thirdparty/common.cpp:10-24).
 *  ORC_RNG_PHILOX : the counter-based Philox4x32-10 stream the CUDA kernels
 *                   draw from (same key/counter layout, see orc_philox_*). */
enum { ORC_RNG_LIBC = 0, ORC_RNG_PHILOX = 1 };

typedef struct orc_rng {
  int kind;
  uint64_t seed;    /* libc: srand(seed); philox: key                    */
  uint32_t chain;   /* philox: chain id (counter word 1)                 */
  uint64_t move;    /* philox: proposal counter (counter words 2,3)      */
} orc_rng;

/* Result of one annealing run. */
typedef struct orc_result {
  double score;        /* final running (incremental) score             */
  int64_t moves;       /* counted moves (the reference's loop index i)  */
  int64_t accepted;    /* accepted moves                                */
  int64_t proposals;   /* proposals drawn, incl. skipped fixed beads    */
  double best;         /* lowest running score seen, the start included
                        * (the smoothing kernel's per-warp best score,
                        * ParallelMonteCarloSmooth.cu:299,341)          */
} orc_result;

/* ---------------- Philox4x32-10 (Salmon et al., SC'11) ---------------- */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]);
/* u32 -> float in [0,1): top 24 bits times 2^-24. */
float orc_u01(uint32_t x);

/* ---------------- arc level (anchor) ---------------- */
/* Full score: LooperSolver::calcScoreDistancesActiveRegion()
 * (src/include/LooperSolver.hpp:3215-3246, incl. 1/d repulsion for e<0)
 * + calcScoreLoopEnergy() (:3339-3353) + sphere penalty for every bead
 * (:4700-4705).  exp_dist is the dense n*n row-major target matrix. */
double orc_arcs_full_score(int n, const float *pos, const float *exp_dist,
                           int n_loops, const int *loop_i, const int *loop_j,
                           const float *loop_k, const float *loop_r0,
                           const orc_params *p);
/* Same without the repulsion term (the energy the incremental updates track). */
double orc_arcs_spring_score(int n, const float *pos, const float *exp_dist,
                             int n_loops, const int *loop_i, const int *loop_j,
                             const float *loop_k, const float *loop_r0,
                             const orc_params *p);
/* The repulsion term alone: sum over pairs i<j with e_ij<0 of 1.0f/|d_ij|. */
double orc_arcs_repulsion(int n, const float *pos, const float *exp_dist);
/* Local score of bead `moved`: calcScoreDistancesActiveRegion(int)
 * (:3250-3281) + calcScoreLoopEnergy(int) (:3355-3371) + sphere penalty of
 * the bead (:4721-4723). */
double orc_arcs_local_score(int n, const float *pos, const float *exp_dist,
                            int n_loops, const int *loop_i, const int *loop_j,
                            const float *loop_k, const float *loop_r0,
                            const orc_params *p, int moved);
/* LooperSolver::MonteCarloArcs (:4670-4796).  pos is updated in place. */
void orc_arcs_anneal(int n, float *pos, const unsigned char *fixed,
                     const float *exp_dist, int n_loops, const int *loop_i,
                     const int *loop_j, const float *loop_k,
                     const float *loop_r0, const orc_params *p,
                     float step_size, orc_rng *rng, orc_result *res);

/* Extended arc energy (opt-in; the reference arc level has no bond or angle
 * term): bond springs on consecutive beads as
 * calcScoreStructureActiveRegionLengths (LooperSolver.hpp:3375-3412) with
 * one target for every bead, plus the stiffness angle term
 * k_angle * angle(v_i, v_{i-1})^3 of calcScoreStructureSmooth
 * (:3414-3495; angle() thirdparty/common.cpp:39-46), weights 1.  The target
 * is clamped at 1e-5 in both the full and the local form (the reference
 * clamps its local length form at 1e-5, :3404-3405). */
typedef struct orc_ext {
  double bond_target;  /* dist_to_next of every bead (a double, as Cluster::dist_to_next) */
  float k_stretch;     /* springConstantStretch of the bonds    */
  float k_squeeze;     /* springConstantSqueeze of the bonds    */
  float k_angle;       /* springAngularConstant                 */
} orc_ext;
/* moved = -1: the full form; else the terms that bead `moved` changes. */
double orc_arcs_ext_score(int n, const float *pos, const orc_ext *x, int moved);
/* orc_arcs_anneal with the extended energy added (x = NULL: none). */
void orc_arcs_anneal_ext(int n, float *pos, const unsigned char *fixed,
                         const float *exp_dist, int n_loops, const int *loop_i,
                         const int *loop_j, const float *loop_k,
                         const float *loop_r0, const orc_params *p,
                         const orc_ext *x, float step_size, orc_rng *rng,
                         orc_result *res);

/* ---------------- expected-distance heatmap ---------------- */
/* LooperSolver::createDistanceHeatmap (src/include/LooperSolver.hpp:
 * 3042-3085): d_ij = scale * powf(c_ij, power) for c_ij >= 1e-6 (0 below,
 * -1 inside the diagonal band |i-j| < diag), from the upper triangle and
 * mirrored; then every value above avg * stretching is clamped to it, avg
 * being Heatmap::getAvg of the distance map (Heatmap.hpp:440-451: a float
 * running sum over j >= i + getDiagonalSize(), :356-367).  Writes the n*n
 * map, the average and the clamp value. */
void orc_distance_heatmap(int n, const float *contact, int diag, float scale,
                          float power, float stretching, float *dist,
                          float *avg_out, float *max_out);

/* ---------------- equidistant model ---------------- */
/* HierarchicalChromosome::gpuHelper's interpolation (src/
 * HierarchicalChromosome.cu:1253-1447, its CPU path; createEqidistantModel
 * :466-519): points every res bp from pos_start, (pos_stop - pos_start + 1)
 * / res + 1 of them; before first_end the first cluster's position, from
 * last_start on the last one's, otherwise the Catmull-Rom spline
 * (interpolateSpline, thirdparty/common.cpp:453-462) through the level's
 * clusters around the point, mirrored end points at the ends.  gpos/pos: the
 * level's clusters in order.  Returns the number of points (writes at most
 * cap). */
long long orc_equidistant(int n, const int *gpos, const float *pos, int first_end,
                          int last_start, int pos_start, int pos_stop, int res,
                          float *out, long long cap);

/* ---------------- heatmap level (chromosome / segment) ---------------- */
/* calcScoreHeatmapActiveRegion(moved) (:3583-3617); moved = -1 -> full. */
double orc_heatmap_score(int n, const float *pos, const float *heat, int diag,
                         int n_bounds, const int *bounds, int moved);
/* MonteCarloHeatmap (:1424-1565).  incremental = 0 re-scores O(N^2) after
 * every move exactly as the reference does; incremental = 1 updates the
 * score with 2*(local_after - local_before) (valid for the symmetric
 * matrices createDistanceHeatmap builds, :3042-3085). */
void orc_heatmap_anneal(int n, float *pos, const unsigned char *fixed,
                        const float *heat, int diag, int n_bounds,
                        const int *bounds, const orc_params *p,
                        float step_size, int incremental, orc_rng *rng,
                        orc_result *res);

/* ---------------- subanchor smoothing ---------------- */
/* calcScoreStructureSmooth(true,true) (:3414-3451), weighted, + sphere. */
double orc_smooth_full_score(int n, const float *pos, const double *dist_to_next,
                             const orc_params *p);
/* calcScoreStructureSmooth(moved,true,true) (:3453-3495), unweighted, +
 * sphere penalty of the moved bead (:4939-4941). */
double orc_smooth_local_score(int n, const float *pos,
                              const double *dist_to_next, const orc_params *p,
                              int moved);
/* MonteCarloArcsSmooth(step, false) (:4798-5047) without the CTCF and
 * subanchor-heatmap terms (both off by default, Settings.hpp:401,405). */
void orc_smooth_anneal(int n, float *pos, const unsigned char *fixed,
                       const double *dist_to_next, const orc_params *p,
                       float step_size, orc_rng *rng, orc_result *res);

/* ---------------- arc marking ---------------- */
/* InteractionArcs::markArcs (src/include/InteractionArcs.hpp:207-336) for one
 * chromosome.  Anchors {start,end}; raw arcs {start,end,score,factor}.
 * Writes up to cap output arcs (7 ints each: start end genomic_start
 * genomic_end score eff_score factor) and returns the count (or -count-1 if
 * cap was too small).  *non_matching receives the skipped-arc count. */
int orc_mark_arcs(int n_anchors, const int *a_start, const int *a_end,
                  int n_raw, const int *r_start, const int *r_end,
                  const int *r_score, const int *r_factor, int *out, int cap,
                  int *non_matching);

/* ---------------- replay of a kernel's move trace ---------------- */
/* Follows a CUDA chain move by move: for move k the trace gives the bead,
 * the displacement and the kernel's decision.  The oracle re-derives the
 * Philox draw of move k (proposal_mismatch counts draws that differ from the
 * trace), scores the move in FP64 on its own copy of the structure
 * (before[k], after[k] = local scores of the reference's local scoring
 * functions), takes its own Metropolis decision from its FP64 running score,
 * temperature T0*dt^k and the move's Philox uniform (orc_acc[k]), records
 * margin[k] = |ln(E_new/E_prev) - ln(threshold ratio)| (how close the
 * decision was), and then applies the KERNEL's decision so that both stay on
 * the same trajectory.  kind: 0 arc level, 1 heatmap (before/after are the
 * local scores of the moved bead), 2 smoothing. */
typedef struct orc_replay_out {
  double *before;
  double *after;
  int *orc_acc;
  double *margin;
  int proposal_mismatch;
  double final_energy; /* oracle running energy after the last move */
  /* Stopping point of p->schedule along the kernel's decisions and the
   * oracle's FP64 running energy: the counted moves after which the
   * annealer stops (-1: not within the trace), and the smallest relative
   * distance of a milestone comparison that decided it from its threshold
   * (a kernel whose running energy differs in the last bits can stop
   * elsewhere only when this is tiny). */
  int64_t stop_at;
  double stop_margin;
} orc_replay_out;

void orc_arcs_replay(int n, const float *pos0, const unsigned char *fixed,
                     const float *exp_dist, int n_loops, const int *loop_i,
                     const int *loop_j, const float *loop_k,
                     const float *loop_r0, const orc_params *p,
                     float step_size, uint64_t seed, uint32_t chain,
                     int n_moves, const int *bead, const float *disp,
                     const int *gpu_acc, orc_replay_out *out);
/* orc_arcs_replay with the extended energy added (x = NULL: none). */
void orc_arcs_replay_ext(int n, const float *pos0, const unsigned char *fixed,
                         const float *exp_dist, int n_loops, const int *loop_i,
                         const int *loop_j, const float *loop_k,
                         const float *loop_r0, const orc_params *p,
                         const orc_ext *x, float step_size, uint64_t seed,
                         uint32_t chain, int n_moves, const int *bead,
                         const float *disp, const int *gpu_acc,
                         orc_replay_out *out);
void orc_smooth_replay(int n, const float *pos0, const unsigned char *fixed,
                       const double *dist_to_next, const orc_params *p,
                       float step_size, uint64_t seed, uint32_t chain,
                       int n_moves, const int *bead, const float *disp,
                       const int *gpu_acc, orc_replay_out *out);
void orc_heatmap_replay(int n, const float *pos0, const unsigned char *fixed,
                        const float *heat, int diag, int n_bounds,
                        const int *bounds, const orc_params *p,
                        float step_size, uint64_t seed, uint32_t chain,
                        int n_moves, const int *bead, const float *disp,
                        const int *gpu_acc, orc_replay_out *out);

/* ---------------- anchor-level expected distances ---------------- */
/* LooperSolver::calcAnchorExpectedDistancesHeatmap (src/include/
 * LooperSolver.hpp:5494-5627) written out literally: the dense n x n matrix
 * (-1, 0 on the diagonal), the arcs of the active clusters through a
 * cluster -> slot map that inserts a missing cluster as slot 0 (as
 * std::map::operator[] does), the long arcs through the linear anchor scan,
 * then the anchor heatmap's influence (heat NULL: off).  n_anc == 0: no
 * anchor list.  stats4 = applied, out of range, inactive, collision.
 * Returns 0, or -1 when an arc does not touch its cluster (the reference
 * exits). */
int orc_anchor_targets(int n, const int *active, const int *arc_ptr,
                       const int *arc_idx, const int *arc_start,
                       const int *arc_end, const int *arc_score, int n_long,
                       const int *long_start, const int *long_end,
                       const int *long_score, int n_anc, const int *anc_start,
                       const int *anc_end, int first_cluster,
                       const float *memo, float count_a, float count_scale,
                       float count_shift, float count_base, const float *heat,
                       float influence, float *dense, long long *stats4);

/* ---------------- stress refinement ---------------- */
/* LooperSolver::stressRefineAnchors (src/include/LooperSolver.hpp:5638-5913)
 * written out literally.  active (n cluster indices) with genomic_pos and
 * pos (n*3) per entry; on return order_out holds active sorted by genomic
 * position (a stable sort: callers avoid ties, which std::sort orders
 * arbitrarily) and pos_out the refined positions in that order. */
typedef struct orc_stress_params {
  float count_a, count_scale, count_shift, count_base; /* countToDist*        */
  float glen_base, glen_scale, glen_power;             /* genomicLengthToDist* */
  float k_stretch, k_squeeze, k_angular;               /* springConstant*      */
} orc_stress_params;

typedef struct orc_stress_out {
  int iterations; /* iterations whose energy was evaluated            */
  int stop;       /* 0 max_iter, 1 converged, 2 step below 1e-6       */
  float lr;       /* step at exit                                     */
  double total, backbone, hic, angular; /* terms of the last evaluation */
  long long n_pairs;
} orc_stress_out;

int orc_stress_refine(int n, const int *active, const int *genomic_pos,
                      const float *pos, int n_arcs, const int *arc_start,
                      const int *arc_end, const int *arc_score, int n_long,
                      const int *long_start, const int *long_end,
                      const int *long_score, int n_anc, const int *anc_start,
                      const int *anc_end, int first_cluster,
                      const orc_stress_params *p, int max_iter, float lr,
                      int *order_out, float *pos_out, orc_stress_out *out);

/* ---------------- HCM text lines ---------------- */
/* Cluster::toFile (src/include/Cluster.hpp:175-181). Returns bytes written. */
int orc_hcm_cluster_line(char *buf, int cap, int start, int end, char orient,
                         float x, float y, float z, int n_children,
                         const int *children);
/* InteractionArc::toFile (src/include/InteractionArc.hpp:122-125). */
int orc_hcm_arc_line(char *buf, int cap, const int arc7[7]);

#ifdef __cplusplus
}
#endif
#endif /* PMMC_ORACLE_H_ */
