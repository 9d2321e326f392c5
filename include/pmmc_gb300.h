/*
 * pmmc_gb300.h -- C ABI of the GB300-native pMMC annealing library.
 *
 * The reference (SFGLab/pMMC) exposes its GPU hot path as C++ member
 * functions of LooperSolver / InteractionArcs that read the solver's state
 * directly.  This library replaces them with plain-C entry points: pointers,
 * sizes and status codes; no C++ or torch types.  Each declaration names the
 * reference interface it replaces.  The C++ shim in pmmc_gb300/shim/ maps
 * the reference's member functions onto these calls.
 *
 * Positions are float xyz triples (n*3 floats, the reference's
 * clusters[active_region[i]].pos order).  Host pointers are copied in and
 * out; the *_device / batch entry points take device pointers and a CUDA
 * stream (passed as void*).  Every call returns a pmmc_status; nothing
 * exits the process and there is no CPU fallback: without a usable GB300
 * device the calls return PMMC_ERR_NO_DEVICE.
 */
#ifndef PMMC_GB300_H_
#define PMMC_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum pmmc_status {
  PMMC_OK = 0,
  PMMC_ERR_INVALID = 1,   /* bad argument or size                       */
  PMMC_ERR_NO_DEVICE = 2, /* no CUDA device / library not usable         */
  PMMC_ERR_CUDA = 3,      /* a CUDA runtime call failed                  */
  PMMC_ERR_NOMEM = 4,     /* device allocation failed                    */
  PMMC_ERR_TIMEOUT = 5,   /* a bounded device wait ran out               */
  PMMC_ERR_BUDGET = 6,    /* request exceeds the device-memory budget    */
  PMMC_ERR_FIXED = 7,     /* reserved, not returned: a region whose beads
                           * are all fixed makes no move                 */
  PMMC_ERR_BUSY = 8,      /* server: no free slot right now              */
  PMMC_ERR_NOT_FOUND = 9, /* server: unknown request id                  */
  PMMC_ERR_CANCELLED = 10 /* server: the request was cancelled            */
} pmmc_status;

/* Stopping schedule of a chain. */
enum {
  /* The reference CUDA kernels: moves in blocks of 256 while fewer than
   * `milestone_steps` are done (so at most `milestone_steps` rounded up to
   * 256, none when it is <= 0).  Arc level (ParallelMonteCarloArcs.cu:
   * 520-655): a milestone after every block, the CPU predicate with its
   * ratio test guarded by milestone energy > 1e-10, stop after
   * `milestone_fails` consecutive misses or below 1e-5; an uphill move is
   * tested only when T > 0 and the previous energy is > 0; with several
   * chains the first to stop ends the others at their next milestone.
   * Smoothing (ParallelMonteCarloSmooth.cu:267-337): every chain makes the
   * whole cap (the kernel's milestone test cannot fire before its last
   * block), and the reported chain is the one whose running energy reached
   * the lowest value. */
  PMMC_SCHEDULE_GPU = 0,
  /* The reference CPU loops (LooperSolver.hpp:4764-4783, 1529-1553,
   * 5014-5034): a milestone every `milestone_steps` moves, stop at the first
   * miss.  `max_moves` (or 200 milestones when 0) bounds the chain. */
  PMMC_SCHEDULE_CPU = 1
};

/* Annealing parameters.  Each field is the reference Settings:: static of
 * the same meaning (src/include/Settings.hpp:242-328, INI sections
 * [simulation_arcs], [simulation_heatmap], [simulation_arcs_smooth],
 * [springs], [simulation], [cuda]).  Use pmmc_default_params() for the
 * reference defaults of a level. */
typedef struct pmmc_anneal_params {
  float max_temp;        /* max_temp*                              */
  float dt_temp;         /* delta_temp*                            */
  float jump_scale;      /* jump_temp_scale*                       */
  float jump_coef;       /* jump_temp_coef*                        */
  float improvement;     /* stop_condition_improvement_threshold*  */
  int min_successes;     /* stop_condition_successes_threshold*    */
  int milestone_steps;   /* stop_condition_steps*                  */
  float k_stretch;       /* stretch_constant(_arcs)                */
  float k_squeeze;       /* squeeze_constant(_arcs)                */
  float k_angle;         /* angular_constant                       */
  float w_dist;          /* dist_weight (smooth)                   */
  float w_angle;         /* angle_weight (smooth)                  */
  float sphere_radius;   /* [simulation] sphere_radius, 0 = off    */
  int use2d;             /* 2D moves                               */
  int milestone_fails;   /* [cuda] milestone_fails                 */
  int schedule;          /* PMMC_SCHEDULE_GPU / PMMC_SCHEDULE_CPU  */
  int resync_every;      /* FP64 energy recompute every L moves (0 = off) */
  int64_t max_moves;     /* hard cap on moves per chain (0 = schedule's);
                          * smoothing: < 0 means -max_moves sweeps, a cap
                          * of -max_moves x movable beads per region     */
  /* Extended arc energy (off = the reference's arcs+loops+sphere): bond
   * springs on consecutive beads with target `bond_target` and constants
   * k_stretch_bond/k_squeeze_bond, and the smooth-level angle term
   * k_angle_ext*((1-cos)/2)^3 at every interior bead. */
  int arcs_extended;
  float bond_target;
  float k_stretch_bond;
  float k_squeeze_bond;
  float k_angle_ext;
} pmmc_anneal_params;

enum { PMMC_LEVEL_ARCS = 0, PMMC_LEVEL_HEATMAP = 1, PMMC_LEVEL_SMOOTH = 2 };

/* Result of an annealing call (one chain, or the best of several). */
typedef struct pmmc_result {
  float score;           /* the FP32 score the reference returns             */
  double energy;         /* running FP64 energy at the end of the chain       */
  double energy_fp64;    /* FP64 recompute of the same energy definition      */
  double rel_error;      /* |energy - energy_fp64| / max(|energy_fp64|,1e-30) */
  int64_t moves;         /* counted moves of the reported chain               */
  int64_t accepted;      /* accepted moves of the reported chain              */
  int64_t total_moves;   /* moves over all chains of the call                 */
  int best_chain;        /* index of the reported chain                       */
  int status;            /* per-chain device status (0 = ok)                  */
} pmmc_result;

/* Anchor-level active region: positions, fixed flags and per-bead arc lists
 * (CSR over both directions).  A pair listed in the CSR with target >= 1e-6
 * is an arc spring; a pair listed with 0 <= target < 1e-6 contributes
 * nothing; every pair not listed contributes the 1/d repulsion to the
 * initial score only (the reference's dense -1 entries,
 * LooperSolver.hpp:3226-3231 vs :3262-3266).  pmmc_arcs_dense_to_csr()
 * converts the reference's dense n x n matrix. */
typedef struct pmmc_arcs_problem {
  int n;
  const float *pos;            /* n*3                                    */
  const unsigned char *fixed;  /* n, nullable                            */
  const int *row_ptr;          /* n+1                                    */
  const int *col;              /* row_ptr[n], sorted within each row     */
  const float *target;         /* row_ptr[n]                             */
  int n_loops;                 /* loop constraints (cluster indices are  */
  const int *loop_i;           /* active-region indices here)            */
  const int *loop_j;
  const float *loop_k;
  const float *loop_r0;
} pmmc_arcs_problem;

/* Heatmap-level active region: dense n x n expected-distance matrix
 * (row-major, symmetric as createDistanceHeatmap builds it,
 * LooperSolver.hpp:3042-3085), diagonal band width and optional chromosome
 * boundaries.  The annealers change the full score by twice a move's local
 * change, which holds only for a symmetric map: a map whose pairs (i, m)
 * inside one block and outside the diagonal band differ from (m, i) -- one
 * side below 1e-6 and the other not, or unequal values -- is refused with
 * PMMC_ERR_INVALID, the message naming the region and its lowest such pair
 * (m, i), m < i.  The maps are copied to the device as given; the check and
 * the reciprocals the kernels read are computed there. */
typedef struct pmmc_heatmap_problem {
  int n;
  const float *pos;            /* n*3                        */
  const unsigned char *fixed;  /* n, nullable                */
  const float *heat;           /* n*n                        */
  int diag;                    /* heatmap_dist.diagonal_size */
  int n_bounds;                /* 0 = one block              */
  const int *bounds;
} pmmc_heatmap_problem;

/* Subanchor smoothing region: positions, fixed flags, dist_to_next. */
typedef struct pmmc_smooth_problem {
  int n;
  const float *pos;            /* n*3           */
  const unsigned char *fixed;  /* n, nullable   */
  const float *dist_to_next;   /* n             */
} pmmc_smooth_problem;

typedef struct pmmc_ctx pmmc_ctx;

/* ---------------- context ---------------- */
/* Replaces GpuResourceCache::init / cleanup (LooperSolver.hpp:54-106,
 * ParallelMonteCarloArcs.cu:84-213): one context owns the device buffers.
 * The calls that take a context come from one host thread at a time (they
 * share its stream, call counter, settings and host packing buffers); the
 * calls of a server made on it (pmmc_server_*) may come from any thread,
 * beside them.  pmmc_last_error then holds the message of whichever failing
 * call came last. */
pmmc_status pmmc_ctx_create(pmmc_ctx **out, int device);
void pmmc_ctx_destroy(pmmc_ctx *ctx);
const char *pmmc_status_string(pmmc_status s);
/* Message of the last failing call on this context. */
const char *pmmc_last_error(const pmmc_ctx *ctx);
/* Replaces setGpuSeed (platform.h:106, ParallelMonteCarloHeatmap.cu:37-39)
 * and LooperSolver_setArcsGpuSeed (ParallelMonteCarloArcs.cu:950-952): the
 * Philox key of every later call.  Each call also advances a per-context
 * call counter so that consecutive calls draw fresh streams. */
void pmmc_set_seed(pmmc_ctx *ctx, uint64_t seed);
/* Number of SMs of the context's device (the reference caches it in
 * GpuResourceCache::sm_count, ParallelMonteCarloArcs.cu:89-90). */
int pmmc_sm_count(const pmmc_ctx *ctx);
/* Reference defaults of a level (Settings.hpp:397-505). */
void pmmc_default_params(int level, pmmc_anneal_params *out);

/* ---------------- conversions ---------------- */
/* Reference dense matrix (heatmap_exp_dist_anchor.v, -1 = no arc) -> CSR
 * over both directions, keeping every off-diagonal entry >= 0.  Entry
 * (i, j) of the CSR holds dense[j*n + i] (the column the reference's local
 * score reads, LooperSolver.hpp:3262); columns ascend within a row.  With
 * col/target NULL only row_ptr and *nnz; a cap below the count returns
 * PMMC_ERR_INVALID with *nnz set. */
pmmc_status pmmc_arcs_dense_to_csr(int n, const float *dense, int *row_ptr,
                                   int *col, float *target, int64_t cap,
                                   int64_t *nnz);
/* The same from the reference's own row pointers (Heatmap::v, float**;
 * rows[j][i] = v[j][i]), read row by row with no n x n copy: what
 * parallelMonteCarloArcs packs from heatmap_exp_dist_anchor
 * (ParallelMonteCarloArcs.cu:789-840). */
pmmc_status pmmc_arcs_rows_to_csr(int n, const float *const *rows, int *row_ptr,
                                  int *col, float *target, int64_t cap,
                                  int64_t *nnz);

/* ---------------- plain drop-in entry points (host buffers) ----------- */
/* Replaces float LooperSolver::parallelMonteCarloArcs(float step_size)
 * (LooperSolver.hpp:682, ParallelMonteCarloArcs.cu:680-944): n_chains
 * independent chains (0 = 4 per SM, the reference's 128-thread x sm_count
 * launch), the first converged chain stops the others, the best chain's
 * positions are written to pos_out. */
pmmc_status pmmc_arcs_anneal(pmmc_ctx *ctx, const pmmc_arcs_problem *pr,
                             const pmmc_anneal_params *prm, float step_size,
                             int n_chains, float *pos_out, pmmc_result *res);

/* Replaces float LooperSolver::ParallelMonteCarloSmooth(float step_size,
 * unsigned long long seed) (LooperSolver.hpp:482-483,
 * ParallelMonteCarloSmooth.cu:357-506): n_chains chains (0 = one per SM),
 * best chain's free beads written to pos_out (fixed beads are copied
 * through unchanged). */
pmmc_status pmmc_smooth_anneal(pmmc_ctx *ctx, const pmmc_smooth_problem *pr,
                               const pmmc_anneal_params *prm, float step_size,
                               int n_chains, float *pos_out, pmmc_result *res);

/* Replaces float LooperSolver::ParallelMonteCarloHeatmap(float step_size)
 * (LooperSolver.hpp:469, ParallelMonteCarloHeatmap.cu:365-511) with the
 * semantics of the reference's CPU MonteCarloHeatmap (LooperSolver.hpp:
 * 1424-1565): one chain, step_size*0.5, full-score Metropolis with the
 * score updated incrementally as 2*(local_after - local_before). */
pmmc_status pmmc_heatmap_anneal(pmmc_ctx *ctx, const pmmc_heatmap_problem *pr,
                                const pmmc_anneal_params *prm, float step_size,
                                float *pos_out, pmmc_result *res);

/* Replaces void InteractionArcs::parallelMarkArcs(bool ignore_missing)
 * (InteractionArcs.hpp, ParallelMarkArcs.cu:69-244) for one chromosome:
 * anchors sorted by start; raw arcs in genomic coordinates.  Writes up to
 * cap arcs of 7 ints (start end genomic_start genomic_end score eff_score
 * factor) in the order of the reference's CPU markArcs
 * (InteractionArcs.hpp:207-336). */
pmmc_status pmmc_mark_arcs(pmmc_ctx *ctx, int n_anchors, const int *a_start,
                           const int *a_end, int n_raw, const int *r_start,
                           const int *r_end, const int *r_score,
                           const int *r_factor, int *out, int cap, int *n_out,
                           int *n_non_matching);

/* ---------------- batched arc annealing (device resident) -------------- */
/* Many independent active regions (ensemble members x interaction blocks,
 * the reference's serial loops at LooperSolver.hpp:4026-4138 and
 * main_reconstruct.cpp:405-477) annealed in one graph launch of persistent
 * work-stealing kernels.  Units are staged once; run() anneals every unit
 * from its staged start positions. */
typedef struct pmmc_arcs_batch pmmc_arcs_batch;
typedef struct pmmc_batch_opts {
  int chains_per_unit;   /* independent chains per unit (>= 1)           */
  int use_graph;         /* capture the launches in a CUDA graph          */
  int lanes_per_chain;   /* lanes that score one proposal: 1, 2, 4, 8 or 32;
                          * a chain's warp scores 32/lanes proposals at
                          * once (0 = the default, 2; PMMC_LANES_AUTO =
                          * the autotuner picks lanes and warps per CTA
                          * for each shared-memory class from timed trial
                          * launches, cached per process and in the JSON
                          * file named by PMMC_AUTOTUNE_CACHE, and
                          * whether chains get a drawing warp)            */
  int drawing_warp;      /* with lanes 1 or 2: 1 = every chain gets a second
                          * warp that draws its moves (Philox proposals and
                          * thresholds) ahead of it, 0 = the chain's warp
                          * draws them itself; the moves are the same     */
} pmmc_batch_opts;
#define PMMC_LANES_AUTO (-1)
pmmc_status pmmc_arcs_batch_create(pmmc_ctx *ctx, int n_units,
                                   const pmmc_arcs_problem *units,
                                   const pmmc_anneal_params *prm,
                                   const float *step_sizes,
                                   const pmmc_batch_opts *opts,
                                   pmmc_arcs_batch **out);
/* Enqueue one annealing pass of every unit on `stream` (NULL = the
 * context's stream).  Asynchronous. */
pmmc_status pmmc_arcs_batch_run(pmmc_arcs_batch *b, void *stream);
/* Copy results to host (synchronises the batch's stream).  pos_out holds
 * sum(n_u)*3 floats in unit order; res holds n_units results. */
pmmc_status pmmc_arcs_batch_results(pmmc_arcs_batch *b, float *pos_out,
                                    pmmc_result *res);
/* Figures of the last run: device time of the pass (ms, CUDA events on the
 * launching stream around the graph), total moves over all chains, and the
 * number of kernels one pass launches (one persistent annealing kernel per
 * shared-memory size class, plus the best-chain pick when units have several
 * chains). */
pmmc_status pmmc_arcs_batch_stats(pmmc_arcs_batch *b, double *kernel_ms,
                                  int64_t *total_moves, int *launches_per_run);
void pmmc_arcs_batch_destroy(pmmc_arcs_batch *b);

/* Host-buffer form of the above: stage, run, fetch, free. */
pmmc_status pmmc_arcs_batch_anneal(pmmc_ctx *ctx, int n_units,
                                   const pmmc_arcs_problem *units,
                                   const pmmc_anneal_params *prm,
                                   const float *step_sizes,
                                   const pmmc_batch_opts *opts, float *pos_out,
                                   pmmc_result *res);

/* pmmc_arcs_batch_create with two more knobs: stop_all != 0 lets the first
 * converged chain of a unit stop its other chains at their next milestone
 * (the reference's shared d_isDone flag, read once per 256-move block,
 * ParallelMonteCarloArcs.cu:520,650); trace_cap > 0 records the first
 * trace_cap moves of every chain of region 0 (bead, local scores
 * before/after, decision, displacement; 32 bytes each) for per-move parity
 * checks. */
pmmc_status pmmc_arcs_batch_create_ex(pmmc_ctx *ctx, int n_units,
                                      const pmmc_arcs_problem *units,
                                      const pmmc_anneal_params *prm,
                                      const float *step_sizes,
                                      const pmmc_batch_opts *opts,
                                      int stop_all, int trace_cap,
                                      pmmc_arcs_batch **out);
/* Tests only (no reference counterpart): compares the kernels' square root
 * with the IEEE single-precision routine on the float bit patterns
 * [lo, lo + count); returns the number of differing results and the lowest
 * differing pattern (0xFFFFFFFF if none). */
pmmc_status pmmc_selftest_sqrt(pmmc_ctx *ctx, uint32_t lo, uint32_t count,
                               uint64_t *mismatches, uint32_t *first_bad);
/* The launch configuration of each shared-memory class of a batch (no
 * reference counterpart): lanes per proposal, chains per CTA, work items,
 * whether arc lists are staged in shared memory and whether each chain has a
 * second warp drawing its moves ahead; up to `cap` classes.  Any output
 * pointer may be NULL. */
pmmc_status pmmc_arcs_batch_classes(pmmc_arcs_batch *b, int cap, int *n_classes,
                                    int *lanes, int *warps, int *items, int *nb_smem,
                                    int *drawing_warp);
/* Copy `count` (<= trace_cap) trace records of chain 0 of the last run to
 * host (tests; no reference counterpart). */
pmmc_status pmmc_arcs_batch_trace(pmmc_arcs_batch *b, void *out, int count);
/* The same for chain `chain` of region 0. */
pmmc_status pmmc_arcs_batch_trace_chain(pmmc_arcs_batch *b, int chain, void *out, int count);
/* The result of every chain of region `unit` of the last run, in chain order
 * (up to `cap`; best_chain holds the chain's own index, total_moves the
 * region's total), and the region's chain count.  The reference keeps the
 * per-warp scores of its drop-in call in d_best_score
 * (ParallelMonteCarloArcs.cu:661-667); this exposes the same per chain. */
pmmc_status pmmc_arcs_batch_chain_results(pmmc_arcs_batch *b, int unit, int cap,
                                          pmmc_result *res, int *n_chains);

/* ---------------- batched smoothing and heatmap annealing -------------- */
/* Many smoothing regions (genome-scale smoothing splits chromosomes at their
 * fixed anchors) with `chains` chains each, one pass; kernel_ms (nullable)
 * receives the device time of the annealing kernel.  pos_out holds
 * sum(n_u)*3 floats (best chain of each region).  trace_out (nullable)
 * receives trace_cap move records of chain 0 of region 0. */
pmmc_status pmmc_smooth_batch_anneal(pmmc_ctx *ctx, int n_units,
                                     const pmmc_smooth_problem *units,
                                     const pmmc_anneal_params *prm,
                                     const float *step_sizes, int chains,
                                     float *pos_out, pmmc_result *res,
                                     double *kernel_ms, void *trace_out,
                                     int trace_cap);
/* The same with the regions packed back to back (a chromosome's beads cut
 * at its anchors, say): region u is beads [bead_off[u], bead_off[u+1]) of
 * pos (3 floats a bead), dist_to_next and fixed (nullable); bead_off holds
 * n_units+1 entries. */
pmmc_status pmmc_smooth_batch_anneal_packed(pmmc_ctx *ctx, int n_units, const int64_t *bead_off,
                                            const float *pos, const float *dist_to_next,
                                            const unsigned char *fixed,
                                            const pmmc_anneal_params *prm,
                                            const float *step_sizes, int chains, float *pos_out,
                                            pmmc_result *res, double *kernel_ms, void *trace_out,
                                            int trace_cap);
/* Smoothing kernel choice for the context's later smoothing calls.  A region
 * is annealed in windows of W proposals (W = 4, 8, 16 or 32 lanes of a warp
 * per chain: the proposals of the next W moves are scored at once and
 * resolved in order, a window closing at the first proposal that reads a
 * bead an accepted earlier one moved), W = window_long for regions with at
 * least long_min_free movable beads (the longest chains) and window_short
 * for the others; a window of 0 anneals those regions one move at a time,
 * two lanes per chain.  Every choice gives the same moves, decisions and
 * positions.  Default: window_short 8, window_long 32, long_min_free 20.
 * Regions whose chain does not fit a shared-memory slice always take one
 * move at a time. */
pmmc_status pmmc_smooth_set_window(pmmc_ctx *ctx, int window_short, int window_long,
                                   int long_min_free);
/* Many independent heatmap chains (distinct matrices), one CTA each.
 * trace_out (nullable) receives trace_cap records of unit 0's first moves. */
pmmc_status pmmc_heatmap_batch_anneal(pmmc_ctx *ctx, int n_units,
                                      const pmmc_heatmap_problem *units,
                                      const pmmc_anneal_params *prm,
                                      const float *step_sizes, float *pos_out,
                                      pmmc_result *res, double *kernel_ms,
                                      void *trace_out, int trace_cap);

/* Heatmap kernel choice for the context's later heatmap calls: each chain on
 * a thread-block cluster of `ctas` CTAs (1, 2, 4, 8 or 16, 16 being beyond the
 * portable cluster size; 0 = by the batch: 16 for up to 4 chains on maps of
 * 1024 beads or more, 8 when every chain can have its own eight SMs and the
 * maps have 512 beads or more, else 1).  In a cluster each CTA scores its
 * slice of every row and CTA 0 takes the decisions, so one chain uses the
 * special-function units and shared memory of several SMs. */
pmmc_status pmmc_heatmap_set_cluster(pmmc_ctx *ctx, int ctas);

/* ---------------- expected-distance heatmap ---------------- */
/* Replaces LooperSolver::createDistanceHeatmap (src/include/LooperSolver.hpp:
 * 3042-3085), which builds heatmap_dist from heatmap[level] on the host
 * before each heatmap level: for i <= j, d = scale * c^power where
 * c >= 1e-6 (0 below, -1 inside the diagonal band |i-j| < diag), mirrored;
 * then values above avg * stretching are clamped to it (avg: the mean over
 * j >= i + w, w the first diagonal holding a value above 1e-6,
 * Heatmap::getAvg / getDiagonalSize).  The caller passes the level's
 * constants (freqToDistHeatmapScale/Power, or the Inter ones for level 0, and
 * heatmapDistanceHeatmapStretching).  Host buffers of n*n floats; avg_out,
 * max_out and kernel_ms are optional.  The average is summed in FP64 (the
 * reference sums in float), so the clamp value can differ from the
 * reference's in its last bits. */
pmmc_status pmmc_distance_heatmap(pmmc_ctx *ctx, int n, const float *contact, int diag,
                                  float scale, float power, float stretching,
                                  float *dist_out, float *avg_out, float *max_out,
                                  double *kernel_ms);
/* The same on device buffers, enqueued on `stream` (NULL: the context's);
 * stats (device, 2 floats) receives avg and the clamp value. */
pmmc_status pmmc_distance_heatmap_device(pmmc_ctx *ctx, int n, const float *contact, int diag,
                                         float scale, float power, float stretching,
                                         float *dist, float *stats, void *stream);

/* ---------------- anchor-level expected distances ---------------- */
/* Replaces LooperSolver::calcAnchorExpectedDistancesHeatmap
 * (LooperSolver.hpp:5494-5627) and the dense n x n matrix it fills: the
 * expected distances of an anchor-level active region, written directly as
 * the CSR pmmc_arcs_problem takes (both directions, columns sorted, the
 * entries pmmc_arcs_dense_to_csr would keep of the reference's matrix).
 *   short arcs   the arcs of every active cluster (Cluster::arcs, indices
 *                into the chromosome's arcs, cluster-index ends) whose other
 *                end is not below it; the last write of a pair wins;
 *   long arcs    genomic-position arcs (InteractionArcs::long_arcs) resolved
 *                to anchors (Anchor::contains; the first anchor holding the
 *                position), then to active slots; a pair that already holds
 *                a distance >= 0 keeps it (a collision);
 *   influence    with anchor_heat (the n x n heatmap_anchor, row-major;
 *                Settings::useAnchorHeatmap on) every distance >= 0 above the
 *                diagonal is scaled by 1 - min(1, heat / max * influence),
 *                max the largest heatmap value from the first diagonal
 *                holding one above 1e-6 (Heatmap::getRange).
 * Distances are freqToDistance(score, memo = true) (LooperSolver.hpp:
 * 3949-3967): freq_memo[score] for 1 <= score <= 100 (the reference's
 * freq_to_distance table; it fills entries 2..100), otherwise the
 * countToDist* formula in FP64.  An arc end outside the active region maps
 * to slot 0, as the reference's std::map::operator[] inserts it.
 * n_anchors == 0 means the chromosome has no anchor list (long arcs are not
 * used).  cap >= 2 * (arc_ptr[n] + n_long) always suffices; with a smaller
 * cap or col/target NULL only *nnz is written (size query).  Long-arc
 * resolution, de-duplication, the influence and the CSR assembly run on the
 * device. */
typedef struct pmmc_anchor_targets_problem {
  int n;                       /* active-region size                       */
  const int *active;           /* n cluster indices (active_region)        */
  const int *arc_ptr;          /* n+1: arcs of cluster active[i]           */
  const int *arc_idx;          /* arc_ptr[n] indices into the arc table    */
  int n_arcs;                  /* the chromosome's arcs                    */
  const int *arc_start;        /* cluster index of each arc's start        */
  const int *arc_end;          /* cluster index of each arc's end          */
  const int *arc_score;        /* PET count                                */
  int n_long;                  /* the chromosome's long arcs               */
  const int *long_start;       /* genomic positions                        */
  const int *long_end;
  const int *long_score;
  int n_anchors;               /* the chromosome's anchors                 */
  const int *anchor_start;
  const int *anchor_end;
  int first_cluster;           /* chr_first_cluster of the chromosome      */
  const float *freq_memo;      /* 101 entries                              */
  float count_a, count_scale, count_shift, count_base; /* Settings::countToDist* */
  const float *anchor_heat;    /* n*n, NULL: no anchor heatmap             */
  float anchor_influence;      /* Settings::anchorHeatmapInfluence         */
} pmmc_anchor_targets_problem;

/* The counters the reference prints for the long arcs, and the device time
 * of each phase (long-arc mapping, its sort, resolution, CSR assembly with
 * the heatmap passes). */
typedef struct pmmc_anchor_targets_stats {
  int64_t applied, out_of_range, inactive, collision;
  float ms_map, ms_sort, ms_resolve, ms_assemble;
} pmmc_anchor_targets_stats;

pmmc_status pmmc_anchor_targets(pmmc_ctx *ctx, const pmmc_anchor_targets_problem *pr,
                                int *row_ptr, int *col, float *target, int64_t cap,
                                int64_t *nnz, pmmc_anchor_targets_stats *stats,
                                double *kernel_ms);

/* ---------------- stress refinement ---------------- */
/* Replaces LooperSolver::stressRefineAnchors(chr, max_iter, lr)
 * (LooperSolver.hpp:5638-5913): gradient descent on the anchors of one
 * chromosome after the anchor-level annealing.  The active region is sorted
 * by genomic position (ties: stable here, unspecified in the reference's
 * std::sort); pair targets are freqToDistance(score, memo = false) of the
 * chromosome's arcs (cluster-index ends) and long arcs (genomic positions
 * through Anchor::contains), the first of a pair wins, targets <= 1e-6 are
 * dropped, and consecutive anchors are left to the backbone when a backbone
 * constant exceeds 1e-6.  Energy: backbone k_{stretch|squeeze} ((d - t)/t)^2
 * with t = genomicLengthToDistance(gap); pairs ((d - t)/t)^2; angles
 * k_angular acos(c)^3 with its finite-difference gradient (h = 1e-3).  The
 * step halves when the energy rises (the run stops below 1e-6) and the run
 * stops when it improves by less than 1e-7 max(1, E) after 20 iterations.
 * order_out (n) receives the sorted active region, pos_out (n*3) the
 * refined positions in that order.  One cooperative launch runs every
 * iteration; each anchor's gradient is summed in the reference's order
 * (backbone, pairs in pair order, angles), so without the angle term the
 * positions equal the reference's bit for bit. */
typedef struct pmmc_stress_problem {
  int n;                       /* active-region size                       */
  const int *active;           /* n cluster indices, any order             */
  const int *genomic_pos;      /* n: Cluster::genomic_pos of each          */
  const float *pos;            /* n*3                                      */
  int n_arcs;                  /* arcs.arcs[chr]: cluster-index ends       */
  const int *arc_start, *arc_end, *arc_score;
  int n_long;                  /* arcs.long_arcs[chr]: genomic positions   */
  const int *long_start, *long_end, *long_score;
  int n_anchors;               /* arcs.anchors[chr]                        */
  const int *anchor_start, *anchor_end;
  int first_cluster;           /* chr_first_cluster[chr]                   */
  float count_a, count_scale, count_shift, count_base;  /* countToDist*    */
  float glen_base, glen_scale, glen_power;  /* genomicLengthToDist*       */
  float k_stretch, k_squeeze, k_angular;    /* springConstantStretch,
                                               springConstantSqueeze,
                                               springAngularConstant      */
} pmmc_stress_problem;

typedef struct pmmc_stress_result {
  int iterations;              /* iterations whose energy was evaluated    */
  int stop;                    /* 0 max_iter, 1 converged, 2 step < 1e-6  */
  float lr;                    /* step at exit                             */
  double total, backbone, hic, angular;  /* terms of the last evaluation   */
  int64_t n_pairs;             /* pair targets                             */
  double kernel_ms;            /* device time of the descent               */
} pmmc_stress_result;

pmmc_status pmmc_stress_refine(pmmc_ctx *ctx, const pmmc_stress_problem *pr, int max_iter,
                               float lr, int *order_out, float *pos_out,
                               pmmc_stress_result *res);

/* ---------------- equidistant model ---------------- */
/* Replaces the interpolation of HierarchicalChromosome::createEqidistantModel
 * (src/HierarchicalChromosome.cu:466-519; gpuHelper :1253-1447 and its
 * kernel parallelFind3DSmoothPosition :420-464): points every `res` bp from
 * pos_start, (pos_stop - pos_start + 1) / res + 1 of them, along one
 * chromosome's current level (n clusters in order: genomic positions gpos and
 * positions pos, n*3).  first_end is the first cluster's end, last_start the
 * last cluster's start (the reference's p1_end, p2_start).  *n_out receives
 * the number of points; with out == NULL or cap < *n_out nothing else
 * happens (size query).  Bit-identical to the reference's CPU path. */
pmmc_status pmmc_equidistant_model(pmmc_ctx *ctx, int n, const int *gpos, const float *pos,
                                   int first_end, int last_start, int pos_start,
                                   int pos_stop, int res, float *out, int64_t cap,
                                   int64_t *n_out, double *kernel_ms);

/* ---------------- HCM model file ---------------- */
/* Writes the reference's HCM text format, as HierarchicalChromosome::toFile
 * (src/HierarchicalChromosome.cu:530-552) with Cluster::toFile
 * (src/include/Cluster.hpp:175-181) and InteractionArc::toFile
 * (src/include/InteractionArc.hpp:122-125): a header, the factor names, one
 * line per cluster (start, end, orientation char, position, children given as
 * CSR child_ptr[n_clusters+1] / children), then per chromosome its name, root
 * cluster and arcs (CSR arc_ptr[n_chrs+1]; 7 ints per arc: start, end,
 * genomic_start, genomic_end, score, eff_score, factor).  Host code only. */
pmmc_status pmmc_hcm_write(const char *path, int n_clusters, const int *start, const int *end,
                           const char *orientation, const float *pos, const int *child_ptr,
                           const int *children, int n_factors, const char *const *factors,
                           int n_chrs, const char *const *chr_names, const int *chr_root,
                           const int *arc_ptr, const int *arcs);

/* ---------------- arc-level anneal that allocates nothing ------------- */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory -- code that must not call cudaMalloc because a host framework owns
 * the device pool and lends out only its own buffers, or a plugin running
 * under a fixed memory budget.  Every pointer in *pr is a DEVICE pointer (the
 * caller's inputs: positions, optional fixed flags, row_ptr/col/target);
 * pos_out is a device buffer of n*3 floats; res is a host struct.  One chain
 * is annealed exactly as pmmc_arcs_batch_* anneals a one-chain region with
 * two lanes per proposal and no drawing warp (key = seed, chain 0): the same
 * kernel, arc-list staging, repulsion sum and recompute order, so positions,
 * energies and move counts are bit-identical to that call.  All
 * intermediates live in one fixed device array of the library (688,352
 * bytes, about 0.69 MB), reserved on a device when the library's module is
 * loaded there -- lazily, at its first use, under CUDA's default lazy module
 * loading -- and held until the process exits: regions of at most 4096 beads
 * and 16384 arc-list entries, no loop constraints; a larger region returns
 * PMMC_ERR_BUDGET, loop constraints or malformed arc lists (row pointers out
 * of order, a column out of range) PMMC_ERR_INVALID, and a rejected call
 * writes nothing to pos_out.  Nothing is allocated: no cudaMalloc/cudaFree
 * and no allocating library call.  The array's device address is looked up
 * (with the device current) at the first call on each device and again after
 * the device's context changed (a cudaDeviceReset); that first call should
 * come before any stream capture.  The call blocks: it waits on `stream`
 * twice, for the check of the arc lists and for the result.  Calls share the
 * array, each one re-initialises it; calls whose work overlaps on the GPU
 * (two streams, two host threads) race on it. */
pmmc_status pmmc_arcs_anneal_noalloc(const pmmc_arcs_problem *pr,
                                     const pmmc_anneal_params *prm,
                                     float step_size, uint64_t seed,
                                     float *pos_out, pmmc_result *res,
                                     void *stream);

/* ---------------- request loop (continuous batching) ------------------ */
/* Replaces running region reconstructions one after another under the
 * reference's memory budget (-M, Settings::maxMemoryMB, checked by
 * checkMemoryBudget in the ensemble loop, apps/pMMC-reconstruct/
 * main_reconstruct.cpp:423, src/main.cpp:2018-2019).  A server accepts
 * arc-level regions from any host thread; a scheduler thread admits them in
 * arrival order as launch slots and device memory (budget_bytes, counted on
 * the device bytes of every resident region) free up, launches each admitted
 * wave as one persistent kernel on its own stream, and overlaps up to
 * max_waves waves on the device.  Every region anneals with the server's
 * parameters, its own step size and its own Philox key (seed, chain 0): its
 * result does not depend on the other regions in flight. */
typedef struct pmmc_server pmmc_server;

typedef struct {
  size_t budget_bytes;    /* device bytes of resident regions; 0 = half the free memory */
  int max_waves;          /* launches in flight at once; 0 = 8 */
  int max_wave_requests;  /* regions per launch; 0 = 4 x SM count */
  int lanes_per_chain;    /* 1, 2, 4, 8 or 32 lanes per proposal; 0 = by
                           * region size (1 from 1024 beads, 2 from 128,
                           * else 4) */
} pmmc_server_opts;

typedef struct {
  long long submitted, completed, rejected, failed, waves, queued;
  long long bytes_in_use, bytes_peak, budget_bytes;
  int running_peak;       /* most regions resident at once */
  int waves_peak;         /* most launches in flight at once */
} pmmc_server_stats;

pmmc_status pmmc_server_create(pmmc_ctx *ctx, const pmmc_anneal_params *prm,
                               const pmmc_server_opts *opts, pmmc_server **out);
/* Queues one region (host arrays, copied before the call returns).
 * PMMC_ERR_BUDGET if the region alone needs more device bytes than the
 * budget. */
pmmc_status pmmc_server_submit(pmmc_server *sv, const pmmc_arcs_problem *pr,
                               float step_size, uint64_t seed, long long *ticket);
/* done = 1 once the region's result is ready. */
pmmc_status pmmc_server_poll(pmmc_server *sv, long long ticket, int *done);
/* Blocks up to timeout_ms (< 0: no limit) for the result; on success the
 * ticket is released.  pos_out receives n*3 floats; latency_ms the time from
 * submit to the result landing in host memory.  PMMC_ERR_TIMEOUT leaves the
 * request queued. */
pmmc_status pmmc_server_wait(pmmc_server *sv, long long ticket, int timeout_ms,
                             float *pos_out, pmmc_result *res, double *latency_ms);
pmmc_status pmmc_server_get_stats(pmmc_server *sv, pmmc_server_stats *st);
/* Withdraws a request that is still queued: its wait then returns
 * PMMC_ERR_CANCELLED at once.  A request already admitted to a wave runs to
 * its end (PMMC_ERR_BUSY); an unknown ticket gives PMMC_ERR_NOT_FOUND. */
pmmc_status pmmc_server_cancel(pmmc_server *sv, long long ticket);
/* Finishes every queued and running region, then frees the server. */
void pmmc_server_destroy(pmmc_server *sv);

#ifdef __cplusplus
}
#endif
#endif /* PMMC_GB300_H_ */
