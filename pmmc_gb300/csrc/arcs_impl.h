// arcs_impl.h -- arc-level annealing internals shared by the batched,
// allocation-free and serving paths (host and device layouts, packing,
// launch).
#pragma once
#include <cstdint>
#include <vector>

#include <cuda_runtime.h>

#include "common.cuh"
#include "internal.h"

namespace pmmc {

struct ArcsUnit {
  int n;          // beads
  int n_mov;      // movable beads
  int pos_off;    // float4 index into pos0
  int rp_off;     // index into row_ptr (n+1 entries, unit-relative values)
  int nbr_off;    // index into nbr / inv_t (spring entries, target >= 1e-6)
  int nnz;
  int mov_off;    // index into movable, -1 = all beads movable
  int lrp_off;    // index into loop row_ptr (n+1), -1 = no loops
  int lent_off;   // index into loop entries
  int n_lent;
  int lst_off;    // index into the loop list (one entry per constraint)
  int n_loops;
  int null_off;   // index into the listed-but-inert pairs (0 <= target < 1e-6)
  int n_null;
  int chains;
  int chain_base; // global chain id of the unit's chain 0
  long long out_off;  // float index of chain 0's xyz output
  float step;
  int rng_chain;  // Philox chain id of the unit's chain 0
  uint64_t seed;  // Philox key of the unit's chains
  int arc_off;    // index into the int4 list array of the region's springs,
  int n_arcs;     // one entry {i, j, target bits, 1/target bits} per arc;
                  // n_arcs < 0: no list (recomputes walk the arc lists)
};

struct ArcsDevParams {
  float max_temp;
  float inv_scale;
  float inv_coef;
  float improvement;
  float k_stretch;
  float k_squeeze;
  float sphere_r;
  int min_successes;
  int window;      // milestone window (moves)
  int fails;       // consecutive misses that stop a chain
  int resync;      // FP64 recompute interval (0 = off)
  int use2d;
  int stop_all;    // the first converged chain stops the unit's others (the
                   // others read the flag at their milestones)
  int trace_cap;   // trace records per traced chain (tests)
  int trace_chains; // chains 0..trace_chains-1 (region 0's) are traced
  int stall_draws; // tests only: drawing warps never publish (the chain's
                   // bounded wait runs out and it ends with status 3)
  long long cap;   // hard move cap (0: no move)
  int cap_is_error;
  int ms_guard;    // reference-kernel rule: ratio test only when E_ms > 1e-10
  uint64_t seed;   // default Philox key (each unit carries its own)
  float dtpow[33];  // dt^l, l = 0..32
  // extended energy (off unless ext): bonds to the next bead with one
  // target, and the stiffness angle term at every interior bead
  int ext;
  float bond_t, inv_bond_t, kb_stretch, kb_squeeze, k_angle;
};

// per-warp scratch: 32 drawn moves (int4) + their ratio thresholds, and the
// window's per-slot delta, conflict mask and (tracing) local scores
// per chain: a ring of kRing drawn moves (16 B) and thresholds (4 B), three
// 32-float trace rows, and the words a drawing warp and its chain's warp
// exchange (ArcsRingCtl).  The ring holds four rounds of 32 draws, so a
// drawing warp stays two rounds ahead of windows that use ~30 moves each.
constexpr int kRing = 128;
constexpr int kMoveBufBytes = kRing * 16 + kRing * 4 + 3 * 32 * 4 + 64;
constexpr int kRingCtlOffset = kRing * 16 + kRing * 4 + 3 * 32 * 4;

struct ArcsRingCtl {
  long long filled;    // moves [0, filled) are drawn
  long long consumed;  // moves [0, consumed) are used up
  int item;            // the pair's current item
  int state;           // 0 running, 1 chain finished, 2 the drawing warp gave up
};
constexpr int kCtaHeader = 256;                    // dt^l table shared by the CTA

// Host-side packing of regions into the flat arrays the kernel reads: float4
// positions, spring-only CSR arc lists {col, target bits} with reciprocals,
// listed-but-inert pairs, movable list, loop-constraint lists.
struct ArcsPack {
  std::vector<ArcsUnit> units;
  std::vector<float4> pos;
  std::vector<int> rp, mov, lrp;
  std::vector<int2> nbr, nulls;
  std::vector<float> inv;
  std::vector<float4> lent;
  std::vector<int4> lst;      // loop constraints, then each region's spring list
  long long out_floats = 0;  // xyz floats over all chains
  int chains = 0;            // chains over all units
  // Appends one region with `chains` chains; Philox key `seed`, chain ids
  // rng_chain .. rng_chain + chains - 1.  The region must be valid.
  void add(const pmmc_arcs_problem &pr, int n_chains, float step, uint64_t seed, int rng_chain);
  // Appends every region of another pack (offsets rebased).
  void append(const ArcsPack &o);
  // Placeholder entries so that no device array is empty.
  void finish();
  // Empties the pack, keeping every array's capacity.
  void clear();
};

// Shared-memory bytes of one chain's slice: everything staged / positions only.
size_t arcs_unit_smem(int n, int nnz, int n_mov, bool has_mov);
size_t arcs_unit_smem_min(int n);
pmmc_status arcs_validate(pmmc_ctx *ctx, const pmmc_arcs_problem *pr);
ArcsDevParams arcs_make_params(const pmmc_anneal_params *prm, uint64_t seed, bool stop_all);

// Device pointers of one persistent pass.
struct ArcsLaunch {
  const ArcsUnit *units;
  const int2 *items;
  int n_items;
  int *head;
  const float4 *pos0;
  const int *row_ptr;
  const int2 *nbr;
  const float *inv_t;
  const int *movable;
  const int *lrp;
  const float4 *lent;
  const int4 *lst;
  const int2 *nulls;
  float *pos_out;
  ChainOut *outs;
  int *done;
  MoveTrace *trace;
  const double *bases;  // frozen repulsion per unit (NULL: each chain computes it)
};

// One persistent pass of `grid` CTAs x `warps` chains over the items on `s`.
// prod: every chain gets a second warp that draws its moves ahead (lanes 1
// or 2 only).
cudaError_t arcs_launch(const ArcsLaunch &a, const ArcsDevParams &P, bool nb_smem, int lanes,
                        int grid, int warps, int smem_per_warp, cudaStream_t s,
                        bool prod = false);
// The frozen repulsion of every unit into bases[u] (one block per unit).
cudaError_t arcs_bases(const ArcsUnit *units, int n_units, const float4 *pos0,
                       const int *row_ptr, const int2 *nbr, const int2 *nulls, double *bases,
                       cudaStream_t s);
// Resident CTAs per SM of that configuration (at least 1).
int arcs_ctas_per_sm(bool nb_smem, int lanes, int warps, int smem_per_warp, bool prod = false);
// Raise the dynamic shared-memory limit of every instantiation to `bytes`.
void arcs_set_smem_limit(int bytes);

}  // namespace pmmc
