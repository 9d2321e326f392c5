// stress.cu -- gradient-descent stress refinement of a chromosome's anchors.
//
// LooperSolver::stressRefineAnchors (LooperSolver.hpp:5638-5913) runs after
// the anchor-level annealing: it sorts the active region by genomic
// position, collects one target per anchor pair from the chromosome's arcs
// and long arcs (the first of a pair wins), and descends
//   E = sum_i k_{str|sqz} ((|X_i - X_i+1| - b_i) / b_i)^2         backbone
//     + sum_pairs ((|X_i - X_j| - t_ij) / t_ij)^2                  pairs
//     + sum_i k_ang acos(cos angle_i)^3                            angles
// with analytic gradients for the first two, a forward difference (h = 1e-3)
// for the angles, a step halved whenever E rises and a relative stop test.
// The reference does this on one host core: O(pairs + 10 anchors) per
// iteration, thousands of iterations.
//
// Here the host builds the pair list once (the reference's filters and
// first-wins order; anchors found by binary search when sorted and
// disjoint) and lays it out per anchor in pair order; then one cooperative
// launch (one 16-warp block per SM) runs every iteration:
//   stage     the positions (16 bytes per anchor) into shared memory;
//   terms     every bond, pair and angle energy evaluated once across the
//             grid into L2-resident buffers (a pair's gradient stored at
//             both its anchors' slots, signed); FP64 energies per block;
//   barrier   (bounded wait) every block sums the block terms in one fixed
//             order and takes the same step decision;
//   sum       one warp per anchor adds its terms in the reference's
//             summation order -- bonds (i-1, i), its pairs in pair order,
//             the angle terms of the centres i-1, i, i+1 -- so every float
//             sum rounds as the reference's does, and moves the anchor;
//   barrier; next iteration.
// Without the angle term the positions equal the reference's bit for bit;
// acosf is CUDA's (the reference's is the host libm's), so with it they
// agree to rounding.
#include <algorithm>
#include <climits>
#include <numeric>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace pmmc {

namespace {

constexpr int kStressThreads = 512;
constexpr int kChunks = 8;  // 32-entry chunks of a pair row loaded per round
constexpr unsigned long long kBarrierLimitNs = 2000000000ull;  // 2 s per barrier

struct StressOut {
  int iterations;
  int stop;
  float lr;
  int err;
  double total, backbone, hic, angular;
};

struct StressArgs {
  int n;
  int n_pairs;
  const int *row_ptr;   // n+1: each anchor's slots in gv, pair order
  const int4 *pair;     // {low anchor, high anchor, target bits, slot of the low end}
  const int *slot_hi;   // slot of the high end of each pair
  const float *bb;      // n: backbone target to the next anchor (<= 1e-6: none)
  float k_stretch, k_squeeze, k_angular;
  int max_iter;
  float lr;
  float4 *X;            // n positions
  int staged;           // X copied to shared memory each iteration
  float4 *gv;           // 2 per pair: +gv at the low end's slot, -gv at the high end's
  float4 *bond;         // n: backbone gv of bond (i, i+1), w = 1 when the bond counts
  float2 *ang;          // 10 per centre: {energy, 1 when the bonds are long enough}:
                        // the centre's own, then anchor c-1+bi moved along ax
  double *part;         // 3 per block
  unsigned long long *bar;  // arrivals, counted up over the whole launch
  StressOut *out;
};

// One spring term ((|d| - t)/t)^2 of weight k: the gradient factor
// 2 k (|d| - t) / (t^2 |d|) and the FP64 energy, rounded as the reference
// (LooperSolver.hpp:5796-5825).
__device__ __forceinline__ float spring(float3 d, float t, float k, double *energy) {
  float dlen = ref_len(d.x, d.y, d.z);
  if (dlen < 1e-9f) dlen = 1e-9f;
  const float diff = __fsub_rn(dlen, t);
  const float e = __fdiv_rn(diff, t);
  *energy = __dmul_rn(__dmul_rn((double)k, (double)e), (double)e);
  return __fdiv_rn(__fmul_rn(__fmul_rn(2.0f, k), diff), __fmul_rn(__fmul_rn(t, t), dlen));
}

// k acos(c)^3 of the angle at centre c; false when a bond is shorter than
// 1e-9 (:5826-5845).
__device__ __forceinline__ bool angle_energy(float3 a, float3 b, float3 c, float k, float *E) {
  const float3 v1 = make_float3(__fsub_rn(b.x, a.x), __fsub_rn(b.y, a.y), __fsub_rn(b.z, a.z));
  const float3 v2 = make_float3(__fsub_rn(c.x, b.x), __fsub_rn(c.y, b.y), __fsub_rn(c.z, b.z));
  const float n1 = ref_len(v1.x, v1.y, v1.z), n2 = ref_len(v2.x, v2.y, v2.z);
  if (n1 < 1e-9f || n2 < 1e-9f) return false;
  const float dot =
      __fadd_rn(__fadd_rn(__fmul_rn(v1.x, v2.x), __fmul_rn(v1.y, v2.y)), __fmul_rn(v1.z, v2.z));
  float cs = __fdiv_rn(dot, __fmul_rn(n1, n2));
  if (cs > 1.0f) cs = 1.0f;
  if (cs < -1.0f) cs = -1.0f;
  const float th = acosf(cs);
  *E = __fmul_rn(__fmul_rn(__fmul_rn(k, th), th), th);
  return true;
}

__device__ __forceinline__ void add_comp(float3 &v, int a, float d) {
  if (a == 0) v.x = __fadd_rn(v.x, d);
  else if (a == 1) v.y = __fadd_rn(v.y, d);
  else v.z = __fadd_rn(v.z, d);
}

__device__ __forceinline__ unsigned long long atom_add_release(unsigned long long *p,
                                                               unsigned long long v) {
  unsigned long long old;
  asm volatile("atom.add.release.gpu.u64 %0, [%1], %2;" : "=l"(old) : "l"(p), "l"(v) : "memory");
  return old;
}
__device__ __forceinline__ unsigned long long ld_acquire(const unsigned long long *p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}

// Grid barrier number `round` over co-resident blocks (cooperative launch):
// one release-add per block on a counter that only grows, then an acquire
// poll until every block of this round arrived.  The wait is bounded; a
// timeout sets out->err and the block returns (the others then time out
// too, none of them waits without limit).
__device__ bool grid_barrier(unsigned long long *count, unsigned long long round,
                             StressOut *out) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    int ok = 1;
    const unsigned long long target = (round + 1) * gridDim.x;
    if (atom_add_release(count, 1ull) + 1ull < target) {
      const unsigned long long t0 = globaltimer_ns();
      unsigned spins = 0;
      while (ld_acquire(count) < target) {
        if ((++spins & 63u) == 0u && globaltimer_ns() - t0 > kBarrierLimitNs) {
          atomicExch(&out->err, 1);
          ok = 0;
          break;
        }
      }
    }
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

__device__ __forceinline__ float3 ldx(const float4 *X, int i, bool staged) {
  const float4 v = staged ? X[i] : __ldcg(X + i);
  return make_float3(v.x, v.y, v.z);
}

// Two phases per iteration.  A: every term evaluated once, in parallel over
// the whole grid (bonds, pairs, the ten angle energies of every centre)
// from positions staged in shared memory, written to L2-resident buffers.
// B (after the barrier and the step decision): one warp per anchor adds its
// terms in the reference's order -- bonds (i-1, i), its pair slots in pair
// order (256 loaded at a time through shared memory, each component summed
// by one lane), the
// angle differences of the centres i-1, i, i+1 -- and moves the anchor.  The
// sequential part of B is the float sum the reference's order requires: 3
// independent adds per term.
__global__ void __launch_bounds__(kStressThreads, 1) stress_kernel(StressArgs a) {
  extern __shared__ float4 sX[];
  __shared__ double s_e[3][kStressThreads / 32];
  __shared__ double s_tot[3];
  __shared__ float4 s_sum[kStressThreads / 32][32 * kChunks];  // a warp's round of its row
  const int n = a.n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int gtid = blockIdx.x * blockDim.x + threadIdx.x;
  const int gthreads = gridDim.x * blockDim.x;
  const int gwarp = blockIdx.x * (kStressThreads / 32) + warp;
  const int nwarps = gridDim.x * (kStressThreads / 32);
  const bool staged = a.staged != 0;
  const float4 *Xr = staged ? sX : a.X;
  const float h = 1e-3f;
  const int n_ang = a.k_angular > 0.0f && n > 2 ? 10 * (n - 2) : 0;
  float lr = a.lr;
  double prev_total = 1e300;
  unsigned long long round = 0;
  // a thread's pair (when there is at most one per thread) stays in registers
  const bool one_pair = a.n_pairs <= gthreads;
  int4 my_pair = make_int4(0, 0, 0, 0);
  int my_hi = 0;
  if (one_pair && gtid < a.n_pairs) {
    my_pair = __ldg(a.pair + gtid);
    my_hi = __ldg(a.slot_hi + gtid);
  }
  for (int it = 0; it < a.max_iter; ++it) {
    if (staged) {
      for (int i = threadIdx.x; i < n; i += blockDim.x) sX[i] = __ldcg(a.X + i);
      __syncthreads();
    }
    // ---- A: every term once ----
    double eb = 0.0, eh = 0.0, ea = 0.0;
    for (int i = gtid; i + 1 < n; i += gthreads) {
      const float t = __ldg(a.bb + i);
      float4 out = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
      if (t > 1e-6f) {
        const float3 x0 = ldx(Xr, i, staged), x1 = ldx(Xr, i + 1, staged);
        const float3 d =
            make_float3(__fsub_rn(x0.x, x1.x), __fsub_rn(x0.y, x1.y), __fsub_rn(x0.z, x1.z));
        const float dl = ref_len(d.x, d.y, d.z);
        const float e = __fdiv_rn(__fsub_rn(dl < 1e-9f ? 1e-9f : dl, t), t);
        double en;
        const float gm = spring(d, t, e >= 0.0f ? a.k_stretch : a.k_squeeze, &en);
        eb = __dadd_rn(eb, en);
        out = make_float4(__fmul_rn(d.x, gm), __fmul_rn(d.y, gm), __fmul_rn(d.z, gm), 1.0f);
      }
      a.bond[i] = out;
    }
    for (int p = gtid; p < a.n_pairs; p += gthreads) {
      const int4 pr = one_pair ? my_pair : __ldg(a.pair + p);
      const float t = __int_as_float(pr.z);
      const float3 xi = ldx(Xr, pr.x, staged), xj = ldx(Xr, pr.y, staged);
      const float3 d =
          make_float3(__fsub_rn(xi.x, xj.x), __fsub_rn(xi.y, xj.y), __fsub_rn(xi.z, xj.z));
      double en;
      const float gm = spring(d, t, 1.0f, &en);
      eh = __dadd_rn(eh, en);
      const float3 g = make_float3(__fmul_rn(d.x, gm), __fmul_rn(d.y, gm), __fmul_rn(d.z, gm));
      a.gv[pr.w] = make_float4(g.x, g.y, g.z, 0.0f);
      a.gv[one_pair ? my_hi : __ldg(a.slot_hi + p)] = make_float4(-g.x, -g.y, -g.z, 0.0f);
    }
    for (int w = gtid; w < n_ang; w += gthreads) {
      const int c = 1 + w / 10, m = w % 10;
      float3 p0 = ldx(Xr, c - 1, staged), p1 = ldx(Xr, c, staged), p2 = ldx(Xr, c + 1, staged);
      if (m > 0) {
        const int bi = (m - 1) / 3, ax = (m - 1) % 3;
        float3 &q = bi == 0 ? p0 : (bi == 1 ? p1 : p2);
        add_comp(q, ax, h);
      }
      float val = 0.0f;
      const bool ok = angle_energy(p0, p1, p2, a.k_angular, &val);
      a.ang[w] = make_float2(val, ok ? 1.0f : 0.0f);
      if (m == 0 && ok) ea = __dadd_rn(ea, (double)val);
    }
    // block terms, then one fixed-order total in every block
    eb = warp_sum_d(eb);
    eh = warp_sum_d(eh);
    ea = warp_sum_d(ea);
    if (lane == 0) {
      s_e[0][warp] = eb;
      s_e[1][warp] = eh;
      s_e[2][warp] = ea;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double t0 = 0.0, t1 = 0.0, t2 = 0.0;
      for (int w = 0; w < kStressThreads / 32; ++w) {
        t0 += s_e[0][w];
        t1 += s_e[1][w];
        t2 += s_e[2][w];
      }
      a.part[3 * blockIdx.x] = t0;
      a.part[3 * blockIdx.x + 1] = t1;
      a.part[3 * blockIdx.x + 2] = t2;
    }
    if (!grid_barrier(a.bar, round++, a.out)) return;
    if (warp == 0) {
      double t0 = 0.0, t1 = 0.0, t2 = 0.0;
      for (int b = lane; b < (int)gridDim.x; b += 32) {
        t0 += __ldcg(a.part + 3 * b);
        t1 += __ldcg(a.part + 3 * b + 1);
        t2 += __ldcg(a.part + 3 * b + 2);
      }
      t0 = warp_sum_d(t0);
      t1 = warp_sum_d(t1);
      t2 = warp_sum_d(t2);
      if (lane == 0) {
        s_tot[0] = t0;
        s_tot[1] = t1;
        s_tot[2] = t2;
      }
    }
    __syncthreads();
    const double total = (s_tot[0] + s_tot[1]) + s_tot[2];
    bool stop_lr = false;
    if (total > prev_total && it > 0) {
      lr *= 0.5f;
      if (lr < 1e-6f) stop_lr = true;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      a.out->iterations = it + 1;
      a.out->total = total;
      a.out->backbone = s_tot[0];
      a.out->hic = s_tot[1];
      a.out->angular = s_tot[2];
      a.out->lr = lr;
      a.out->stop = stop_lr ? 2 : 0;
    }
    if (stop_lr) return;
    // ---- B: each anchor's sum in the reference's order, then the step ----
    for (int k = gwarp; k < n; k += nwarps) {
      // every load of the anchor issued up front
      const int q0 = __ldg(a.row_ptr + k), q1 = __ldg(a.row_ptr + k + 1);
      const float4 bprev = k >= 1 ? __ldcg(a.bond + k - 1) : make_float4(0, 0, 0, 0);
      const float4 bnext = k + 1 < n ? __ldcg(a.bond + k) : make_float4(0, 0, 0, 0);
      // lanes 0-11: centre k-1+L/4, its energy (L%4 == 0) or anchor k moved
      // along axis L%4-1
      float2 av = make_float2(0.0f, 0.0f);
      if (n_ang && lane < 12) {
        const int c = k - 1 + lane / 4, m = lane % 4;
        if (c >= 1 && c + 1 < n)
          av = __ldcg(a.ang + 10 * (c - 1) + (m == 0 ? 0 : 1 + 3 * (k - (c - 1)) + m - 1));
      }
      const float4 xk = lane == 0 ? __ldcg(a.X + k) : make_float4(0, 0, 0, 0);
      float4 cur[kChunks];
#pragma unroll
      for (int u = 0; u < kChunks; ++u) {
        const int q = q0 + 32 * u + lane;
        cur[u] = q < q1 ? __ldcg(a.gv + q) : make_float4(0, 0, 0, 0);
      }
      float3 g = make_float3(0.0f, 0.0f, 0.0f);
      if (bprev.w != 0.0f)
        g = make_float3(__fsub_rn(g.x, bprev.x), __fsub_rn(g.y, bprev.y), __fsub_rn(g.z, bprev.z));
      if (bnext.w != 0.0f)
        g = make_float3(__fadd_rn(g.x, bnext.x), __fadd_rn(g.y, bnext.y), __fadd_rn(g.z, bnext.z));
      // lanes 0, 1, 2 each carry one component through the pair sum
      float acc = lane == 0 ? g.x : (lane == 1 ? g.y : g.z);
      for (int base = q0; base < q1; base += 32 * kChunks) {
#pragma unroll
        for (int u = 0; u < kChunks; ++u) s_sum[warp][32 * u + lane] = cur[u];
        __syncwarp();
        // the next round in flight while lane 0 adds this one
#pragma unroll
        for (int u = 0; u < kChunks; ++u) {
          const int q = base + 32 * (kChunks + u) + lane;
          cur[u] = q < q1 ? __ldcg(a.gv + q) : make_float4(0, 0, 0, 0);
        }
        if (lane < 3) {
          const int cnt = min(32 * kChunks, q1 - base);
          const float *col = reinterpret_cast<const float *>(&s_sum[warp][0]) + lane;
#pragma unroll 32
          for (int i = 0; i < cnt; ++i) acc = __fadd_rn(acc, col[4 * i]);
        }
        __syncwarp();
      }
      g = make_float3(__shfl_sync(0xffffffffu, acc, 0), __shfl_sync(0xffffffffu, acc, 1),
                      __shfl_sync(0xffffffffu, acc, 2));
      if (n_ang) {
        for (int ci = 0; ci < 3; ++ci) {
          const float2 e0 = make_float2(__shfl_sync(0xffffffffu, av.x, 4 * ci),
                                        __shfl_sync(0xffffffffu, av.y, 4 * ci));
          for (int ax = 0; ax < 3; ++ax) {
            const float vx = __shfl_sync(0xffffffffu, av.x, 4 * ci + 1 + ax);
            const float ok = __shfl_sync(0xffffffffu, av.y, 4 * ci + 1 + ax);
            if (e0.y != 0.0f && ok != 0.0f)
              add_comp(g, ax, __fdiv_rn(__fsub_rn(vx, e0.x), h));
          }
        }
      }
      if (lane == 0)
        a.X[k] = make_float4(__fsub_rn(xk.x, __fmul_rn(lr, g.x)), __fsub_rn(xk.y, __fmul_rn(lr, g.y)),
                             __fsub_rn(xk.z, __fmul_rn(lr, g.z)), 0.0f);
    }
    if (prev_total - total < 1e-7 * fmax(1.0, total) && it > 20) {
      if (blockIdx.x == 0 && threadIdx.x == 0) a.out->stop = 1;
      return;
    }
    prev_total = total;
    if (!grid_barrier(a.bar, round++, a.out)) return;
  }
}

// genomicLengthToDistance (LooperSolver.hpp:3900-3904).
double genomic_length_to_distance(int length, const pmmc_stress_problem *p) {
  return (double)p->glen_base +
         (double)p->glen_scale * std::pow(length / 1000.0, (double)p->glen_power);
}

}  // namespace

}  // namespace pmmc

using namespace pmmc;

extern "C" pmmc_status pmmc_stress_refine(pmmc_ctx *ctx, const pmmc_stress_problem *pr,
                                          int max_iter, float lr, int *order_out,
                                          float *pos_out, pmmc_stress_result *res) {
  if (!ctx || !pr || pr->n < 0 || pr->n_arcs < 0 || pr->n_long < 0 || pr->n_anchors < 0 ||
      (pr->n > 0 && (!pr->active || !pr->genomic_pos || !pr->pos || !order_out || !pos_out)) ||
      (pr->n_arcs > 0 && (!pr->arc_start || !pr->arc_end || !pr->arc_score)) ||
      (pr->n_long > 0 && (!pr->long_start || !pr->long_end || !pr->long_score)) ||
      (pr->n_anchors > 0 && (!pr->anchor_start || !pr->anchor_end)))
    return fail(ctx, PMMC_ERR_INVALID, "stress refinement: bad arguments");
  const int n = pr->n;
  pmmc_stress_result r{};
  r.lr = lr;
  for (int i = 0; i < n; ++i) order_out[i] = pr->active[i];
  if (n > 0) std::copy(pr->pos, pr->pos + 3 * (size_t)n, pos_out);
  if (max_iter <= 0 || n < 2) {
    if (res) *res = r;
    return PMMC_OK;
  }
  // active region by genomic position (:5647-5650)
  std::vector<int> ord(n);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int x, int y) {
    return pr->genomic_pos[x] < pr->genomic_pos[y];
  });
  for (int i = 0; i < n; ++i) order_out[i] = pr->active[ord[i]];
  const int n_anc = pr->n_anchors, cs = pr->first_cluster;
  std::vector<int> slot_of_cluster(std::max(n_anc, 1), -1);
  for (int i = 0; i < n; ++i) {
    const int ci = order_out[i];
    if (ci >= cs && ci - cs < n_anc) slot_of_cluster[ci - cs] = i;
  }
  // pair targets, the first of a pair wins (:5670-5729)
  const bool with_backbone = pr->k_stretch > 1e-6f || pr->k_squeeze > 1e-6f;
  struct TargetPair {
    int i, j;
    float t;
  };
  std::vector<TargetPair> pairs;
  std::unordered_map<uint64_t, int> seen;
  seen.reserve((size_t)(pr->n_arcs + pr->n_long) + 16);
  auto take_target = [&](int ai, int aj, float t) {
    if (ai == aj) return;
    if (ai > aj) std::swap(ai, aj);
    if (with_backbone && aj - ai <= 1) return;
    const uint64_t key = (uint64_t)ai * (uint64_t)n + (uint64_t)aj;
    if (seen.emplace(key, (int)pairs.size()).second) pairs.push_back({ai, aj, t});
  };
  for (int k = 0; k < pr->n_arcs; ++k) {
    const int ca = pr->arc_start[k], cb = pr->arc_end[k];
    if (ca < cs || ca - cs >= n_anc || cb < cs || cb - cs >= n_anc) continue;
    const int ai = slot_of_cluster[ca - cs], aj = slot_of_cluster[cb - cs];
    if (ai < 0 || aj < 0) continue;
    const float t = count_to_distance(pr->arc_score[k], pr->count_a, pr->count_scale,
                                      pr->count_shift, pr->count_base);
    if (t > 1e-6f) take_target(ai, aj, t);
  }
  // Anchor::contains, the first anchor holding pos: binary search over
  // sorted, disjoint anchors, else the reference's scan
  bool sorted = true;
  for (int i = 1; i < n_anc && sorted; ++i)
    sorted = pr->anchor_start[i] > pr->anchor_start[i - 1] &&
             pr->anchor_start[i] > pr->anchor_end[i - 1];
  auto anchor_at = [&](int pos) -> int {
    if (sorted) {
      const int i = (int)(std::upper_bound(pr->anchor_start, pr->anchor_start + n_anc, pos) -
                          pr->anchor_start) - 1;
      return (i >= 0 && pos <= pr->anchor_end[i]) ? i : -1;
    }
    for (int i = 0; i < n_anc; ++i)
      if (pos >= pr->anchor_start[i] && pos <= pr->anchor_end[i]) return i;
    return -1;
  };
  for (int k = 0; k < pr->n_long; ++k) {
    const int ia = anchor_at(pr->long_start[k]), ib = anchor_at(pr->long_end[k]);
    if (ia < 0 || ib < 0) continue;
    const int as = slot_of_cluster[ia], bs = slot_of_cluster[ib];
    if (as < 0 || bs < 0) continue;
    const float t = count_to_distance(pr->long_score[k], pr->count_a, pr->count_scale,
                                      pr->count_shift, pr->count_base);
    if (t > 1e-6f) take_target(as, bs, t);
  }
  r.n_pairs = (int64_t)pairs.size();
  // each anchor's slots in pair order; a pair knows its two slots
  std::vector<int> row_ptr(n + 1, 0);
  for (const TargetPair &p : pairs) {
    ++row_ptr[p.i + 1];
    ++row_ptr[p.j + 1];
  }
  for (int i = 0; i < n; ++i) row_ptr[i + 1] += row_ptr[i];
  std::vector<int> fill(row_ptr.begin(), row_ptr.end() - 1);
  std::vector<int4> pair4(std::max<size_t>(1, pairs.size()));
  std::vector<int> slot_hi(std::max<size_t>(1, pairs.size()));
  for (size_t q = 0; q < pairs.size(); ++q) {
    const TargetPair &p = pairs[q];
    int tb;
    memcpy(&tb, &p.t, 4);
    pair4[q] = make_int4(p.i, p.j, tb, fill[p.i]++);
    slot_hi[q] = fill[p.j]++;
  }
  // backbone targets from the genomic gaps (:5754-5762)
  std::vector<float> bb(n, -1.0f);
  for (int i = 0; i + 1 < n; ++i) {
    const int gap = std::abs(pr->genomic_pos[ord[i + 1]] - pr->genomic_pos[ord[i]]);
    if (gap > 0) bb[i] = (float)genomic_length_to_distance(gap, pr);
  }
  std::vector<float4> X(n);
  for (int i = 0; i < n; ++i)
    X[i] = make_float4(pr->pos[3 * ord[i]], pr->pos[3 * ord[i] + 1], pr->pos[3 * ord[i] + 2], 0.0f);

  // one cooperative launch: every block resident
  // one 16-warp block per SM (fewer for a small region: a warp per anchor in
  // the summing phase);
  // positions staged in shared memory when they fit
  cudaFuncAttributes fa{};
  cudaFuncGetAttributes(&fa, stress_kernel);
  const size_t dyn_max = ctx->smem_optin > fa.sharedSizeBytes ? ctx->smem_optin - fa.sharedSizeBytes : 0;
  // set on every call: the attribute belongs to the current device
  cudaFuncSetAttribute(stress_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn_max);
  const size_t smem = sizeof(float4) * (size_t)n;
  const int staged = smem <= dyn_max ? 1 : 0;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, stress_kernel, kStressThreads,
                                                staged ? smem : 0);
  if (per_sm < 1)
    return fail(ctx, PMMC_ERR_CUDA, "stress refinement: kernel does not fit an SM");
  const int want = (n + kStressThreads / 32 - 1) / (kStressThreads / 32);
  const int blocks = std::max(1, std::min(want, per_sm * ctx->sm_count));
  cudaStream_t s = ctx->stream;
  const size_t n_pairs = pairs.size();
  const size_t n_ang = n > 2 ? 10 * (size_t)(n - 2) : 1;
  DevBuf<float4> dX, dgv, dbond;
  DevBuf<int> drow, dslot;
  DevBuf<int4> dpair;
  DevBuf<float> dbb;
  DevBuf<float2> dang;
  DevBuf<double> dpart;
  DevBuf<unsigned long long> dbar;
  DevBuf<StressOut> dout;
  cudaError_t e = dX.alloc(n);
  if (e == cudaSuccess) e = dgv.alloc(std::max<size_t>(1, 2 * n_pairs));
  if (e == cudaSuccess) e = dbond.alloc(n);
  if (e == cudaSuccess) e = drow.alloc(n + 1);
  if (e == cudaSuccess) e = dslot.alloc(slot_hi.size());
  if (e == cudaSuccess) e = dpair.alloc(pair4.size());
  if (e == cudaSuccess) e = dbb.alloc(n);
  if (e == cudaSuccess) e = dang.alloc(n_ang);
  if (e == cudaSuccess) e = dpart.alloc(3 * (size_t)blocks);
  if (e == cudaSuccess) e = dbar.alloc(1);
  if (e == cudaSuccess) e = dout.alloc(1);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dX.p, X.data(), sizeof(float4) * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(drow.p, row_ptr.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dpair.p, pair4.data(), sizeof(int4) * pair4.size(), cudaMemcpyHostToDevice,
                        s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dslot.p, slot_hi.data(), sizeof(int) * slot_hi.size(),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dbb.p, bb.data(), sizeof(float) * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(dbar.p, 0, sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(dout.p, 0, sizeof(StressOut), s);
  if (e != cudaSuccess)
    return fail(ctx, e == cudaErrorMemoryAllocation ? PMMC_ERR_NOMEM : PMMC_ERR_CUDA,
                "stress refinement: %s", cudaGetErrorString(e));
  StressArgs args{n,         (int)n_pairs, drow.p,   dpair.p,    dslot.p,      dbb.p,
                  pr->k_stretch, pr->k_squeeze, pr->k_angular, max_iter, lr, dX.p,
                  staged,    dgv.p,        dbond.p,  dang.p,     dpart.p,
                  dbar.p,    dout.p};
  void *kargs[] = {&args};
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  e = cudaLaunchCooperativeKernel((const void *)stress_kernel, dim3(blocks), dim3(kStressThreads),
                                  kargs, staged ? smem : 0, s);
  cudaEventRecord(e1, s);
  StressOut o{};
  std::vector<float4> Xo(n);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&o, dout.p, sizeof(StressOut), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(Xo.data(), dX.p, sizeof(float4) * n, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  float ms = 0.0f;
  if (e == cudaSuccess) cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess)
    return fail(ctx, PMMC_ERR_CUDA, "stress refinement: %s", cudaGetErrorString(e));
  if (o.err) return fail(ctx, PMMC_ERR_TIMEOUT, "stress refinement: grid barrier timed out");
  for (int i = 0; i < n; ++i) {
    pos_out[3 * i] = Xo[i].x;
    pos_out[3 * i + 1] = Xo[i].y;
    pos_out[3 * i + 2] = Xo[i].z;
  }
  r.iterations = o.iterations;
  r.stop = o.stop;
  r.lr = o.lr;
  r.total = o.total;
  r.backbone = o.backbone;
  r.hic = o.hic;
  r.angular = o.angular;
  r.kernel_ms = ms;
  if (res) *res = r;
  return PMMC_OK;
}
