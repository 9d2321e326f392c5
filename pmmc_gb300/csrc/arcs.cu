// arcs.cu -- arc-level (anchor) simulated annealing on GB300.
//
// Energy of an active region (LooperSolver.hpp:3215-3281, 3339-3371,
// 4700-4730; ParallelMonteCarloArcs.cu:294-351):
//   springs  sum over arcs (i,j), e_ij >= 1e-6:  k(d)*((d - e)/e)^2,
//            k = stretch if d >= e else squeeze
//   loops    sum over loop constraints: k_l (d - r0)^2
//   sphere   sum over beads: max(0, |p| - R)^2
//   and, in the initial score only, 1/d for every pair without an arc (the
//   reference's -1 entries).  Moves are scored incrementally on the moved
//   bead's arcs, so the running total is  R0 + springs + loops + sphere  with
//   R0 the repulsion of the starting structure; the FP64 recompute uses the
//   same definition.
//
// Layout in device memory: beads as float4 (16 B, one vector load), per-bead
// arc lists as CSR with {col, target} packed in one int2 (8 B) and 1/target
// beside it.  A chain is one warp: the region's positions and arc lists are
// staged in the warp's slice of shared memory (arc lists fall back to
// L1-cached global loads when the region is too large).  Proposals come from
// a counter-based Philox stream (move m: bead, displacement and the
// precomputed Metropolis ratio threshold), drawn 32 at a time into a
// 128-move ring -- by the chain's own warp, or by a second "drawing" warp
// that stays ahead of it.  The chain scores W = 32/G proposals at once (G
// lanes each) against the positions at the window's start and resolves them
// in order (downhill slots at once, uphill slots by a warp prefix sum of the
// accepted changes); the window ends at the first slot whose bead or
// partner an accepted earlier slot moved (a per-bead slot mask in shared
// memory finds those), so the accepted sequence is the one-move-at-a-time
// one.  The per-move delta is FP32, the running total a float-float pair
// refreshed by an energy recompute every `resync` moves, and the milestones
// and the end-of-chain recompute are FP64.
//
// Work distribution: persistent warps (or warp pairs) pull (unit, chain)
// items from an atomic queue, largest regions first, one launch per
// shared-memory size class; the classes run on forked streams and the whole
// pass is captured in a CUDA graph.  An autotuner picks each class's lanes
// per proposal, chains per CTA and drawing warp; the classes whose regions
// set the pass's length take the lowest-latency configuration.
#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include <cuda.h>  // driver types only (CUcontext); no link to the driver library

#include "arcs_impl.h"

namespace pmmc {


__device__ __forceinline__ float dist3(float ax, float ay, float az, float4 b) {
  const float x = ax - b.x, y = ay - b.y, z = az - b.z;
  return sqrtf(x * x + y * y + z * z);
}

// |a - b| as the reference rounds it (see ref_len).
__device__ __forceinline__ float fast_len(float ax, float ay, float az, float4 b) {
  return ref_len(__fsub_rn(ax, b.x), __fsub_rn(ay, b.y), __fsub_rn(az, b.z));
}

// 1/t for a target t >= 1e-6: the approximate reciprocal refined by one
// Newton-Raphson step, r' = r + r (1 - t r), which leaves it within about half
// an ulp of the exact reciprocal (Newton's method for f(r) = 1/r - t).  One
// special-function operation and two fused multiply-adds, where the
// correctly rounded library reciprocal costs several times that.
__device__ __forceinline__ float recip_nr(float t) {
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(t));
  return fmaf(r, fmaf(-t, r, 1.0f), r);
}

// Spring term of one arc: ((len - t) / t)^2 * k, with 1/t precomputed.
__device__ __forceinline__ float spring_fast(float len, float t, float it, float ks,
                                             float kq) {
  const float f = (len - t) * it;
  return f * f * (f >= 0.0f ? ks : kq);
}

// float-float accumulation (Knuth two-sum) of a float increment
__device__ __forceinline__ void ff_add(float &hi, float &lo, float d) {
  const float s = hi + d;
  const float bb = s - hi;
  const float err = (hi - (s - bb)) + (d - bb);
  const float l = lo + err;
  hi = s + l;
  lo = l - (hi - s);
}

// FP64 energy without repulsion: springs (pairs counted once, col < row so
// that the target is the reference's upper-triangle entry v[col][row]),
// loops and sphere.  Whole warp; result on every lane.
__device__ double arcs_spring_energy(int n, const float4 *spos, const int *srp,
                                     const int2 *nb, const int4 *loops,
                                     int n_loops, const ArcsDevParams &P,
                                     int lane) {
  double acc = 0.0;
  for (int i = lane; i < n; i += 32) {
    const float4 pi = spos[i];
    const int e1 = srp[i + 1];
    for (int e = srp[i]; e < e1; ++e) {
      const int2 ent = nb[e];
      if (ent.x >= i) continue;
      const float t = __int_as_float(ent.y);
      const float f = (dist3(pi.x, pi.y, pi.z, spos[ent.x]) - t) / t;
      const double df = f;
      acc += df * df * (double)(df >= 0.0 ? P.k_stretch : P.k_squeeze);
    }
    acc += sphere_penalty(pi.x, pi.y, pi.z, P.sphere_r);
  }
  for (int c = lane; c < n_loops; c += 32) {
    const int4 L = loops[c];
    const double d = dist3(spos[L.x].x, spos[L.x].y, spos[L.x].z, spos[L.y]);
    const double delta = d - (double)__int_as_float(L.w);
    acc += (double)__int_as_float(L.z) * delta * delta;
  }
  return warp_sum_d(acc);
}

// ---------------------------------------------------------------------------
// Extended energy (opt-in): bond springs ((|p_i - p_i+1| - t)/t)^2 * k (k the
// stretch constant when longer than t, else the squeeze constant), as
// calcScoreStructureActiveRegionLengths (LooperSolver.hpp:3375-3412), and
// k_angle * a^3 with a = (1 - cos)/2 of the angle between p_i-1 - p_i and
// p_i - p_i+1 at every interior bead, as calcScoreStructureSmooth
// (:3414-3495, angle() thirdparty/common.cpp:39-46), weights 1.
// ---------------------------------------------------------------------------
__device__ __forceinline__ float ext_bond(float4 a, float4 b, const ArcsDevParams &P) {
  const float d = (ref_len(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z)) -
                   P.bond_t) * P.inv_bond_t;
  return d * d * (d >= 0.0f ? P.kb_stretch : P.kb_squeeze);
}

// angle term at the bead between u = a - b and v = b - c (both normalised)
__device__ __forceinline__ float ext_angle(float4 a, float4 b, float4 c, const ArcsDevParams &P) {
  const float ux = a.x - b.x, uy = a.y - b.y, uz = a.z - b.z;
  const float vx = b.x - c.x, vy = b.y - c.y, vz = b.z - c.z;
  float lu = ref_len(ux, uy, uz), lv = ref_len(vx, vy, vz);
  lu = lu > 0.0f ? 1.0f / lu : 0.0f;
  lv = lv > 0.0f ? 1.0f / lv : 0.0f;
  const float dot = (ux * lu) * (vx * lv) + (uy * lu) * (vy * lv) + (uz * lu) * (vz * lv);
  const float an = 1.0f - (dot + 1.0f) * 0.5f;
  return an * an * an * P.k_angle;
}

// The terms bead b changes (bonds b-1|b, b|b+1; angles at b-1, b, b+1) with
// bead b at x.
__device__ float ext_local(const float4 *spos, int n, int b, float4 x, const ArcsDevParams &P) {
  float4 q[5];
#pragma unroll
  for (int k = 0; k < 5; ++k) {
    const int i = b - 2 + k;
    q[k] = k == 2 ? x : (i >= 0 && i < n ? spos[i] : make_float4(0.f, 0.f, 0.f, 0.f));
  }
  float s = 0.0f;
  if (b >= 1) s += ext_bond(q[1], q[2], P);
  if (b + 1 < n) s += ext_bond(q[2], q[3], P);
  if (b >= 2) s += ext_angle(q[0], q[1], q[2], P);
  if (b >= 1 && b + 1 < n) s += ext_angle(q[1], q[2], q[3], P);
  if (b + 2 < n) s += ext_angle(q[2], q[3], q[4], P);
  return s;
}

// Full extended energy in FP64 over the warp.
__device__ double ext_full(int n, const float4 *spos, const ArcsDevParams &P, int lane) {
  double acc = 0.0;
  for (int i = lane; i + 1 < n; i += 32) {
    acc += (double)ext_bond(spos[i], spos[i + 1], P);
    if (i >= 1) acc += (double)ext_angle(spos[i - 1], spos[i], spos[i + 1], P);
  }
  return warp_sum_d(acc);
}

// The same energy for the periodic resync, which only has to remove the
// drift of the running total: each term in FP32 (hardware reciprocal square
// root for the length), summed per lane in float-float (error-free two-sum)
// and across lanes in FP64.  A lane walks four bead rows at once with four
// independent accumulators so that the loads and arithmetic of different rows
// overlap; the per-term work stays off the narrow FP64 pipe.
__device__ __forceinline__ float resync_len(float4 a, float4 b) {
  const float x = a.x - b.x, y = a.y - b.y, z = a.z - b.z;
  const float s = fmaf(x, x, fmaf(y, y, z * z));
  return s * rsqrtf(fmaxf(s, 1e-30f));
}

__device__ double arcs_spring_energy_ff(int n, const float4 *spos, const int *srp,
                                        const int2 *nb, const float *inv, const int4 *loops,
                                        int n_loops, const ArcsDevParams &P, int lane) {
  const float ks = P.k_stretch, kq = P.k_squeeze, R = P.sphere_r;
  float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
  for (int i0 = lane; i0 < n; i0 += 128) {
    float4 pi[4];
    int e[4], e1[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const int i = min(i0 + 32 * r, n - 1);
      const bool ok = i0 + 32 * r < n;
      pi[r] = spos[i];
      e[r] = srp[i];
      e1[r] = ok ? srp[i + 1] : e[r];
      ff_add(hi[r], lo[r], ok ? sphere_penalty(pi[r].x, pi[r].y, pi[r].z, R) : 0.0f);
    }
    // branch-free: the four rows' chains interleave
    for (;;) {
      bool any = false;
#pragma unroll
      for (int r = 0; r < 4; ++r) {
        const bool ok = e[r] < e1[r];
        any |= ok;
        const int ee = ok ? e[r] : 0;
        const int2 ent = nb[ee];
        const float4 q = spos[ent.x];
        const float v = spring_fast(resync_len(pi[r], q), __int_as_float(ent.y), inv[ee], ks, kq);
        ff_add(hi[r], lo[r], (ok && ent.x < i0 + 32 * r) ? v : 0.0f);
        e[r] += ok ? 1 : 0;
      }
      if (!any) break;
    }
  }
  for (int c = lane; c < n_loops; c += 32) {
    const int4 L = loops[c];
    const float d = (L.x == L.y ? 0.0f : resync_len(spos[L.x], spos[L.y])) - __int_as_float(L.w);
    ff_add(hi[0], lo[0], __int_as_float(L.z) * d * d);
  }
  const double t = ((double)hi[0] + (double)lo[0]) + ((double)hi[1] + (double)lo[1]) +
                   ((double)hi[2] + (double)lo[2]) + ((double)hi[3] + (double)lo[3]);
  return warp_sum_d(t);
}

// The same recompute from the region's flat spring list: every lane takes
// every 32nd spring, four at a time with independent accumulators, so no lane
// waits for another's longer arc list.
__device__ double arcs_spring_energy_list(int n, const float4 *spos, const int4 *arcl,
                                          int n_arcs, const int4 *loops, int n_loops,
                                          const ArcsDevParams &P, int lane) {
  const float ks = P.k_stretch, kq = P.k_squeeze, R = P.sphere_r;
  float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
  if (R > 0.0f)
    for (int i = lane; i < n; i += 32) {
      const float4 q = spos[i];
      ff_add(hi[1], lo[1], sphere_penalty(q.x, q.y, q.z, R));
    }
  int c = lane;
  for (; c + 96 < n_arcs; c += 128) {
    int4 a[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) a[r] = arcl[c + 32 * r];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const float v = spring_fast(resync_len(spos[a[r].x], spos[a[r].y]), __int_as_float(a[r].z),
                                  __int_as_float(a[r].w), ks, kq);
      ff_add(hi[r], lo[r], v);
    }
  }
  for (; c < n_arcs; c += 32) {
    const int4 a = arcl[c];
    ff_add(hi[0], lo[0], spring_fast(resync_len(spos[a.x], spos[a.y]), __int_as_float(a.z),
                                     __int_as_float(a.w), ks, kq));
  }
  for (int k = lane; k < n_loops; k += 32) {
    const int4 L = loops[k];
    const float d = (L.x == L.y ? 0.0f : resync_len(spos[L.x], spos[L.y])) - __int_as_float(L.w);
    ff_add(hi[2], lo[2], __int_as_float(L.z) * d * d);
  }
  const double t = ((double)hi[0] + (double)lo[0]) + ((double)hi[1] + (double)lo[1]) +
                   ((double)hi[2] + (double)lo[2]) + ((double)hi[3] + (double)lo[3]);
  return warp_sum_d(t);
}

// FP64 sum of 1/d over every pair (i<j) that the arc lists do not name.
__device__ double arcs_repulsion(int n, const float4 *spos, const int *srp,
                                 const int2 *nb, const int2 *nulls, int n_null,
                                 int lane) {
  double acc = 0.0;
  for (int i = lane; i < n; i += 32) {
    const float4 pi = spos[i];
    float part = 0.0f;
    int cnt = 0;
    for (int j = i + 1; j < n; ++j) {
      const float4 pj = spos[j];
      const float x = pi.x - pj.x, y = pi.y - pj.y, z = pi.z - pj.z;
      part += rsqrtf(fmaf(x, x, fmaf(y, y, z * z)));
      if (++cnt == 64) {
        acc += part;
        part = 0.0f;
        cnt = 0;
      }
    }
    acc += part;
    const int e1 = srp[i + 1];
    for (int e = srp[i]; e < e1; ++e) {
      const int j = nb[e].x;
      if (j < i) acc -= (double)(1.0f / dist3(spos[j].x, spos[j].y, spos[j].z, pi));
    }
  }
  for (int c = lane; c < n_null; c += 32) {
    const int2 q = nulls[c];
    acc -= (double)(1.0f / dist3(spos[q.x].x, spos[q.x].y, spos[q.x].z, spos[q.y]));
  }
  return warp_sum_d(acc);
}

// Bounded wait of one lane on a shared-memory word written by the other warp
// of a chain's pair: returns false when the time limit ran out.
constexpr unsigned long long kPairWaitNs = 2000000000ull;

__device__ __forceinline__ void pair_sync(int slot) {
  asm volatile("bar.sync %0, 64;" ::"r"(1 + slot) : "memory");
}

template <bool NB_SMEM, int G, bool PROD>
__global__ void __launch_bounds__(PROD ? 256 : 128, PROD ? 2 : 4)
arcs_anneal_kernel(const ArcsUnit *__restrict__ units,
                   const int2 *__restrict__ items, int n_items,
                   int *__restrict__ head, const float4 *__restrict__ pos0,
                   const int *__restrict__ row_ptr,
                   const int2 *__restrict__ nbr, const float *__restrict__ inv_t,
                   const int *__restrict__ movable,
                   const int *__restrict__ lrp, const float4 *__restrict__ lent,
                   const int4 *__restrict__ lst, const int2 *__restrict__ nulls,
                   ArcsDevParams P, int smem_per_warp, float *__restrict__ pos_out,
                   ChainOut *__restrict__ outs, int *__restrict__ done,
                   MoveTrace *__restrict__ trace, const double *__restrict__ bases) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31;
  // PROD: warps come in pairs, the even one runs the chain, the odd one
  // draws its moves into the ring ahead of it
  const int wid = threadIdx.x >> 5;
  const int slot_w = PROD ? (wid >> 1) : wid;
  const bool producer = PROD && (wid & 1) != 0;
  float *s_dtpow = reinterpret_cast<float *>(smem);
  for (int i = threadIdx.x; i < 33; i += blockDim.x) s_dtpow[i] = P.dtpow[i];
  __syncthreads();
  unsigned char *wbase = smem + kCtaHeader + (size_t)slot_w * smem_per_warp;
  ArcsRingCtl *ctl = reinterpret_cast<ArcsRingCtl *>(wbase + kRingCtlOffset);
  int4 *s_mv = reinterpret_cast<int4 *>(wbase);  // move m at slot m % kRing
  float *s_thr = reinterpret_cast<float *>(wbase + kRing * 16);
  float *s_d = reinterpret_cast<float *>(wbase + kRing * 20);
  float *s_so = reinterpret_cast<float *>(wbase + kRing * 20 + 32 * 4);
  float *s_sn = reinterpret_cast<float *>(wbase + kRing * 20 + 32 * 8);
  float4 *spos = reinterpret_cast<float4 *>(wbase + kMoveBufBytes);

  for (;;) {
    int item = 0;
    if (PROD) {
      if (!producer && lane == 0) *(volatile int *)&ctl->item = atomicAdd(head, 1);
      pair_sync(slot_w);
      item = *(volatile int *)&ctl->item;
    } else {
      if (lane == 0) item = atomicAdd(head, 1);
      item = __shfl_sync(0xffffffffu, item, 0);
    }
    if (item >= n_items) break;
    const int2 it = items[item];
    const ArcsUnit U = units[it.x];
    const int chain = it.y;
    const int n = U.n;
    const uint32_t chain_id = (uint32_t)(U.rng_chain + chain);
    int *done_flag = done + it.x;

    // ---- stage the region in this warp's shared-memory slice ----
    int *srp = reinterpret_cast<int *>(spos + n);
    // per-bead mask of the current window's slots holding that bead
    unsigned *smask = reinterpret_cast<unsigned *>(srp + n + 1);
    size_t off = (size_t)kMoveBufBytes + (size_t)n * 16 + (size_t)(n + 1) * 4 + (size_t)n * 4;
    off = (off + 7) & ~(size_t)7;
    int2 *snb = reinterpret_cast<int2 *>(wbase + off);
    if (NB_SMEM) off += (size_t)U.nnz * 8;
    const bool has_mov = U.mov_off >= 0;
    const bool mov_smem = has_mov && off + (size_t)U.n_mov * 4 <= (size_t)smem_per_warp;
    int *smov = reinterpret_cast<int *>(wbase + off);

    if (producer) {
      // ---- the drawing warp: moves [next, next + 32) into the ring once
      // the chain has used the moves that held those slots ----
      const int *MOVp = has_mov ? (mov_smem ? smov : movable + U.mov_off) : nullptr;
      pair_sync(slot_w);  // staging done (the movable list may be in shared memory)
      if (P.stall_draws) {
        // nothing is drawn: wait (bounded) for the chain to give up
        if (lane == 0) {
          const unsigned long long t0 = globaltimer_ns();
          while (*(volatile int *)&ctl->state == 0 && globaltimer_ns() - t0 < 2 * kPairWaitNs)
            __nanosleep(1000);
        }
        __syncwarp();
      } else if (U.n_mov > 0) {
        double Tp = P.max_temp;
        const float step = U.step;
        int4 *s_mv = reinterpret_cast<int4 *>(wbase);
        float *s_thr = reinterpret_cast<float *>(wbase + kRing * 16);
        for (long long next = 0;; next += 32) {
          int st = 0;
          if (lane == 0) {
            unsigned long long t0 = 0;
            for (unsigned spins = 0;; ++spins) {
              st = *(volatile int *)&ctl->state;
              if (st != 0) break;
              if (next <= *(volatile long long *)&ctl->consumed + (kRing - 32)) break;
              if ((spins & 63u) == 63u) {
                const unsigned long long t = globaltimer_ns();
                if (t0 == 0) t0 = t;
                else if (t - t0 > kPairWaitNs) {
                  st = 2;
                  *(volatile int *)&ctl->state = 2;
                  break;
                }
              }
              __nanosleep(20);
            }
          }
          st = __shfl_sync(0xffffffffu, st, 0);
          if (st != 0) break;
          __threadfence_block();  // the chain's reads of these slots are done
          const uint64_t m = (uint64_t)next + lane;
          const uint4 r = philox_move(U.seed, chain_id, m, 0u);
          const uint4 a = philox_move(U.seed, chain_id, m, 1u);
          const int k = uniform_index(r.x, U.n_mov);
          const int b = MOVp ? MOVp[k] : k;
          const float dx = (2.0f * u01(r.y) - 1.0f) * step;
          const float dy = (2.0f * u01(r.z) - 1.0f) * step;
          const float dz = P.use2d ? 0.0f : (2.0f * u01(r.w) - 1.0f) * step;
          const float Tl = (float)Tp * s_dtpow[lane];
          const int sl = (int)(m & (uint64_t)(kRing - 1));
          s_mv[sl] = make_int4(b, __float_as_int(dx), __float_as_int(dy), __float_as_int(dz));
          s_thr[sl] = ratio_threshold(u01(a.x), Tl, P.inv_scale, P.inv_coef);
          Tp *= (double)s_dtpow[32];
          __syncwarp();
          __threadfence_block();
          if (lane == 0) *(volatile long long *)&ctl->filled = next + 32;
        }
      }
      pair_sync(slot_w);  // the chain is finished
      continue;
    }

    for (int i = lane; i < n; i += 32) spos[i] = pos0[U.pos_off + i];
    for (int i = lane; i <= n; i += 32) srp[i] = row_ptr[U.rp_off + i];
    for (int i = lane; i < n; i += 32) smask[i] = 0u;
    if (NB_SMEM) {
      for (int e = lane; e < U.nnz; e += 32) snb[e] = nbr[U.nbr_off + e];
    }
    if (mov_smem)
      for (int k = lane; k < U.n_mov; k += 32) smov[k] = movable[U.mov_off + k];
    if (PROD && lane == 0) {
      *(volatile long long *)&ctl->filled = 0;
      *(volatile long long *)&ctl->consumed = 0;
      *(volatile int *)&ctl->state = 0;
    }
    __syncwarp();
    if (PROD) {
      __threadfence_block();
      pair_sync(slot_w);  // staging done: the drawing warp starts
    }
    const int2 *NB = NB_SMEM ? snb : nbr + U.nbr_off;
    // reciprocal targets: the global copy for the recompute without a spring
    // list; the window's terms derive them from the target
    const float *INV = inv_t + U.nbr_off;
    const int *MOV = has_mov ? (mov_smem ? smov : movable + U.mov_off) : nullptr;
    const bool has_loops = U.lrp_off >= 0;
    const int *LRP = has_loops ? lrp + U.lrp_off : nullptr;
    const float4 *LENT = has_loops ? lent + U.lent_off : nullptr;
    const int4 *LST = lst + U.lst_off;

    // ---- initial FP64 energy: repulsion (frozen) + springs/loops/sphere ----
    // (precomputed per region by arcs_base_kernel when the caller has room)
    const double base = bases ? bases[it.x]
                              : arcs_repulsion(n, spos, srp, NB, nulls + U.null_off, U.n_null,
                                               lane);
    double E = base + arcs_spring_energy(n, spos, srp, NB, LST, U.n_loops, P, lane);
    if (P.ext) E += ext_full(n, spos, P, lane);
    // running energy of the chain (identical on every lane): float-float
    // pair on the move path, widened to FP64 at milestones, resyncs, the end
    float e_hi = (float)E, e_lo = (float)(E - (double)(float)E);
    double E_ms = E;
    double T = P.max_temp;
    long long moves = 0, accepted = 0;
    int succ_ms = 0, misses = 0, status = kDevOk;
    bool stop = U.n_mov == 0 || P.cap <= 0;
    if (U.n_mov == 0) status = kDevNoMovable;
    const float step = U.step;
    const float ks = P.k_stretch, kq = P.k_squeeze, R = P.sphere_r;
    const bool tracing = trace != nullptr && chain_id < (uint32_t)P.trace_chains;
    MoveTrace *const ctrace = tracing ? trace + (size_t)chain_id * P.trace_cap : nullptr;

    // ---- windows of W = 32/G proposals, G lanes each ----
    // Every proposal of a window is scored against the positions at the
    // window's start; the proposals are then resolved in order.  A proposal
    // whose bead, or one of whose arc / loop partners, was moved by an earlier
    // accepted proposal of the same window closes the window there: it is
    // re-scored from the updated positions as the first proposal of the next
    // window.  The accepted sequence is therefore the one the one-move-at-a-
    // time algorithm produces.  Which slots hold a bead is a per-bead bit mask
    // in shared memory (set for the window, cleared after it), so a partner
    // check is one load whatever the window size.
    constexpr int W = 32 / G;
    const int g = lane / G;    // proposal slot of this lane
    const int sub = lane % G;  // lane within the slot
    // Draws live in a kRing-move ring, refilled 32 moves at a time, so that
    // a window can always take 32 proposals whatever move it starts at.
    // [lo, lo + kRing) are drawn; T is the temperature of move lo + kRing
    // (the first move of the next refill).  With a drawing warp (PROD) that
    // warp fills the ring and this one only waits for it.
    long long lo = 0;
    auto refill = [&](long long first) {
      const uint64_t m = (uint64_t)first + lane;
      const uint4 r = philox_move(U.seed, chain_id, m, 0u);
      const uint4 a = philox_move(U.seed, chain_id, m, 1u);
      const int k = uniform_index(r.x, U.n_mov);
      const int b = MOV ? MOV[k] : k;
      const float dx = (2.0f * u01(r.y) - 1.0f) * step;
      const float dy = (2.0f * u01(r.z) - 1.0f) * step;
      const float dz = P.use2d ? 0.0f : (2.0f * u01(r.w) - 1.0f) * step;
      const float Tl = (float)T * s_dtpow[lane];
      const int slot = (int)(m & (uint64_t)(kRing - 1));
      s_mv[slot] = make_int4(b, __float_as_int(dx), __float_as_int(dy), __float_as_int(dz));
      s_thr[slot] = ratio_threshold(u01(a.x), Tl, P.inv_scale, P.inv_coef);
      T *= (double)s_dtpow[32];
    };
    long long have = 0;  // PROD: moves the drawing warp has published
    if (!PROD && !stop)
      for (int r = 0; r < kRing; r += 32) refill(r);
    __syncwarp();

    long long next_ms = P.window;
    long long next_rs = P.resync > 0 ? (long long)P.resync : LLONG_MAX;
    while (!stop) {
      const long long lim = min(min(next_ms, next_rs), P.cap);
      const int L = (int)min((long long)W, lim - moves);
      if (PROD) {
        if (moves + L > have) {  // wait for the drawing warp
          long long f = 0;
          int ok = 1;
          if (lane == 0) {
            unsigned long long t0 = 0;
            for (unsigned spins = 0;; ++spins) {
              f = *(volatile long long *)&ctl->filled;
              if (f >= moves + L) break;
              if (*(volatile int *)&ctl->state == 2) {
                ok = 0;
                break;
              }
              if ((spins & 63u) == 63u) {
                const unsigned long long t = globaltimer_ns();
                if (t0 == 0) t0 = t;
                else if (t - t0 > kPairWaitNs) {
                  ok = 0;
                  break;
                }
              }
              __nanosleep(32);
            }
          }
          have = __shfl_sync(0xffffffffu, f, 0);
          if (!__shfl_sync(0xffffffffu, ok, 0)) {
            status = kDevDrawWait;
            break;
          }
          __threadfence_block();  // the slots up to `have` are written
        }
      } else if (moves + L > lo + kRing) {  // the oldest 32 are used: draw the next 32
        __syncwarp();
        refill(lo + kRing);
        lo += 32;
        __syncwarp();
      }
      const bool active = g < L;
      const int slot = (int)((moves + g) & (kRing - 1));
      const int4 mv = active ? s_mv[slot] : make_int4(0, 0, 0, 0);
      const float thr = active ? s_thr[slot] : 0.0f;
      const int b = mv.x;
      if (active && sub == 0) atomicOr(&smask[b], 1u << g);
      __syncwarp();
      float so = 0.0f, sn = 0.0f;
      unsigned cm = 0u;
      float4 pb = make_float4(0.f, 0.f, 0.f, 0.f);
      float nx = 0.f, ny = 0.f, nz = 0.f;
      if (active) {
        pb = spos[b];
        nx = pb.x + __int_as_float(mv.y);
        ny = pb.y + __int_as_float(mv.z);
        nz = pb.z + __int_as_float(mv.w);
        const int beg = srp[b], end = srp[b + 1];
        const unsigned earlier = (1u << g) - 1u;  // slots before this one
        // two arcs per lane per iteration: independent loads and lengths in
        // flight
        constexpr int UA = 2;
        for (int e = beg + sub; e < end; e += UA * G) {
          int2 ent[UA];
          float iv[UA];
#pragma unroll
          for (int k = 0; k < UA; ++k) {
            const int ek = e + k * G;
            const bool ok = ek < end;
            ent[k] = NB[ok ? ek : e];
            // 1/t from the target (8 staged bytes per entry instead of 12)
            iv[k] = recip_nr(__int_as_float(ent[k].y));
          }
#pragma unroll
          for (int k = 0; k < UA; ++k) {
            const bool ok = e + k * G < end;
            const float4 q = spos[ent[k].x];
            const float t = __int_as_float(ent[k].y);
            const float o1 = spring_fast(fast_len(pb.x, pb.y, pb.z, q), t, iv[k], ks, kq);
            const float n1 = spring_fast(fast_len(nx, ny, nz, q), t, iv[k], ks, kq);
            so += ok ? o1 : 0.0f;
            sn += ok ? n1 : 0.0f;
            const unsigned mk = smask[ent[k].x];
            cm |= ok ? (mk & earlier) : 0u;
          }
        }
        if (has_loops) {
          const int l1 = LRP[b + 1];
          for (int e = LRP[b] + sub; e < l1; e += G) {
            const float4 le = LENT[e];
            const int pj = __float_as_int(le.x);
            const float4 q = spos[pj];
            // a constraint of a bead with itself stays at distance 0
            const float d0 = (pj == b ? 0.0f : fast_len(pb.x, pb.y, pb.z, q)) - le.z;
            const float d1 = (pj == b ? 0.0f : fast_len(nx, ny, nz, q)) - le.z;
            so += le.y * d0 * d0;
            sn += le.y * d1 * d1;
            cm |= smask[pj] & ((1u << g) - 1u);
          }
        }
        if (sub == 0) {
          if (R > 0.0f) {
            so += sphere_penalty(pb.x, pb.y, pb.z, R);
            sn += sphere_penalty(nx, ny, nz, R);
          }
          unsigned hit = smask[b];
          if (P.ext) {
            // bonds and angles reach two beads along the chain: a window
            // proposal within that distance is a partner too
            so += ext_local(spos, n, b, pb, P);
            sn += ext_local(spos, n, b, make_float4(nx, ny, nz, 0.0f), P);
            if (b >= 1) hit |= smask[b - 1];
            if (b >= 2) hit |= smask[b - 2];
            if (b + 1 < n) hit |= smask[b + 1];
            if (b + 2 < n) hit |= smask[b + 2];
          }
          cm |= hit & ((1u << g) - 1u);
        }
      }
      float d = sn - so;
#pragma unroll
      for (int o = G >> 1; o > 0; o >>= 1) {
        cm |= __shfl_xor_sync(0xffffffffu, cm, o);
        if (tracing) {
          so += __shfl_xor_sync(0xffffffffu, so, o);
          sn += __shfl_xor_sync(0xffffffffu, sn, o);
        } else {
          d += __shfl_xor_sync(0xffffffffu, d, o);
        }
      }
      if (tracing) {
        d = sn - so;
        if (active && sub == 0) {
          s_so[g] = so;
          s_sn[g] = sn;
          s_d[g] = d;
        }
      }
      // ---- resolution, equivalent to the in-order loop.  A downhill slot
      // is always accepted, an uphill slot's test needs the sum of the
      // accepted changes before it: all downhill slots are taken at once;
      // then, repeatedly, a warp scan gives every slot the sum of the
      // accepted changes before it and the first uphill slot that passes is
      // accepted (every slot before it is then final).  The window ends at
      // the first slot that depends on an accepted earlier slot ----
      const bool leader = active && sub == 0;
      unsigned acc_l = __ballot_sync(0xffffffffu, leader && d <= 0.0f);  // by lane
      float inc;  // inclusive scan of the accepted changes over lanes
      for (int from = 0;;) {
        const float v = ((acc_l >> lane) & 1u) ? d : 0.0f;
        inc = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const float t = __shfl_up_sync(0xffffffffu, inc, o);
          if (lane >= o) inc += t;
        }
        const float pre = __shfl_up_sync(0xffffffffu, inc, 1);
        const float ef = e_hi + (lane == 0 ? 0.0f : pre);
        const bool up = leader && lane >= from && !((acc_l >> lane) & 1u) &&
                        d < ef * (thr - 1.0f);
        const unsigned um = __ballot_sync(0xffffffffu, up);
        if (um == 0u) break;
        const int l1 = __ffs(um) - 1;
        acc_l |= 1u << l1;
        from = l1 + 1;
      }
      unsigned accm =
          __reduce_or_sync(0xffffffffu, (leader && ((acc_l >> lane) & 1u)) ? 1u << g : 0u);
      const unsigned dep =
          __ballot_sync(0xffffffffu, leader && (cm & accm & ((1u << g) - 1u)) != 0u);
      const int lend = dep ? (__ffs(dep) - 1) / G : L;
      accm &= lend >= 32 ? 0xffffffffu : (1u << lend) - 1u;
      const float pacc = __shfl_sync(0xffffffffu, inc, lend * G - 1);
      if (leader && g < lend && ((accm >> g) & 1u)) spos[b] = make_float4(nx, ny, nz, 0.0f);
      if (tracing) {
        __syncwarp();
        if (lane == 0) {
          for (int j = 0; j < lend && moves + j < P.trace_cap; ++j) {
            const int4 m = s_mv[(moves + j) & (kRing - 1)];
            MoveTrace tr;
            tr.bead = m.x;
            tr.accepted = (accm >> j) & 1u;
            tr.before = s_so[j];
            tr.after = s_sn[j];
            tr.dx = __int_as_float(m.y);
            tr.dy = __int_as_float(m.z);
            tr.dz = __int_as_float(m.w);
            tr.pad = s_d[j];
            ctrace[moves + j] = tr;
          }
        }
      }
      __syncwarp();
      if (active && sub == 0) smask[b] = 0u;  // every reader is past the window
      __syncwarp();
      if (accm) ff_add(e_hi, e_lo, pacc);
      const int na = __popc(accm);
      accepted += na;
      succ_ms += na;
      moves += lend;
      if (PROD && lane == 0) {
        __threadfence_block();  // this window's reads of the ring are done
        *(volatile long long *)&ctl->consumed = moves;
      }

      // ---- milestone (the reference predicate, FP64, every lane; the
      // reference kernel guards the ratio test by E_ms > 1e-10) ----
      bool flag = false;
      const bool at_ms = moves == next_ms;
      if (at_ms) {
        next_ms += P.window;
        const double E = (double)e_hi + (double)e_lo;
        const bool miss =
            (E > (double)P.improvement * E_ms && succ_ms < P.min_successes) ||
            E < 1e-5 || ((!P.ms_guard || E_ms > 1e-10) && E / E_ms > 0.9999);
        misses = miss ? misses + 1 : 0;
        if (misses >= P.fails || E < 1e-5) flag = true;
        E_ms = E;
        succ_ms = 0;
      }
      if (moves == next_rs) {
        next_rs += P.resync;
        if (!flag) {
          double es = U.n_arcs >= 0
                          ? arcs_spring_energy_list(n, spos, lst + U.arc_off, U.n_arcs, LST,
                                                    U.n_loops, P, lane)
                          : arcs_spring_energy_ff(n, spos, srp, NB, INV, LST, U.n_loops, P, lane);
          if (P.ext) es += ext_full(n, spos, P, lane);
          const double Er = base + es;
          e_hi = (float)Er;
          e_lo = (float)(Er - (double)e_hi);
        }
      }
      if (!flag && moves >= P.cap) {
        flag = true;
        if (P.cap_is_error) status = kDevMoveCap;
      }
      // the first chain to stop ends its unit's others at their next
      // milestone (the reference's shared d_isDone, read once per 256-move
      // block, ParallelMonteCarloArcs.cu:520,650)
      int f = flag ? 1 : 0;
      if (lane == 0) {
        if (f && P.stop_all) atomicExch(done_flag, 1);
        if (!f && P.stop_all && at_ms && *((volatile int *)done_flag) != 0) f = 1;
      }
      stop = __shfl_sync(0xffffffffu, f, 0) != 0;
    }

    // ---- final FP64 recompute and outputs ----
    double es = arcs_spring_energy(n, spos, srp, NB, LST, U.n_loops, P, lane);
    if (P.ext) es += ext_full(n, spos, P, lane);
    if (lane == 0) {
      ChainOut o;
      o.energy = (double)e_hi + (double)e_lo;
      o.energy_fp64 = base + es;
      o.base = base;
      o.best = o.energy;  // not tracked at the arc level
      o.score = e_hi;
      o.status = status;
      o.moves = moves;
      o.accepted = accepted;
      outs[U.chain_base + chain] = o;
    }
    float *po = pos_out + U.out_off + (long long)chain * n * 3;
    for (int i = lane; i < n; i += 32) {
      const float4 p = spos[i];
      po[3 * i] = p.x;
      po[3 * i + 1] = p.y;
      po[3 * i + 2] = p.z;
    }
    __syncwarp();
    if (PROD) {
      if (lane == 0 && *(volatile int *)&ctl->state == 0) *(volatile int *)&ctl->state = 1;
      pair_sync(slot_w);  // the drawing warp has stopped
    }
  }
}

// Best chain of each unit (lowest running energy, ties to the lower index,
// as the reference's host argmin, ParallelMonteCarloArcs.cu:899-910).
__global__ void arcs_pick_best_kernel(const ArcsUnit *__restrict__ units,
                                      int n_units, const ChainOut *outs,
                                      int *best) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= n_units) return;
  const ArcsUnit U = units[u];
  int b = 0;
  double be = outs[U.chain_base].energy;
  for (int c = 1; c < U.chains; ++c) {
    const double e = outs[U.chain_base + c].energy;
    if (e < be) {
      be = e;
      b = c;
    }
  }
  best[u] = b;
}

using ArcsKernelFn = void (*)(const ArcsUnit *, const int2 *, int, int *, const float4 *,
                              const int *, const int2 *, const float *, const int *,
                              const int *, const float4 *, const int4 *, const int2 *,
                              ArcsDevParams, int, float *, ChainOut *, int *, MoveTrace *,
                              const double *);

// The frozen repulsion sum of every region (the 1/d of every pair the arc
// lists do not name, in the initial score only): one 512-thread block per
// region, rows interleaved over its warps, lanes striding the row, float
// partial sums of 64 terms widened to FP64, a fixed-order block reduction.
// The per-chain warp would otherwise spend O(n^2 / 32) steps on it before its
// first move.
__global__ void __launch_bounds__(512)
arcs_base_kernel(const ArcsUnit *__restrict__ units, int n_units,
                 const float4 *__restrict__ pos0, const int *__restrict__ row_ptr,
                 const int2 *__restrict__ nbr, const int2 *__restrict__ nulls,
                 double *__restrict__ bases) {
  __shared__ double red[16];
  const int u = blockIdx.x;
  if (u >= n_units) return;
  const ArcsUnit U = units[u];
  const float4 *P = pos0 + U.pos_off;
  const int *rp = row_ptr + U.rp_off;
  const int2 *NB = nbr + U.nbr_off;
  const int n = U.n;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  // per-lane float-float accumulation (~48 bits): FP64 arithmetic is a
  // narrow pipe on this part and a double add per row kept it 85 % busy
  float hi = 0.0f, lo = 0.0f;
  for (int i = warp; i < n; i += nw) {
    const float4 pi = P[i];
    float part = 0.0f;
    int cnt = 0;
    for (int j = i + 1 + lane; j < n; j += 32) {
      const float4 pj = P[j];
      const float x = pi.x - pj.x, y = pi.y - pj.y, z = pi.z - pj.z;
      part += rsqrtf(fmaf(x, x, fmaf(y, y, z * z)));
      if (++cnt == 64) {
        ff_add(hi, lo, part);
        part = 0.0f;
        cnt = 0;
      }
    }
    ff_add(hi, lo, part);
    const int e1 = rp[i + 1];
    for (int e = rp[i] + lane; e < e1; e += 32) {
      const int j = NB[e].x;
      if (j < i) ff_add(hi, lo, -(1.0f / dist3(P[j].x, P[j].y, P[j].z, pi)));
    }
  }
  for (int c = threadIdx.x; c < U.n_null; c += blockDim.x) {
    const int2 q = nulls[U.null_off + c];
    ff_add(hi, lo, -(1.0f / dist3(P[q.x].x, P[q.x].y, P[q.x].z, P[q.y])));
  }
  double acc = warp_sum_d((double)hi + (double)lo);
  if (lane == 0) red[warp] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < nw; ++w) t += red[w];
    bases[u] = t;
  }
}

// The instantiation for a launch: arc lists staged or not, G lanes per move,
// a drawing warp per chain or not (lanes 1 and 2 only).
inline ArcsKernelFn arcs_kernel_for(bool nb_smem, int lanes, bool prod = false) {
  if (prod && lanes == 1)
    return nb_smem ? arcs_anneal_kernel<true, 1, true> : arcs_anneal_kernel<false, 1, true>;
  if (prod && lanes == 2)
    return nb_smem ? arcs_anneal_kernel<true, 2, true> : arcs_anneal_kernel<false, 2, true>;
  switch (lanes) {
    case 1: return nb_smem ? arcs_anneal_kernel<true, 1, false> : arcs_anneal_kernel<false, 1, false>;
    case 2: return nb_smem ? arcs_anneal_kernel<true, 2, false> : arcs_anneal_kernel<false, 2, false>;
    case 8: return nb_smem ? arcs_anneal_kernel<true, 8, false> : arcs_anneal_kernel<false, 8, false>;
    case 32:
      return nb_smem ? arcs_anneal_kernel<true, 32, false> : arcs_anneal_kernel<false, 32, false>;
    case 4: return nb_smem ? arcs_anneal_kernel<true, 4, false> : arcs_anneal_kernel<false, 4, false>;
    default: return nb_smem ? arcs_anneal_kernel<true, 2, false> : arcs_anneal_kernel<false, 2, false>;
  }
}

}  // namespace pmmc

// ===========================================================================
// Host side
// ===========================================================================
using namespace pmmc;

struct ArcsClass {
  int item_begin = 0, item_end = 0;
  bool nb_smem = true;
  int smem_per_warp = 0;
  int warps_per_cta = 1;
  int lanes = 2;          // lanes per proposal
  bool prod = false;      // a drawing warp per chain
  int grid = 0;
  cudaStream_t stream = nullptr;
  cudaEvent_t join = nullptr;
};

struct pmmc_arcs_batch {
  pmmc_ctx *ctx = nullptr;
  int n_units = 0;
  std::vector<ArcsUnit> h_units;
  std::vector<int> h_n;
  long long total_pos_out = 0;  // floats over all chains
  int total_chains = 0;
  ArcsDevParams P{};
  DevBuf<ArcsUnit> units;
  DevBuf<int2> items;
  DevBuf<int> heads;
  DevBuf<float4> pos0;
  DevBuf<int> row_ptr;
  DevBuf<int2> nbr;
  DevBuf<float> inv_t;
  DevBuf<int2> nulls;
  DevBuf<int> movable;
  DevBuf<int> lrp;
  DevBuf<float4> lent;
  DevBuf<int4> lst;
  DevBuf<float> pos_out;
  DevBuf<ChainOut> outs;
  DevBuf<int> done;
  DevBuf<int> best;
  DevBuf<double> bases;  // frozen repulsion of each region
  MoveTrace *trace = nullptr;  // tests only (owned)
  std::vector<ArcsClass> classes;
  cudaEvent_t ev_fork = nullptr, ev_start = nullptr, ev_stop = nullptr;
  cudaGraphExec_t graph = nullptr;
  bool use_graph = true;
  bool ran = false;
  int lanes = 32;

  ~pmmc_arcs_batch() {
    for (auto &c : classes) {
      if (c.stream) cudaStreamDestroy(c.stream);
      if (c.join) cudaEventDestroy(c.join);
    }
    if (ev_fork) cudaEventDestroy(ev_fork);
    if (ev_start) cudaEventDestroy(ev_start);
    if (ev_stop) cudaEventDestroy(ev_stop);
    if (graph) cudaGraphExecDestroy(graph);
    if (trace) cudaFree(trace);
  }
};

namespace pmmc {

size_t arcs_unit_smem(int n, int nnz, int n_mov, bool has_mov) {
  size_t s = (size_t)kMoveBufBytes + (size_t)n * 16 + (size_t)(n + 1) * 4 + (size_t)n * 4;
  s = (s + 7) & ~(size_t)7;
  s += (size_t)nnz * 8;
  if (has_mov) s += (size_t)n_mov * 4;
  return s;
}

size_t arcs_unit_smem_min(int n) {
  size_t s = (size_t)kMoveBufBytes + (size_t)n * 16 + (size_t)(n + 1) * 4 + (size_t)n * 4;
  return (s + 7) & ~(size_t)7;
}

pmmc_status arcs_validate(pmmc_ctx *ctx, const pmmc_arcs_problem *pr) {
  if (!pr || pr->n < 1 || !pr->pos || !pr->row_ptr)
    return fail(ctx, PMMC_ERR_INVALID, "arcs problem: n, pos and row_ptr are required");
  if (pr->row_ptr[0] != 0)
    return fail(ctx, PMMC_ERR_INVALID, "arcs problem: row_ptr[0] must be 0");
  for (int i = 0; i < pr->n; ++i)
    if (pr->row_ptr[i + 1] < pr->row_ptr[i])
      return fail(ctx, PMMC_ERR_INVALID, "arcs problem: row_ptr not monotone");
  const int nnz = pr->row_ptr[pr->n];
  if (nnz > 0 && (!pr->col || !pr->target))
    return fail(ctx, PMMC_ERR_INVALID, "arcs problem: col/target missing");
  for (int e = 0; e < nnz; ++e)
    if (pr->col[e] < 0 || pr->col[e] >= pr->n)
      return fail(ctx, PMMC_ERR_INVALID, "arcs problem: column %d out of range", pr->col[e]);
  if (pr->n_loops < 0 || (pr->n_loops > 0 && (!pr->loop_i || !pr->loop_j ||
                                               !pr->loop_k || !pr->loop_r0)))
    return fail(ctx, PMMC_ERR_INVALID, "arcs problem: loop arrays missing");
  return PMMC_OK;
}

ArcsDevParams arcs_make_params(const pmmc_anneal_params *prm, uint64_t seed, bool stop_all) {
  ArcsDevParams P{};
  P.max_temp = prm->max_temp;
  P.inv_scale = prm->jump_scale != 0.0f ? 1.0f / prm->jump_scale : 0.0f;
  P.inv_coef = prm->jump_coef != 0.0f ? 1.0f / prm->jump_coef : 0.0f;
  P.improvement = prm->improvement;
  P.k_stretch = prm->k_stretch;
  P.k_squeeze = prm->k_squeeze;
  P.sphere_r = prm->sphere_radius;
  P.min_successes = prm->min_successes;
  P.use2d = prm->use2d;
  P.resync = prm->resync_every > 0 ? prm->resync_every : 0;
  P.stop_all = stop_all ? 1 : 0;
  P.seed = seed;
  if (prm->schedule == PMMC_SCHEDULE_CPU) {
    P.window = std::max(1, prm->milestone_steps);
    P.fails = 1;
    P.cap = prm->max_moves > 0 ? prm->max_moves : 200ll * P.window;
    P.cap_is_error = 0;
  } else {
    // MonteCarloArcsKernel (ParallelMonteCarloArcs.cu:520-655): blocks of
    // 256 moves while fewer than stop_condition_steps are done, a milestone
    // after each block, stop after milestone_fails consecutive misses (a
    // threshold <= 0 stops at the first milestone, as there)
    P.window = 256;
    P.fails = prm->milestone_fails;
    P.ms_guard = 1;
    long long cap = prm->milestone_steps > 0 ? ((long long)prm->milestone_steps + 255) / 256 * 256
                                             : 0;
    if (prm->max_moves > 0) cap = std::min(cap, (long long)prm->max_moves);
    P.cap = cap;
    P.cap_is_error = 0;
  }
  double d = 1.0;
  for (int l = 0; l <= 32; ++l) {
    P.dtpow[l] = (float)d;
    d *= (double)prm->dt_temp;
  }
  P.ext = prm->arcs_extended ? 1 : 0;
  // the reference clamps a bond target at 1e-5 (LooperSolver.hpp:3404-3405)
  P.bond_t = std::max(prm->bond_target, 1e-5f);
  P.inv_bond_t = 1.0f / P.bond_t;
  P.kb_stretch = prm->k_stretch_bond;
  P.kb_squeeze = prm->k_squeeze_bond;
  P.k_angle = prm->k_angle_ext;
  return P;
}

void ArcsPack::add(const pmmc_arcs_problem &pr, int n_chains, float step, uint64_t seed,
                   int rng_chain) {
  ArcsUnit U{};
  const int n = pr.n;
  U.n = n;
  U.pos_off = (int)pos.size();
  pos.resize(pos.size() + n);
  float4 *P = pos.data() + U.pos_off;
  for (int i = 0; i < n; ++i)
    P[i] = make_float4(pr.pos[3 * i], pr.pos[3 * i + 1], pr.pos[3 * i + 2], 0.0f);
  // loop constraints first (their records open this unit's slice of lst):
  // rebuildActiveLoopMap (LooperSolver.hpp:3318-3337): key (min,max), the
  // last constraint of a key wins, std::map order
  U.lst_off = (int)lst.size();
  U.n_loops = 0;
  U.lrp_off = -1;
  U.lent_off = 0;
  U.n_lent = 0;
  if (pr.n_loops > 0) {
    std::map<std::pair<int, int>, int> lm;
    for (int c = 0; c < pr.n_loops; ++c) {
      int i = pr.loop_i[c], j = pr.loop_j[c];
      if (i < 0 || j < 0 || i >= n || j >= n) continue;
      lm[i < j ? std::make_pair(i, j) : std::make_pair(j, i)] = c;
    }
    U.n_loops = (int)lm.size();
    if (!lm.empty()) {
      std::vector<std::vector<float4>> per(n);
      for (auto &kv : lm) {
        const int c = kv.second, i = kv.first.first, j = kv.first.second;
        lst.push_back(make_int4(i, j, __float_as_int_host(pr.loop_k[c]),
                                __float_as_int_host(pr.loop_r0[c])));
        per[i].push_back(make_float4(__int_as_float_host(j), pr.loop_k[c], pr.loop_r0[c], 0.0f));
        if (j != i)
          per[j].push_back(make_float4(__int_as_float_host(i), pr.loop_k[c], pr.loop_r0[c], 0.0f));
      }
      U.lrp_off = (int)lrp.size();
      U.lent_off = (int)lent.size();
      int acc = 0;
      for (int i = 0; i < n; ++i) {
        lrp.push_back(acc);
        for (auto &e : per[i]) lent.push_back(e);
        acc += (int)per[i].size();
      }
      lrp.push_back(acc);
      U.n_lent = acc;
    }
  }
  // one pass over the arc lists: spring entries (target >= 1e-6) with
  // 1/target, listed pairs with 0 <= target < 1e-6 (inert: they only leave
  // the repulsion sum), and every spring once (entries whose partner
  // precedes the row) in the flat list of the periodic recompute
  U.rp_off = (int)rp.size();
  U.nbr_off = (int)nbr.size();
  U.null_off = (int)nulls.size();
  U.arc_off = (int)lst.size();
  const int n_ent = pr.row_ptr[n];
  rp.resize(rp.size() + n + 1);
  int *R = rp.data() + U.rp_off;
  nbr.resize(nbr.size() + n_ent);
  inv.resize(inv.size() + n_ent);
  lst.resize(lst.size() + n_ent);  // trimmed below
  int2 *NB = nbr.data() + U.nbr_off;
  float *IV = inv.data() + U.nbr_off;
  int4 *LS = lst.data() + U.arc_off;
  int cnt = 0, n_arcs = 0;
  R[0] = 0;
  for (int i = 0; i < n; ++i) {
    for (int e = pr.row_ptr[i]; e < pr.row_ptr[i + 1]; ++e) {
      const int j = pr.col[e];
      const float t = pr.target[e];
      if (j == i) continue;  // the reference never pairs a bead with itself
      if (t >= 1e-6f) {
        const float it = 1.0f / t;
        NB[cnt] = make_int2(j, __float_as_int_host(t));
        IV[cnt] = it;
        ++cnt;
        if (j < i) LS[n_arcs++] = make_int4(j, i, __float_as_int_host(t), __float_as_int_host(it));
      } else if (t >= 0.0f && j < i) {
        nulls.push_back(make_int2(j, i));
      }
    }
    R[i + 1] = cnt;
  }
  nbr.resize(U.nbr_off + cnt);
  inv.resize(U.nbr_off + cnt);
  lst.resize(U.arc_off + n_arcs);
  U.nnz = cnt;
  U.n_null = (int)nulls.size() - U.null_off;
  U.n_arcs = n_arcs;
  // movable beads, listed only when some bead is fixed
  int n_mov = n;
  if (pr.fixed)
    for (int i = 0; i < n; ++i) n_mov -= pr.fixed[i] ? 1 : 0;
  U.n_mov = n_mov;
  if (n_mov < n) {
    U.mov_off = (int)mov.size();
    for (int i = 0; i < n; ++i)
      if (!pr.fixed[i]) mov.push_back(i);
  } else {
    U.mov_off = -1;
  }
  U.chains = n_chains;
  U.chain_base = chains;
  U.out_off = out_floats;
  U.step = step;
  U.rng_chain = rng_chain;
  U.seed = seed;
  chains += n_chains;
  out_floats += (long long)n_chains * n * 3;
  units.push_back(U);
}

void ArcsPack::append(const ArcsPack &o) {
  const int pos0 = (int)pos.size(), rp0 = (int)rp.size(), nbr0 = (int)nbr.size();
  const int null0 = (int)nulls.size(), mov0 = (int)mov.size(), lrp0 = (int)lrp.size();
  const int lent0 = (int)lent.size(), lst0 = (int)lst.size();
  for (ArcsUnit U : o.units) {
    U.pos_off += pos0;
    U.rp_off += rp0;
    U.nbr_off += nbr0;
    U.null_off += null0;
    if (U.mov_off >= 0) U.mov_off += mov0;
    if (U.lrp_off >= 0) U.lrp_off += lrp0;
    U.lent_off += lent0;
    U.lst_off += lst0;
    if (U.n_arcs >= 0) U.arc_off += lst0;
    U.chain_base += chains;
    U.out_off += out_floats;
    units.push_back(U);
  }
  pos.insert(pos.end(), o.pos.begin(), o.pos.end());
  rp.insert(rp.end(), o.rp.begin(), o.rp.end());
  mov.insert(mov.end(), o.mov.begin(), o.mov.end());
  lrp.insert(lrp.end(), o.lrp.begin(), o.lrp.end());
  nbr.insert(nbr.end(), o.nbr.begin(), o.nbr.end());
  nulls.insert(nulls.end(), o.nulls.begin(), o.nulls.end());
  inv.insert(inv.end(), o.inv.begin(), o.inv.end());
  lent.insert(lent.end(), o.lent.begin(), o.lent.end());
  lst.insert(lst.end(), o.lst.begin(), o.lst.end());
  chains += o.chains;
  out_floats += o.out_floats;
}

void ArcsPack::clear() {
  units.clear();
  pos.clear();
  rp.clear();
  mov.clear();
  lrp.clear();
  nbr.clear();
  nulls.clear();
  inv.clear();
  lent.clear();
  lst.clear();
  out_floats = 0;
  chains = 0;
}

void ArcsPack::finish() {
  if (lst.empty()) lst.push_back(make_int4(0, 0, 0, 0));
  if (nulls.empty()) nulls.push_back(make_int2(0, 0));
}

cudaError_t arcs_launch(const ArcsLaunch &a, const ArcsDevParams &P, bool nb_smem, int lanes,
                        int grid, int warps, int smem_per_warp, cudaStream_t s, bool prod) {
  prod = prod && (lanes == 1 || lanes == 2);
  const size_t dyn = kCtaHeader + (size_t)warps * smem_per_warp;
  arcs_kernel_for(nb_smem, lanes, prod)<<<grid, 32 * warps * (prod ? 2 : 1), dyn, s>>>(
      a.units, a.items, a.n_items, a.head, a.pos0, a.row_ptr, a.nbr, a.inv_t, a.movable, a.lrp,
      a.lent, a.lst, a.nulls, P, smem_per_warp, a.pos_out, a.outs, a.done, a.trace, a.bases);
  return cudaGetLastError();
}

cudaError_t arcs_bases(const ArcsUnit *units, int n_units, const float4 *pos0,
                       const int *row_ptr, const int2 *nbr, const int2 *nulls, double *bases,
                       cudaStream_t s) {
  if (n_units <= 0) return cudaSuccess;
  arcs_base_kernel<<<n_units, 512, 0, s>>>(units, n_units, pos0, row_ptr, nbr, nulls, bases);
  return cudaGetLastError();
}

int arcs_ctas_per_sm(bool nb_smem, int lanes, int warps, int smem_per_warp, bool prod) {
  prod = prod && (lanes == 1 || lanes == 2);
  int per_sm = 0;
  const size_t dyn = kCtaHeader + (size_t)warps * smem_per_warp;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, arcs_kernel_for(nb_smem, lanes, prod),
                                                32 * warps * (prod ? 2 : 1), dyn);
  return per_sm < 1 ? 1 : per_sm;
}

void arcs_set_smem_limit(int bytes) {
  for (int lanes : {1, 2, 4, 8, 32})
    for (bool nbs : {true, false})
      for (bool prod : {false, true})
        cudaFuncSetAttribute(arcs_kernel_for(nbs, lanes, prod),
                             cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

}  // namespace pmmc

// ---------------------------------------------------------------------------
// Autotuner: lanes per proposal (G: 1, 2, 4 or 8, i.e. 32, 16, 8 or 4
// proposals scored per window), a drawing warp per chain or not (G 1 and 2),
// and chains per CTA (1, 2 or 4 sharing a CTA's shared memory) for each
// shared-memory class of a batch.  Every candidate
// runs the class's largest items (up to 4 per SM) for kTuneMoves moves with
// milestones and resyncs off, timed with events after one warm-up launch; the
// fastest in moves/s wins.  The trial chains run at the temperature the
// schedule reaches after kTuneCool moves: almost every move of a long chain
// is made cold, where few proposals are accepted and long windows pay, while
// the first moves at the start temperature accept many proposals and favour
// short windows.  Classes holding regions within an eighth of the size of
// the batch's largest are not tuned for throughput: their chains set, or come
// close to, the length of the pass, so they take the configuration with the
// lowest latency per move (one lane per proposal, a drawing warp, one chain
// per CTA).  On the benchmark ensemble (sizes 32-2048) giving that
// configuration to the classes above 1/2, 1/3, 1/4 and all of the largest
// size measured 152, 147, 148 and 143 ms per pass: the throughput trials,
// run with a class alone on the device, choose configurations that lose
// once the classes share it.  Choices are kept per process, keyed by the
// device (SM count, shared memory) and the class's shape (staged or not,
// slice size, mean region size and arc degree, loops, extended energy), and
// mirrored in a JSON file when PMMC_AUTOTUNE_CACHE names one.
// ---------------------------------------------------------------------------
namespace {

constexpr int kTuneMoves = 8192;
constexpr int kTuneCool = 50000;

struct TuneChoice {
  int lanes = 2, warps = 4, prod = 0;
  double moves_per_s = 0.0;
};

std::mutex g_tune_mu;
std::map<std::string, TuneChoice> g_tune;
std::string g_tune_loaded;  // the cache file read into g_tune

void tune_load(const std::string &path) {
  if (path.empty() || path == g_tune_loaded) return;
  g_tune_loaded = path;
  FILE *f = fopen(path.c_str(), "r");
  if (!f) return;
  char line[512];
  while (fgets(line, sizeof(line), f)) {
    char key[256];
    TuneChoice c;
    if (sscanf(line,
               " \"%255[^\"]\": {\"lanes\": %d, \"warps\": %d, \"prod\": %d, "
               "\"moves_per_s\": %lf",
               key, &c.lanes, &c.warps, &c.prod, &c.moves_per_s) == 5)
      g_tune[key] = c;
  }
  fclose(f);
}

void tune_save(const std::string &path) {
  if (path.empty()) return;
  const std::string tmp = path + ".tmp";
  FILE *f = fopen(tmp.c_str(), "w");
  if (!f) return;
  fprintf(f, "{\n  \"pmmc_autotune\": 1,\n  \"entries\": {\n");
  size_t k = 0;
  for (auto &kv : g_tune)
    fprintf(f,
            "    \"%s\": {\"lanes\": %d, \"warps\": %d, \"prod\": %d, \"moves_per_s\": %.6e}%s\n",
            kv.first.c_str(), kv.second.lanes, kv.second.warps, kv.second.prod,
            kv.second.moves_per_s, ++k < g_tune.size() ? "," : "");
  fprintf(f, "  }\n}\n");
  fclose(f);
  rename(tmp.c_str(), path.c_str());
}

std::string class_key(const pmmc_arcs_batch *b, const ArcsClass &c, const std::vector<int2> &items) {
  double n = 0.0, deg = 0.0;
  int loops = 0;
  for (int k = c.item_begin; k < c.item_end; ++k) {
    const ArcsUnit &U = b->h_units[items[k].x];
    n += U.n;
    deg += (double)U.nnz / std::max(1, U.n);
    loops |= U.n_loops > 0;
  }
  const int cnt = std::max(1, c.item_end - c.item_begin);
  n /= cnt;
  deg /= cnt;
  char buf[256];
  snprintf(buf, sizeof(buf), "sm%d_smem%zu_nb%d_slice%d_n%d_deg%d_loops%d_ext%d_cold",
           b->ctx->sm_count,
           b->ctx->smem_optin, c.nb_smem ? 1 : 0,
           (int)std::ceil(std::log2(std::max(16, c.smem_per_warp))),
           (int)std::lround(2.0 * std::log2(std::max(1.0, n))), (int)std::lround(2.0 * deg),
           loops, b->P.ext);
  return buf;
}

}  // namespace

static cudaError_t autotune_classes(pmmc_arcs_batch *b, cudaStream_t s) {
  pmmc_ctx *ctx = b->ctx;
  const char *env = getenv("PMMC_AUTOTUNE_CACHE");
  const std::string path = env ? env : "";
  std::vector<int2> items(b->items.n);
  cudaError_t e = cudaMemcpy(items.data(), b->items.p, sizeof(int2) * items.size(),
                             cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return e;
  std::lock_guard<std::mutex> lock(g_tune_mu);
  const bool fresh_path = !path.empty() && path != g_tune_loaded;
  tune_load(path);
  const size_t cap_smem = ctx->smem_optin - kCtaHeader;
  ArcsDevParams T = b->P;
  T.max_temp = (float)((double)b->P.max_temp * std::pow((double)b->P.dtpow[1], (double)kTuneCool));
  T.cap = kTuneMoves;
  T.window = 1 << 30;
  T.resync = 0;
  T.stop_all = 0;
  T.trace_cap = 0;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  bool changed = false;
  // the regions whose chains set the pass's length: within an eighth of the
  // size of the batch's largest (move counts grow with the region)
  int n_max = 0;
  for (const ArcsUnit &U : b->h_units) n_max = std::max(n_max, U.n);
  for (size_t k = 0; k < b->classes.size() && e == cudaSuccess; ++k) {
    ArcsClass &c = b->classes[k];
    int c_max = 0;
    for (int q = c.item_begin; q < c.item_end; ++q)
      c_max = std::max(c_max, b->h_units[items[q].x].n);
    TuneChoice best;
    const bool critical = 8 * c_max >= n_max;
    const std::string key = class_key(b, c, items) + (critical ? "_critical" : "");
    auto it = g_tune.find(key);
    if (critical) {
      // the lowest latency per move, not the highest throughput: one lane
      // per proposal, a drawing warp, a chain per CTA
      best.lanes = 1;
      best.warps = 1;
      best.prod = 1;
      best.moves_per_s = 0.0;
      if (it == g_tune.end()) {
        g_tune[key] = best;
        changed = true;
      }
    } else if (it != g_tune.end()) {
      best = it->second;
    } else {
      const int m = std::min(c.item_end - c.item_begin, 4 * ctx->sm_count);
      best.moves_per_s = -1.0;
      for (int cand = 0; cand < 6; ++cand) {  // lanes 1, 2 with and without drawing warp; 4, 8
        const int lanes = cand < 2 ? 1 : cand < 4 ? 2 : cand == 4 ? 4 : 8;
        const bool prod = cand < 4 && (cand & 1);
        for (int w : {4, 2, 1}) {
          if ((size_t)w * c.smem_per_warp > cap_smem) continue;
          const int per_sm = arcs_ctas_per_sm(c.nb_smem, lanes, w, c.smem_per_warp, prod);
          const int grid = std::max(1, std::min(per_sm * ctx->sm_count, (m + w - 1) / w));
          ArcsLaunch a{b->units.p, b->items.p + c.item_begin, m, b->heads.p + k, b->pos0.p,
                       b->row_ptr.p, b->nbr.p, b->inv_t.p, b->movable.p, b->lrp.p, b->lent.p,
                       b->lst.p, b->nulls.p, b->pos_out.p, b->outs.p, b->done.p, nullptr,
                       b->bases.p};
          float ms = 0.0f;
          for (int rep = 0; rep < 2 && e == cudaSuccess; ++rep) {
            e = cudaMemsetAsync(b->heads.p + k, 0, sizeof(int), s);
            if (e == cudaSuccess && rep == 1) e = cudaEventRecord(e0, s);
            if (e == cudaSuccess)
              e = arcs_launch(a, T, c.nb_smem, lanes, grid, w, c.smem_per_warp, s, prod);
            if (e == cudaSuccess && rep == 1) e = cudaEventRecord(e1, s);
          }
          if (e == cudaSuccess) e = cudaEventSynchronize(e1);
          if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
          if (e != cudaSuccess) break;
          const double rate = (double)m * kTuneMoves / std::max(1e-6, (double)ms * 1e-3);
          if (rate > best.moves_per_s) {
            best.lanes = lanes;
            best.warps = w;
            best.prod = prod ? 1 : 0;
            best.moves_per_s = rate;
          }
        }
        if (e != cudaSuccess) break;
      }
      if (e == cudaSuccess) {
        g_tune[key] = best;
        changed = true;
      }
    }
    if (e != cudaSuccess) break;
    c.lanes = best.lanes;
    c.warps_per_cta = best.warps;
    c.prod = best.prod != 0;
    const int per_sm =
        arcs_ctas_per_sm(c.nb_smem, c.lanes, c.warps_per_cta, c.smem_per_warp, c.prod);
    const int items_n = c.item_end - c.item_begin;
    c.grid = std::max(1, std::min(per_sm * ctx->sm_count,
                                  (items_n + c.warps_per_cta - 1) / c.warps_per_cta));
  }
  if (changed || fresh_path) tune_save(path);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return e;
}

extern "C" pmmc_status pmmc_arcs_batch_create_ex(
    pmmc_ctx *ctx, int n_units, const pmmc_arcs_problem *units,
    const pmmc_anneal_params *prm, const float *steps,
    const pmmc_batch_opts *opts, int stop_all, int trace_cap,
    pmmc_arcs_batch **out) {
  if (!ctx || !out || n_units < 1 || !units || !prm || !steps)
    return fail(ctx, PMMC_ERR_INVALID, "arcs batch: bad arguments");
  *out = nullptr;
  const int chains = opts && opts->chains_per_unit > 0 ? opts->chains_per_unit : 1;
  // validation and packing of many regions run on the context's host
  // worker threads
  const int n_threads = n_units >= 64
      ? (int)std::max(1u, std::min(std::thread::hardware_concurrency(), 16u)) : 1;
  if (n_threads > 1)
    std::call_once(ctx->host_pool_once, [ctx, n_threads] {
      ctx->host_pool = std::make_unique<pmmc::HostPool>(n_threads);
    });
  auto parallel = [&](auto &&fn) {  // fn(first, last) over unit ranges
    if (n_threads == 1) {
      fn(0, n_units);
      return;
    }
    const int per = (n_units + n_threads - 1) / n_threads;
    ctx->host_pool->run(n_threads, [&fn, per, n_units](int t) {
      const int a = t * per, z = std::min(n_units, a + per);
      if (a < z) fn(a, z);
    });
  };
  {
    std::vector<int> bad(n_threads > 1 ? n_units : 0, 0);
    int first_bad = -1;
    if (n_threads == 1) {
      for (int u = 0; u < n_units; ++u)
        if (arcs_validate(nullptr, &units[u]) != PMMC_OK) {
          first_bad = u;
          break;
        }
    } else {
      parallel([&](int a, int z) {
        for (int u = a; u < z; ++u) bad[u] = arcs_validate(nullptr, &units[u]) != PMMC_OK;
      });
      for (int u = 0; u < n_units && first_bad < 0; ++u)
        if (bad[u]) first_bad = u;
    }
    if (first_bad >= 0) return arcs_validate(ctx, &units[first_bad]);  // records the message
  }
  auto *b = new pmmc_arcs_batch();
  b->ctx = ctx;
  b->n_units = n_units;
  b->use_graph = !opts || opts->use_graph != 0;
  b->P = arcs_make_params(prm, next_key(ctx), stop_all != 0);
  b->P.trace_cap = trace_cap;
  // tests only: the wait of a chain on its drawing warp runs out (no fault,
  // no hang: both sides give up after their 2 s limit)
  b->P.stall_draws = getenv("PMMC_TEST_STALL_DRAWS") != nullptr ? 1 : 0;

  // ---- pack host arrays (unit u's chains have global ids u*chains...) ----
  // Each host thread packs a contiguous range of units into its own part;
  // the parts are not concatenated on the host (a serial copy of every
  // array): each is uploaded to its offset in the device arrays, and only
  // the unit records are rebased.
  const int per = (n_units + n_threads - 1) / n_threads;
  // The parts live in the context and are reused: their memory is already
  // paged in, where fresh arrays of this size spend most of their packing
  // time in first-touch page faults.  One batch creation packs at a time per
  // context.
  struct PackCache {
    std::mutex mu;
    std::vector<ArcsPack> parts;
  };
  std::call_once(ctx->arcs_host_cache_once,
                 [ctx] { ctx->arcs_host_cache = std::make_shared<PackCache>(); });
  PackCache &cache = *static_cast<PackCache *>(ctx->arcs_host_cache.get());
  std::lock_guard<std::mutex> pack_lock(cache.mu);
  std::vector<ArcsPack> &parts = cache.parts;
  parts.resize((n_units + per - 1) / per);
  for (ArcsPack &q : parts) q.clear();
  parallel([&](int a, int z) {
    ArcsPack &q = parts[a / per];
    size_t beads = 0, entries = 0;
    for (int u = a; u < z; ++u) {
      beads += (size_t)units[u].n;
      entries += (size_t)units[u].row_ptr[units[u].n];
    }
    q.units.reserve(z - a);
    q.pos.reserve(beads);
    q.rp.reserve(beads + (size_t)(z - a));
    q.nbr.reserve(entries);
    q.inv.reserve(entries);
    q.lst.reserve(entries / 2 + 1);
    for (int u = a; u < z; ++u) q.add(units[u], chains, steps[u], b->P.seed, u * chains);
  });
  struct PartOff {
    size_t pos, rp, nbr, nulls, mov, lrp, lent, lst;
  };
  std::vector<PartOff> po(parts.size() + 1, PartOff{0, 0, 0, 0, 0, 0, 0, 0});
  long long out_off = 0;
  int chain_base = 0;
  b->h_units.clear();
  b->h_units.reserve(n_units);
  for (size_t k = 0; k < parts.size(); ++k) {
    const ArcsPack &q = parts[k];
    const PartOff &o = po[k];
    for (ArcsUnit U : q.units) {
      U.pos_off += (int)o.pos;
      U.rp_off += (int)o.rp;
      U.nbr_off += (int)o.nbr;
      U.null_off += (int)o.nulls;
      if (U.mov_off >= 0) U.mov_off += (int)o.mov;
      if (U.lrp_off >= 0) U.lrp_off += (int)o.lrp;
      U.lent_off += (int)o.lent;
      U.lst_off += (int)o.lst;
      if (U.n_arcs >= 0) U.arc_off += (int)o.lst;
      U.chain_base += chain_base;
      U.out_off += out_off;
      b->h_units.push_back(U);
    }
    po[k + 1] = PartOff{o.pos + q.pos.size(),     o.rp + q.rp.size(),   o.nbr + q.nbr.size(),
                        o.nulls + q.nulls.size(), o.mov + q.mov.size(), o.lrp + q.lrp.size(),
                        o.lent + q.lent.size(),   o.lst + q.lst.size()};
    out_off += q.out_floats;
    chain_base += q.chains;
  }
  b->h_n.resize(n_units);
  for (int u = 0; u < n_units; ++u) b->h_n[u] = units[u].n;
  b->total_pos_out = out_off;
  b->total_chains = chain_base;

  // ---- shared-memory classes: items sorted by need, largest first ----
  // A unit whose arc lists fit next to its positions is staged whole
  // (NB_SMEM); otherwise only positions go to shared memory.
  const size_t cap_smem = ctx->smem_optin - kCtaHeader;
  struct Need { int unit; size_t bytes; bool nb_smem; };
  std::vector<Need> needs(n_units);
  for (int u = 0; u < n_units; ++u) {
    const ArcsUnit &U = b->h_units[u];
    const size_t full = arcs_unit_smem(U.n, U.nnz, U.n_mov, U.mov_off >= 0);
    const size_t minimal = arcs_unit_smem_min(U.n);
    if (minimal > cap_smem) {
      delete b;
      return fail(ctx, PMMC_ERR_INVALID,
                  "arcs batch: region of %d beads exceeds the %zu B shared-memory "
                  "slice a chain can hold", U.n, cap_smem);
    }
    needs[u] = full <= cap_smem ? Need{u, full, true} : Need{u, minimal, false};
  }
  std::stable_sort(needs.begin(), needs.end(), [](const Need &a, const Need &c) {
    if (a.nb_smem != c.nb_smem) return !a.nb_smem;
    return a.bytes > c.bytes;
  });
  std::vector<int2> h_items;
  const bool tune = opts && opts->lanes_per_chain == PMMC_LANES_AUTO;
  int lanes = opts && opts->lanes_per_chain > 0 ? opts->lanes_per_chain : 2;
  if (lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8 && lanes != 32) lanes = 2;
  b->lanes = lanes;
  const bool prod_fixed = opts && opts->drawing_warp != 0 && (lanes == 1 || lanes == 2);
  arcs_set_smem_limit((int)ctx->smem_optin);
  size_t i0 = 0;
  while (i0 < needs.size()) {
    const size_t top = needs[i0].bytes;
    const bool nbs = needs[i0].nb_smem;
    size_t i1 = i0;
    while (i1 < needs.size() && needs[i1].nb_smem == nbs && needs[i1].bytes * 2 > top) ++i1;
    ArcsClass c;
    c.nb_smem = nbs;
    c.item_begin = (int)h_items.size();
    for (size_t k = i0; k < i1; ++k)
      for (int ch = 0; ch < chains; ++ch) h_items.push_back(make_int2(needs[k].unit, ch));
    c.item_end = (int)h_items.size();
    c.smem_per_warp = (int)((top + 15) & ~(size_t)15);
    // warps per CTA: keep a CTA's footprint within the opt-in limit
    int w = 4;
    while (w > 1 && (size_t)w * c.smem_per_warp > cap_smem) w >>= 1;
    c.warps_per_cta = w;
    c.lanes = lanes;
    c.prod = prod_fixed;
    const int per_sm = arcs_ctas_per_sm(nbs, lanes, w, c.smem_per_warp, c.prod);
    const int items_n = c.item_end - c.item_begin;
    c.grid = std::max(1, std::min(per_sm * ctx->sm_count, (items_n + w - 1) / w));
    b->classes.push_back(c);
    i0 = i1;
  }

  // ---- upload ----
  cudaStream_t s = ctx->stream;
  cudaError_t e = cudaSuccess;
  // every device array at its total size (at least one entry), each part's
  // slice copied to its offset
  const PartOff &tot = po.back();
#define UP(buf, field, member)                                                  \
  if (e == cudaSuccess) e = b->buf.alloc(std::max<size_t>(1, tot.field));      \
  for (size_t k = 0; k < parts.size() && e == cudaSuccess; ++k)                \
    if (!parts[k].member.empty())                                              \
      e = cudaMemcpyAsync(b->buf.p + po[k].field, parts[k].member.data(),      \
                          parts[k].member.size() * sizeof(parts[k].member[0]), \
                          cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = b->units.upload(b->h_units, s);
  if (e == cudaSuccess) e = b->items.upload(h_items, s);
  UP(pos0, pos, pos);
  UP(row_ptr, rp, rp);
  UP(nbr, nbr, nbr);
  UP(inv_t, nbr, inv);
  UP(nulls, nulls, nulls);
  UP(movable, mov, mov);
  UP(lrp, lrp, lrp);
  UP(lent, lent, lent);
  UP(lst, lst, lst);
#undef UP
  if (e == cudaSuccess) e = b->heads.alloc(b->classes.size());
  if (e == cudaSuccess) e = b->pos_out.alloc((size_t)out_off);
  if (e == cudaSuccess) e = b->outs.alloc((size_t)chain_base);
  if (e == cudaSuccess) e = b->done.alloc((size_t)n_units);
  if (e == cudaSuccess) e = b->best.alloc((size_t)n_units);
  if (e == cudaSuccess) e = b->bases.alloc((size_t)n_units);
  if (e == cudaSuccess) e = arcs_bases(b->units.p, n_units, b->pos0.p, b->row_ptr.p, b->nbr.p,
                                       b->nulls.p, b->bases.p, s);
  // tests: the first trace_cap moves of every chain of region 0
  b->P.trace_chains = trace_cap > 0 ? b->h_units[0].chains : 0;
  if (e == cudaSuccess && trace_cap > 0)
    e = cudaMalloc(&b->trace, sizeof(MoveTrace) * (size_t)trace_cap * b->P.trace_chains);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev_fork);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev_start);
  if (e == cudaSuccess) e = cudaEventCreate(&b->ev_stop);
  for (auto &c : b->classes) {
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c.join, cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && tune) e = autotune_classes(b, s);
  if (e != cudaSuccess) {
    delete b;
    return fail(ctx, e == cudaErrorMemoryAllocation ? PMMC_ERR_NOMEM : PMMC_ERR_CUDA,
                "arcs batch upload: %s", cudaGetErrorString(e));
  }
  if (!b->classes.empty()) b->lanes = b->classes[0].lanes;
  *out = b;
  return PMMC_OK;
}

namespace {

cudaError_t enqueue_pass(pmmc_arcs_batch *b, cudaStream_t s) {
  cudaError_t e = cudaMemsetAsync(b->heads.p, 0, sizeof(int) * b->classes.size(), s);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->done.p, 0, sizeof(int) * b->n_units, s);
  if (e != cudaSuccess) return e;
  e = cudaEventRecord(b->ev_fork, s);
  for (size_t k = 0; k < b->classes.size() && e == cudaSuccess; ++k) {
    ArcsClass &c = b->classes[k];
    e = cudaStreamWaitEvent(c.stream, b->ev_fork, 0);
    if (e != cudaSuccess) break;
    ArcsLaunch a{b->units.p, b->items.p + c.item_begin, c.item_end - c.item_begin,
                 b->heads.p + k, b->pos0.p, b->row_ptr.p, b->nbr.p, b->inv_t.p, b->movable.p,
                 b->lrp.p, b->lent.p, b->lst.p, b->nulls.p, b->pos_out.p, b->outs.p,
                 b->done.p, b->trace, b->bases.p};
    e = arcs_launch(a, b->P, c.nb_smem, c.lanes, c.grid, c.warps_per_cta, c.smem_per_warp,
                    c.stream, c.prod);
    if (e == cudaSuccess) e = cudaEventRecord(c.join, c.stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(s, c.join, 0);
  }
  if (e == cudaSuccess && b->classes.size() > 0 &&
      b->h_units.size() > 0) {
    int need_best = 0;
    for (auto &U : b->h_units) need_best |= U.chains > 1;
    if (need_best) {
      arcs_pick_best_kernel<<<(b->n_units + 127) / 128, 128, 0, s>>>(
          b->units.p, b->n_units, b->outs.p, b->best.p);
      e = cudaGetLastError();
    }
  }
  return e;
}

}  // namespace

extern "C" pmmc_status pmmc_arcs_batch_create(pmmc_ctx *ctx, int n_units,
                                              const pmmc_arcs_problem *units,
                                              const pmmc_anneal_params *prm,
                                              const float *step_sizes,
                                              const pmmc_batch_opts *opts,
                                              pmmc_arcs_batch **out) {
  return pmmc_arcs_batch_create_ex(ctx, n_units, units, prm, step_sizes, opts, 0, 0, out);
}

extern "C" pmmc_status pmmc_arcs_batch_run(pmmc_arcs_batch *b, void *stream) {
  if (!b) return PMMC_ERR_INVALID;
  pmmc_ctx *ctx = b->ctx;
  cudaStream_t s = stream ? (cudaStream_t)stream : ctx->stream;
  PMMC_CUDA(ctx, cudaEventRecord(b->ev_start, s));
  if (b->use_graph) {
    if (!b->graph) {
      cudaStream_t cap;
      PMMC_CUDA(ctx, cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
      cudaGraph_t g = nullptr;
      cudaError_t e = cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal);
      if (e == cudaSuccess) {
        cudaError_t e2 = enqueue_pass(b, cap);
        e = cudaStreamEndCapture(cap, &g);
        if (e2 != cudaSuccess) e = e2;
      }
      if (e == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
      if (g) cudaGraphDestroy(g);
      cudaStreamDestroy(cap);
      if (e != cudaSuccess)
        return fail(ctx, PMMC_ERR_CUDA, "arcs batch graph capture: %s", cudaGetErrorString(e));
    }
    PMMC_CUDA(ctx, cudaGraphLaunch(b->graph, s));
  } else {
    PMMC_CUDA(ctx, enqueue_pass(b, s));
  }
  PMMC_CUDA(ctx, cudaEventRecord(b->ev_stop, s));
  b->ran = true;
  return PMMC_OK;
}

extern "C" pmmc_status pmmc_arcs_batch_results(pmmc_arcs_batch *b, float *pos_out,
                                               pmmc_result *res) {
  if (!b || !b->ran) return PMMC_ERR_INVALID;
  pmmc_ctx *ctx = b->ctx;
  PMMC_CUDA(ctx, cudaEventSynchronize(b->ev_stop));
  std::vector<ChainOut> outs(b->total_chains);
  PMMC_CUDA(ctx, cudaMemcpy(outs.data(), b->outs.p, sizeof(ChainOut) * outs.size(),
                            cudaMemcpyDeviceToHost));
  std::vector<int> best(b->n_units, 0);
  bool multi = false;
  for (auto &U : b->h_units) multi |= U.chains > 1;
  if (multi)
    PMMC_CUDA(ctx, cudaMemcpy(best.data(), b->best.p, sizeof(int) * b->n_units,
                              cudaMemcpyDeviceToHost));
  // positions: one copy; with one chain per unit the device layout is the
  // caller's, otherwise the best chain of each unit is gathered on the host
  std::vector<float> all;
  if (pos_out) {
    if (!multi) {
      PMMC_CUDA(ctx, cudaMemcpy(pos_out, b->pos_out.p, sizeof(float) * b->total_pos_out,
                                cudaMemcpyDeviceToHost));
    } else {
      all.resize((size_t)b->total_pos_out);
      PMMC_CUDA(ctx, cudaMemcpy(all.data(), b->pos_out.p, sizeof(float) * all.size(),
                                cudaMemcpyDeviceToHost));
    }
  }
  long long dst = 0;
  for (int u = 0; u < b->n_units; ++u) {
    const ArcsUnit &U = b->h_units[u];
    const int c = best[u];
    if (pos_out && multi)
      memcpy(pos_out + dst, all.data() + U.out_off + (long long)c * U.n * 3,
             sizeof(float) * U.n * 3);
    dst += (long long)U.n * 3;
    if (res) {
      const ChainOut &o = outs[U.chain_base + c];
      pmmc_result r{};
      r.score = o.score;
      r.energy = o.energy;
      r.energy_fp64 = o.energy_fp64;
      r.rel_error = std::fabs(o.energy - o.energy_fp64) /
                    std::max(std::fabs(o.energy_fp64), 1e-30);
      r.moves = o.moves;
      r.accepted = o.accepted;
      long long tot = 0;
      for (int k = 0; k < U.chains; ++k) tot += outs[U.chain_base + k].moves;
      r.total_moves = tot;
      r.best_chain = c;
      r.status = o.status;
      res[u] = r;
    }
  }
  return PMMC_OK;
}

extern "C" pmmc_status pmmc_arcs_batch_stats(pmmc_arcs_batch *b, double *kernel_ms,
                                             int64_t *total_moves,
                                             int *launches_per_run) {
  if (!b || !b->ran) return PMMC_ERR_INVALID;
  pmmc_ctx *ctx = b->ctx;
  PMMC_CUDA(ctx, cudaEventSynchronize(b->ev_stop));
  if (kernel_ms) {
    float ms = 0.0f;
    PMMC_CUDA(ctx, cudaEventElapsedTime(&ms, b->ev_start, b->ev_stop));
    *kernel_ms = ms;
  }
  if (total_moves) {
    std::vector<ChainOut> outs(b->total_chains);
    PMMC_CUDA(ctx, cudaMemcpy(outs.data(), b->outs.p, sizeof(ChainOut) * outs.size(),
                              cudaMemcpyDeviceToHost));
    long long t = 0;
    for (auto &o : outs) t += o.moves;
    *total_moves = t;
  }
  if (launches_per_run) {
    int multi = 0;
    for (auto &U : b->h_units) multi |= U.chains > 1;
    *launches_per_run = (int)b->classes.size() + multi;
  }
  return PMMC_OK;
}

extern "C" pmmc_status pmmc_arcs_batch_classes(pmmc_arcs_batch *b, int cap, int *n_classes,
                                               int *lanes, int *warps, int *items,
                                               int *nb_smem, int *drawing_warp) {
  if (!b || !n_classes) return PMMC_ERR_INVALID;
  *n_classes = (int)b->classes.size();
  for (int k = 0; k < (int)b->classes.size() && k < cap; ++k) {
    const ArcsClass &c = b->classes[k];
    if (lanes) lanes[k] = c.lanes;
    if (warps) warps[k] = c.warps_per_cta;
    if (items) items[k] = c.item_end - c.item_begin;
    if (nb_smem) nb_smem[k] = c.nb_smem ? 1 : 0;
    if (drawing_warp) drawing_warp[k] = c.prod ? 1 : 0;
  }
  return PMMC_OK;
}

// Tests only: copy the per-move trace of chain `chain` of region 0.
extern "C" pmmc_status pmmc_arcs_batch_trace_chain(pmmc_arcs_batch *b, int chain, void *out,
                                                   int count) {
  if (!b || !b->trace || !out || count < 0 || count > b->P.trace_cap || chain < 0 ||
      chain >= b->P.trace_chains)
    return PMMC_ERR_INVALID;
  pmmc_ctx *ctx = b->ctx;
  PMMC_CUDA(ctx, cudaEventSynchronize(b->ev_stop));
  PMMC_CUDA(ctx, cudaMemcpy(out, b->trace + (size_t)chain * b->P.trace_cap,
                            sizeof(MoveTrace) * (size_t)count, cudaMemcpyDeviceToHost));
  return PMMC_OK;
}

extern "C" pmmc_status pmmc_arcs_batch_trace(pmmc_arcs_batch *b, void *out, int count) {
  return pmmc_arcs_batch_trace_chain(b, 0, out, count);
}

// Every chain of one region (positions aside), in chain order.
extern "C" pmmc_status pmmc_arcs_batch_chain_results(pmmc_arcs_batch *b, int unit, int cap,
                                                     pmmc_result *res, int *n_chains) {
  if (!b || !b->ran || unit < 0 || unit >= b->n_units || (cap > 0 && !res))
    return PMMC_ERR_INVALID;
  pmmc_ctx *ctx = b->ctx;
  const ArcsUnit &U = b->h_units[unit];
  if (n_chains) *n_chains = U.chains;
  PMMC_CUDA(ctx, cudaEventSynchronize(b->ev_stop));
  std::vector<ChainOut> outs((size_t)U.chains);
  PMMC_CUDA(ctx, cudaMemcpy(outs.data(), b->outs.p + U.chain_base,
                            sizeof(ChainOut) * outs.size(), cudaMemcpyDeviceToHost));
  long long tot = 0;
  for (const ChainOut &o : outs) tot += o.moves;
  for (int c = 0; c < U.chains && c < cap; ++c) {
    const ChainOut &o = outs[c];
    pmmc_result r{};
    r.score = o.score;
    r.energy = o.energy;
    r.energy_fp64 = o.energy_fp64;
    r.rel_error = std::fabs(o.energy - o.energy_fp64) / std::max(std::fabs(o.energy_fp64), 1e-30);
    r.moves = o.moves;
    r.accepted = o.accepted;
    r.total_moves = tot;
    r.best_chain = c;
    r.status = o.status;
    res[c] = r;
  }
  return PMMC_OK;
}

extern "C" void pmmc_arcs_batch_destroy(pmmc_arcs_batch *b) { delete b; }

extern "C" pmmc_status pmmc_arcs_batch_anneal(pmmc_ctx *ctx, int n_units,
                                              const pmmc_arcs_problem *units,
                                              const pmmc_anneal_params *prm,
                                              const float *step_sizes,
                                              const pmmc_batch_opts *opts,
                                              float *pos_out, pmmc_result *res) {
  pmmc_arcs_batch *b = nullptr;
  pmmc_batch_opts o = opts ? *opts : pmmc_batch_opts{1, 0, 0, 0};
  o.use_graph = 0;  // one pass: nothing to replay
  pmmc_status s = pmmc_arcs_batch_create(ctx, n_units, units, prm, step_sizes, &o, &b);
  if (s != PMMC_OK) return s;
  s = pmmc_arcs_batch_run(b, nullptr);
  if (s == PMMC_OK) s = pmmc_arcs_batch_results(b, pos_out, res);
  pmmc_arcs_batch_destroy(b);
  return s;
}

extern "C" pmmc_status pmmc_arcs_anneal(pmmc_ctx *ctx, const pmmc_arcs_problem *pr,
                                        const pmmc_anneal_params *prm, float step_size,
                                        int n_chains, float *pos_out, pmmc_result *res) {
  if (!ctx || !pr || !prm) return fail(ctx, PMMC_ERR_INVALID, "arcs anneal: bad arguments");
  if (n_chains <= 0) n_chains = 4 * ctx->sm_count;
  // a few chains: latency per move decides (one lane per proposal and a
  // drawing warp); many: throughput (two lanes, the chain draws itself)
  const bool few = n_chains <= ctx->sm_count;
  pmmc_batch_opts o{n_chains, 0, few ? 1 : 0, few ? 1 : 0};
  pmmc_arcs_batch *b = nullptr;
  pmmc_status s =
      pmmc_arcs_batch_create_ex(ctx, 1, pr, prm, &step_size, &o, 1, 0, &b);
  if (s != PMMC_OK) return s;
  s = pmmc_arcs_batch_run(b, nullptr);
  if (s == PMMC_OK) s = pmmc_arcs_batch_results(b, pos_out, res);
  pmmc_arcs_batch_destroy(b);
  return s;
}

// ===========================================================================
// Arc-level anneal that allocates nothing
// ===========================================================================
// For callers that cannot allocate device memory themselves or through us:
// code running where cudaMalloc is unavailable or forbidden (a host
// framework that owns the whole device pool and hands out only its own
// buffers, a plugin loaded into a process with a fixed memory budget, code
// between stream-capture phases that must not trigger allocations).  The
// caller passes device-resident inputs and an output buffer; every
// intermediate the anneal needs lives in one file-scope device array of
// fixed size, reserved on a device when this library's module is loaded
// there (lazily, at its first use, under CUDA's default lazy loading) and
// held until the process exits.
namespace {

constexpr int kNoAllocMaxBeads = 4096;      // beads of the region
constexpr int kNoAllocMaxEntries = 16384;   // arc-list entries, both directions

struct NoAllocScratch {
  ArcsUnit unit;
  int2 item;
  int head;
  int done;
  int best;
  int n_null;
  // written by noalloc_check_kernel, read back by the host in one copy
  int status;     // 0 ok, 1 malformed arc lists, 2 more entries than the scratch holds
  int nnz;        // entries of the caller's arc lists (row_ptr[n])
  int n_spring;   // spring entries (target >= 1e-6, partner != bead)
  int n_mov;      // movable beads
  ChainOut out;
  double base;    // frozen repulsion of the start (arcs_base_kernel)
  float4 pos0[kNoAllocMaxBeads];
  int row_ptr[kNoAllocMaxBeads + 1];
  int movable[kNoAllocMaxBeads];
  int2 nbr[kNoAllocMaxEntries];
  float inv_t[kNoAllocMaxEntries];
  int2 nulls[kNoAllocMaxEntries];
  int4 lst[kNoAllocMaxEntries];  // every spring once: the energy recompute's list
};

static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

// One block checks the caller's arc lists before anything reads through
// them (row pointers in order and within row_ptr[n], columns in range, the
// entry count within the scratch) and counts the spring entries and the
// movable beads, which decide the shared-memory layout as in the batched
// path.  A rejected region leaves every caller buffer untouched.
__global__ void noalloc_check_kernel(NoAllocScratch *S, int n, const unsigned char *fixed,
                                     const int *row_ptr, const int *col, const float *target,
                                     int lists_given) {
  __shared__ int s_bad, s_spring, s_mov;
  const int t = threadIdx.x;
  const int nnz = row_ptr[n];
  if (t == 0) {
    s_bad = (row_ptr[0] != 0 || nnz < 0 || (nnz > 0 && !lists_given)) ? 1 : 0;
    if (nnz > kNoAllocMaxEntries) s_bad = 2;
    s_spring = 0;
    s_mov = 0;
  }
  __syncthreads();
  if (s_bad == 0)
    for (int i = t; i < n; i += blockDim.x) {
      const int a = row_ptr[i], z = row_ptr[i + 1];
      if (a < 0 || z < a || z > nnz) atomicOr(&s_bad, 1);
    }
  __syncthreads();
  if (s_bad == 0) {
    int sp = 0, mv = 0;
    for (int i = t; i < n; i += blockDim.x) {
      mv += (fixed && fixed[i]) ? 0 : 1;
      for (int e = row_ptr[i]; e < row_ptr[i + 1]; ++e) {
        const int j = col[e];
        if (j < 0 || j >= n) atomicOr(&s_bad, 1);
        sp += (target[e] >= 1e-6f && j != i) ? 1 : 0;
      }
    }
    atomicAdd(&s_spring, sp);
    atomicAdd(&s_mov, mv);
  }
  __syncthreads();
  if (t == 0) {
    S->status = s_bad;
    S->nnz = nnz;
    S->n_spring = s_spring;
    S->n_mov = s_mov;
  }
}

// One block packs a checked region into the scratch array as the batched
// path packs it on the host: float4 positions, spring-only arc lists with
// reciprocals, inert pairs, the flat spring list, the movable list, the
// work item and counters (which must start at zero).
__global__ void noalloc_stage_kernel(NoAllocScratch *S, int n, const float *pos,
                                     const unsigned char *fixed, const int *row_ptr,
                                     const int *col, const float *target, float step,
                                     uint64_t seed) {
  __shared__ int s_cnt[kNoAllocMaxBeads + 1];
  __shared__ int s_mov[kNoAllocMaxBeads + 1];
  const int t = threadIdx.x;
  for (int i = t; i < n; i += blockDim.x) {
    S->pos0[i] = make_float4(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], 0.0f);
    int c = 0;
    for (int e = row_ptr[i]; e < row_ptr[i + 1]; ++e)
      c += (target[e] >= 1e-6f && col[e] != i) ? 1 : 0;
    s_cnt[i] = c;
    s_mov[i] = (fixed && fixed[i]) ? 0 : 1;
  }
  __syncthreads();
  if (t == 0) {  // prefix sums and the ordered lists (n <= 4096: one thread)
    int acc = 0, m = 0, nn = 0, na = 0;
    for (int i = 0; i < n; ++i) {
      const int c = s_cnt[i];
      s_cnt[i] = acc;
      acc += c;
      const int mv = s_mov[i];
      s_mov[i] = m;
      m += mv;
      for (int e = row_ptr[i]; e < row_ptr[i + 1]; ++e) {
        const int j = col[e];
        const float tg = target[e];
        if (j == i) continue;
        if (tg >= 1e-6f) {
          if (j < i)
            S->lst[na++] = make_int4(j, i, __float_as_int(tg), __float_as_int(1.0f / tg));
        } else if (tg >= 0.0f && j < i) {
          S->nulls[nn++] = make_int2(j, i);
        }
      }
    }
    s_cnt[n] = acc;
    s_mov[n] = m;
    S->n_null = nn;
    ArcsUnit U{};
    U.n = n;
    U.n_mov = m;
    U.pos_off = 0;
    U.rp_off = 0;
    U.nbr_off = 0;
    U.nnz = acc;
    U.mov_off = m < n ? 0 : -1;
    U.lrp_off = -1;
    U.lent_off = 0;
    U.n_lent = 0;
    U.lst_off = 0;
    U.n_loops = 0;
    U.null_off = 0;
    U.n_null = nn;
    U.chains = 1;
    U.chain_base = 0;
    U.out_off = 0;
    U.step = step;
    U.rng_chain = 0;
    U.seed = seed;
    U.arc_off = 0;
    U.n_arcs = na;
    S->unit = U;
    S->item = make_int2(0, 0);
    S->head = 0;
    S->done = 0;
    S->best = 0;
  }
  __syncthreads();
  for (int i = t; i <= n; i += blockDim.x) S->row_ptr[i] = s_cnt[i];
  for (int i = t; i < n; i += blockDim.x) {
    if (!(fixed && fixed[i])) S->movable[s_mov[i]] = i;
    int k = s_cnt[i];
    for (int e = row_ptr[i]; e < row_ptr[i + 1]; ++e) {
      const float tg = target[e];
      if (tg >= 1e-6f && col[e] != i) {
        S->nbr[k] = make_int2(col[e], __float_as_int(tg));
        S->inv_t[k] = 1.0f / tg;
        ++k;
      }
    }
  }
}

// The unique id of the calling thread's current CUDA context (0 when there
// is none or the driver cannot say), through the runtime's driver entry
// points, so that the library needs no link to the driver library.
unsigned long long current_context_id() {
  typedef CUresult (*GetCurrentFn)(CUcontext *);
  typedef CUresult (*GetIdFn)(CUcontext, unsigned long long *);
  static GetCurrentFn get_current = nullptr;
  static GetIdFn get_id = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void *p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_current = reinterpret_cast<GetCurrentFn>(p);
    p = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess && q == cudaDriverEntryPointSuccess)
      get_id = reinterpret_cast<GetIdFn>(p);
    cudaGetLastError();
  });
  CUcontext c = nullptr;
  unsigned long long id = 0;
  if (!get_current || !get_id || get_current(&c) != CUDA_SUCCESS || !c ||
      get_id(c, &id) != CUDA_SUCCESS)
    return 0;
  return id;
}

// Device address of the scratch array for the current device: looked up
// (cudaGetSymbolAddress, with the device current) once per device and
// context, and again whenever the context changed (a cudaDeviceReset, a
// caller's own context), since the array moves with its module.
std::mutex g_noalloc_mutex;
struct NoAllocAddr {
  unsigned long long ctx_id;
  NoAllocScratch *ptr;
};
NoAllocAddr g_noalloc_addr[64] = {};

cudaError_t noalloc_scratch(int dev, NoAllocScratch **out) {
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  NoAllocAddr &a = g_noalloc_addr[dev];
  const unsigned long long id = current_context_id();
  if (a.ptr && id != 0 && a.ctx_id == id) {
    *out = a.ptr;
    return cudaSuccess;
  }
  void *p = nullptr;
  const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
  if (e != cudaSuccess || !p) {
    cudaGetLastError();
    return e != cudaSuccess ? e : cudaErrorInvalidSymbol;
  }
  a.ptr = reinterpret_cast<NoAllocScratch *>(p);
  a.ctx_id = current_context_id();  // the lookup made the context current
  *out = a.ptr;
  return cudaSuccess;
}

}  // namespace

extern "C" pmmc_status pmmc_arcs_anneal_noalloc(const pmmc_arcs_problem *pr,
                                                const pmmc_anneal_params *prm,
                                                float step_size, uint64_t seed,
                                                float *pos_out, pmmc_result *res,
                                                void *stream) {
  if (!pr || !prm || !pos_out || !res || !pr->pos || !pr->row_ptr || pr->n < 1)
    return PMMC_ERR_INVALID;
  if (pr->n_loops != 0) return PMMC_ERR_INVALID;       // loop constraints need packing
  if (pr->n > kNoAllocMaxBeads) return PMMC_ERR_BUDGET; // beyond the fixed scratch
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return PMMC_ERR_NO_DEVICE;
  NoAllocScratch *S = nullptr;
  if (noalloc_scratch(dev, &S) != cudaSuccess) return PMMC_ERR_CUDA;
  cudaStream_t s = (cudaStream_t)stream;
  const int n = pr->n;
  // 1. check the caller's arc lists and count what the layout depends on
  noalloc_check_kernel<<<1, 256, 0, s>>>(S, n, pr->fixed, pr->row_ptr, pr->col, pr->target,
                                         pr->col && pr->target ? 1 : 0);
  int hdr[4] = {0, 0, 0, 0};  // status, nnz, n_spring, n_mov
  if (cudaGetLastError() != cudaSuccess ||
      cudaMemcpyAsync(hdr, &S->status, sizeof(hdr), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return PMMC_ERR_CUDA;
  if (hdr[0] == 2) return PMMC_ERR_BUDGET;   // more arc-list entries than the scratch holds
  if (hdr[0] != 0) return PMMC_ERR_INVALID;  // malformed arc lists: nothing was written
  const int n_spring = hdr[2], n_mov = hdr[3];
  // 2. the batched path's shared-memory decision for this region
  int dev_smem = 0;
  cudaDeviceGetAttribute(&dev_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  const size_t cap_smem = (size_t)dev_smem - kCtaHeader;
  const size_t full = arcs_unit_smem(n, n_spring, n_mov, n_mov < n);
  const size_t minimal = arcs_unit_smem_min(n);
  const bool nbs = full <= cap_smem;
  if (!nbs && minimal > cap_smem) return PMMC_ERR_INVALID;
  const size_t per_warp = ((nbs ? full : minimal) + 15) & ~(size_t)15;
  ArcsDevParams P = arcs_make_params(prm, seed, false);
  ArcsKernelFn fn = arcs_kernel_for(nbs, 2);
  // the device's opt-in maximum, as the batched path sets it: never lower
  // the limit under a batch created earlier
  if (cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, dev_smem) !=
      cudaSuccess)
    return PMMC_ERR_CUDA;
  // 3. stage, the frozen repulsion, one chain
  noalloc_stage_kernel<<<1, 256, 0, s>>>(S, n, pr->pos, pr->fixed, pr->row_ptr, pr->col,
                                         pr->target, step_size, seed);
  if (arcs_bases(&S->unit, 1, S->pos0, S->row_ptr, S->nbr, S->nulls, &S->base, s) !=
      cudaSuccess)
    return PMMC_ERR_CUDA;
  fn<<<1, 32, kCtaHeader + per_warp, s>>>(&S->unit, &S->item, 1, &S->head, S->pos0,
                                          S->row_ptr, S->nbr, S->inv_t, S->movable, nullptr,
                                          nullptr, S->lst, S->nulls, P, (int)per_warp, pos_out,
                                          &S->out, &S->done, nullptr, &S->base);
  if (cudaGetLastError() != cudaSuccess) return PMMC_ERR_CUDA;
  ChainOut o;
  if (cudaMemcpyAsync(&o, &S->out, sizeof(o), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess)
    return PMMC_ERR_CUDA;
  pmmc_result r{};
  r.score = o.score;
  r.energy = o.energy;
  r.energy_fp64 = o.energy_fp64;
  r.rel_error = std::fabs(o.energy - o.energy_fp64) / std::max(std::fabs(o.energy_fp64), 1e-30);
  r.moves = o.moves;
  r.accepted = o.accepted;
  r.total_moves = o.moves;
  r.best_chain = 0;
  r.status = o.status;
  *res = r;
  return PMMC_OK;
}
