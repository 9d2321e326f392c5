// smooth.cu -- subanchor smoothing simulated annealing on GB300.
//
// Energy of a smoothing region (LooperSolver.hpp:3414-3495,
// ParallelMonteCarloSmooth.cu:86-209):
//   bonds   ((|p_i - p_{i+1}| - d0_i) / d0_i)^2 * (stretch | squeeze),
//           d0_i = dist_to_next[i] clamped to 1e-6
//   angles  k_ang * a^3 with a = 1 - (cos(v_i, v_{i-1}) + 1) / 2 at every
//           interior bead, v_i = p_i - p_{i+1}
//   sphere  max(0, |p| - R)^2 per bead
// The full score weights bonds by dist_weight and angles by angle_weight; the
// local score of a move (2 bonds, 3 angles, 1 sphere term) is unweighted --
// the reference's own convention, kept so that the running score matches
// (the two agree at the default weights of 1).
//
// A move touches five beads, so one thread runs one chain: 32 independent
// chains per warp.  A chain's positions sit in the thread's slice of shared
// memory when the region is small (genome-scale smoothing splits chromosomes
// at their fixed anchors into regions of ~10 beads), else in a per-chain
// working copy in global memory (the reference's per-warp copies,
// ParallelMonteCarloSmooth.cu:415-423).
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace pmmc {

struct SmoothUnit {
  int n;
  int n_mov;
  int pos_off;    // float4 index into pos0
  int mov_off;    // into movable (-1 = all movable)
  int dtn_off;    // into dist_to_next
  int chains;
  int chain_base;
  int pad;
  long long out_off;   // float index of chain 0's xyz output
  long long work_off;  // float4 index of chain 0's global working copy
  float step;
  int pad2;
  long long cap;       // hard move cap of the unit's chains
};

struct SmoothDevParams {
  float max_temp;
  float dt;
  float inv_scale;
  float inv_coef;
  float improvement;
  float ks, kq, kang, wd, wa, R;
  int min_succ;
  int window;
  int fails;
  int use2d;
  int resync;     // full recompute every `resync` moves (0 = off)
  int slice;      // beads per thread slice (shared-memory path)
  int gpu_sched;  // the reference kernel's schedule: no milestone, fixed cap,
                  // ratio denominator at least 1e-12
  int pad;
  long long cap;
  uint64_t seed;
};

// Bond term with the clamped target d0 and its reciprocal precomputed:
// ((|a - b| - d0) / d0)^2 * (stretch | squeeze).
__device__ __forceinline__ float bond_e(float4 a, float4 b, float2 d, float ks,
                                        float kq) {
  const float len = ref_len(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
  const float f = (len - d.x) * d.y;
  return f * f * (f >= 0.0f ? ks : kq);
}

// angle() of the reference (common.cpp:39-46) for v1 = a - b, v2 = b - c
// (the bonds before and after bead b): (1 - cos) / 2, cubed and scaled; a
// zero-length bond normalises to the zero vector (cos = 0).
__device__ __forceinline__ float angle_e(float4 a, float4 b, float4 c,
                                         float kang) {
  const float x1 = a.x - b.x, y1 = a.y - b.y, z1 = a.z - b.z;
  const float x2 = b.x - c.x, y2 = b.y - c.y, z2 = b.z - c.z;
  const float s1 = fmaf(x1, x1, fmaf(y1, y1, z1 * z1));
  const float s2 = fmaf(x2, x2, fmaf(y2, y2, z2 * z2));
  const float m = (s1 > 0.0f && s2 > 0.0f) ? rsqrtf(s1) * rsqrtf(s2) : 0.0f;
  const float dot = fmaf(x1, x2, fmaf(y1, y2, z1 * z2)) * m;
  const float ang = 0.5f - 0.5f * dot;
  return ang * ang * ang * kang;
}

// Local score of bead p at position q (calcScoreStructureSmooth(p,true,true)
// plus the bead's sphere term).
// P[i * st]: bead i of the chain (st = 32 when a warp's chains interleave).
__device__ __forceinline__ float smooth_local(const float4 *P, int st, const float2 *dtn,
                                              int n, int p, float4 q,
                                              const SmoothDevParams &S) {
  float s = 0.0f;
  const float4 pm1 = p >= 1 ? P[(p - 1) * st] : q;
  const float4 pp1 = p + 1 < n ? P[(p + 1) * st] : q;
  if (p >= 1) s += bond_e(pm1, q, dtn[p - 1], S.ks, S.kq);
  if (p + 1 < n) s += bond_e(q, pp1, dtn[p], S.ks, S.kq);
  if (p >= 2) s += angle_e(P[(p - 2) * st], pm1, q, S.kang);       // angle at p-1
  if (p >= 1 && p + 1 < n) s += angle_e(pm1, q, pp1, S.kang);      // at p
  if (p + 2 < n) s += angle_e(q, pp1, P[(p + 2) * st], S.kang);    // at p+1
  s += sphere_penalty(q.x, q.y, q.z, S.R);
  return s;
}

// Exact (IEEE sqrt / division) forms for the FP64 recompute.
__device__ __forceinline__ double bond_exact(float4 a, float4 b, float d0, float ks, float kq) {
  const float x = a.x - b.x, y = a.y - b.y, z = a.z - b.z;
  const double f = ((double)sqrtf(x * x + y * y + z * z) - (double)d0) / (double)d0;
  return f * f * (double)(f >= 0.0 ? ks : kq);
}

__device__ __forceinline__ double angle_exact(float4 a, float4 b, float4 c, float kang) {
  float x1 = a.x - b.x, y1 = a.y - b.y, z1 = a.z - b.z;
  float x2 = b.x - c.x, y2 = b.y - c.y, z2 = b.z - c.z;
  float m1 = sqrtf(x1 * x1 + y1 * y1 + z1 * z1);
  float m2 = sqrtf(x2 * x2 + y2 * y2 + z2 * z2);
  m1 = m1 > 0.0f ? 1.0f / m1 : 0.0f;
  m2 = m2 > 0.0f ? 1.0f / m2 : 0.0f;
  const float dot = (x1 * m1) * (x2 * m2) + (y1 * m1) * (y2 * m2) + (z1 * m1) * (z2 * m2);
  const double ang = 1.0f - (dot + 1.0f) / 2.0f;
  return ang * ang * ang * (double)kang;
}

// FP64 full score (calcScoreStructureSmooth(true,true) + sphere).
__device__ double smooth_full(const float4 *P, int st, const float2 *dtn, int n,
                              const SmoothDevParams &S) {
  double sa = 0.0, sb = 0.0, sp = 0.0;
  for (int i = 0; i + 1 < n; ++i) {
    sa += bond_exact(P[i * st], P[(i + 1) * st], dtn[i].x, S.ks, S.kq);
    if (i > 0) sb += angle_exact(P[(i - 1) * st], P[i * st], P[(i + 1) * st], S.kang);
  }
  for (int i = 0; i < n; ++i) {
    const float4 q = P[i * st];
    sp += sphere_penalty(q.x, q.y, q.z, S.R);
  }
  return sa * (double)S.wd + sb * (double)S.wa + sp;
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

// Two lanes per chain: a move's two local energies (the bead at its old and
// at its proposed position) are evaluated side by side, one per lane, and
// its two draws (proposal, Metropolis threshold) likewise; the lanes swap
// their results with one shuffle and keep identical copies of the chain's
// state.  A thread alone ran one long dependent instruction chain per move
// with few warps to hide it.
constexpr int kSmoothLanes = 2;

template <bool SMEM>
__global__ void __launch_bounds__(128)
smooth_anneal_kernel(const SmoothUnit *__restrict__ units,
                     const int2 *__restrict__ items, int n_items,
                     const float4 *__restrict__ pos0, const float2 *__restrict__ dtn_all,
                     const int *__restrict__ movable, SmoothDevParams S,
                     float4 *__restrict__ work, float *__restrict__ pos_out,
                     ChainOut *__restrict__ outs, MoveTrace *__restrict__ trace,
                     int trace_cap) {
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr int CPW = 32 / kSmoothLanes;  // chains per warp
  const int lane = threadIdx.x & 31;
  const int sub = lane & (kSmoothLanes - 1);
  const int item = (blockIdx.x * blockDim.x + threadIdx.x) / kSmoothLanes;
  if (item >= n_items) return;  // both lanes of a chain leave together
  const unsigned gm = ((1u << kSmoothLanes) - 1u) << (lane & ~(kSmoothLanes - 1));
  const int2 it = items[item];
  const SmoothUnit U = units[it.x];
  const int chain = it.y;
  const int n = U.n;
  const uint32_t chain_id = (uint32_t)(U.chain_base + chain);
  // shared-memory path: the chains of a warp interleave bead by bead (bead i
  // of chain c at i * CPW + c), so that the chains' loads of any beads fall
  // on distinct banks within a quarter warp; the two lanes of a chain read
  // the same words
  const int st = SMEM ? CPW : 1;
  float4 *P = SMEM ? reinterpret_cast<float4 *>(smem) +
                         (size_t)(threadIdx.x >> 5) * S.slice * CPW + (lane / kSmoothLanes)
                   : work + U.work_off + (long long)chain * n;
  const float2 *dtn = dtn_all + U.dtn_off;
  const int *MOV = U.mov_off >= 0 ? movable + U.mov_off : nullptr;
  for (int i = sub; i < n; i += kSmoothLanes) P[i * st] = pos0[U.pos_off + i];
  __syncwarp(gm);

  const double E0 = smooth_full(P, st, dtn, n, S);
  // running score: float-float pair per move, widened to FP64 at milestones
  float e_hi = (float)E0, e_lo = (float)(E0 - (double)(float)E0);
  double E_ms = E0, best = E0;
  float T = S.max_temp;
  long long moves = 0, accepted = 0;
  int succ = 0, misses = 0, status = kDevOk;
  bool stop = U.n_mov == 0 || U.cap <= 0;
  if (U.n_mov == 0) status = kDevNoMovable;
  // milestone and recompute counters (no 64-bit division per move)
  long long next_ms = S.window > 0 ? (long long)S.window : 0x7fffffffffffffffLL;
  long long next_rs = S.resync > 0 ? (long long)S.resync : 0x7fffffffffffffffLL;
  // The draws of a move depend only on its index and temperature, not on the
  // chain's state; those of the next move are made while this move is
  // scored.  Lane 0 draws the proposal (tag 0), lane 1 the threshold (tag 1).
  struct Draw {
    int b;
    float dx, dy, dz, thr;
  };
  auto draw = [&](long long mv, float Tm) {
    const uint4 r = philox_move(S.seed, chain_id, (uint64_t)mv, (uint32_t)sub);
    const int k = uniform_index(r.x, U.n_mov);
    Draw w;
    w.b = MOV ? MOV[k] : k;
    w.dx = (2.0f * u01(r.y) - 1.0f) * U.step;
    w.dy = (2.0f * u01(r.z) - 1.0f) * U.step;
    w.dz = S.use2d ? 0.0f : (2.0f * u01(r.w) - 1.0f) * U.step;
    w.thr = ratio_threshold(u01(r.x), Tm, S.inv_scale, S.inv_coef);
    return w;
  };
  const int lead = lane & ~(kSmoothLanes - 1);
  auto share = [&](const Draw &w) {
    Draw o;
    o.b = __shfl_sync(gm, w.b, lead);
    o.dx = __shfl_sync(gm, w.dx, lead);
    o.dy = __shfl_sync(gm, w.dy, lead);
    o.dz = __shfl_sync(gm, w.dz, lead);
    o.thr = __shfl_sync(gm, w.thr, lead + 1);
    return o;
  };
  Draw cur = share(draw(moves, T));
  while (!stop) {
    const Draw nxt = draw(moves + 1, T * S.dt);  // T of the next move
    const int b = cur.b;
    const float ddx = cur.dx, ddy = cur.dy, ddz = cur.dz;
    const float4 ob = P[b * st];
    float4 nb = ob;
    nb.x += ddx;
    nb.y += ddy;
    nb.z += ddz;
    // lane 0 the old local energy, lane 1 the new one
    const float mine = smooth_local(P, st, dtn, n, b, sub ? nb : ob, S);
    const float other = __shfl_xor_sync(gm, mine, 1);
    const float so = sub ? other : mine;
    const float sn = sub ? mine : other;
    const float d = sn - so;
    // strict improvement (LooperSolver.hpp:4974), else the ratio test
    bool acc = d < 0.0f;
    if (!acc && T > 0.0f) {
      const float thr = cur.thr;
      // the reference kernel divides by max(E_prev, 1e-12)
      // (ParallelMonteCarloSmooth.cu:293-294)
      acc = (S.gpu_sched && e_hi < 1e-12f) ? d < 1e-12f * thr - e_hi
                                           : d < e_hi * (thr - 1.0f);
    }
    if (acc) {
      if (sub == 0) P[b * st] = nb;
      ff_add(e_hi, e_lo, d);
      ++accepted;
      ++succ;
      if (S.gpu_sched) best = fmin(best, (double)e_hi + (double)e_lo);
    }
    if (trace != nullptr && chain_id == 0 && sub == 0 && moves < trace_cap) {
      MoveTrace tr;
      tr.bead = b;
      tr.accepted = acc ? 1 : 0;
      tr.before = so;
      tr.after = sn;
      tr.dx = ddx;
      tr.dy = ddy;
      tr.dz = ddz;
      tr.pad = d;
      trace[moves] = tr;
    }
    __syncwarp(gm);  // the accepted position is visible to both lanes
    ++moves;
    if (moves == next_rs) {
      // remove the drift of the running score (a region is small: the
      // recompute is a few dozen terms)
      next_rs += S.resync;
      const double Er = smooth_full(P, st, dtn, n, S);
      e_hi = (float)Er;
      e_lo = (float)(Er - (double)e_hi);
    }
    if (moves == next_ms) {
      next_ms += S.window;
      const double E = (double)e_hi + (double)e_lo;
      const bool miss = (E > (double)S.improvement * E_ms && succ < S.min_succ) || E < 1e-6;
      misses = miss ? misses + 1 : 0;
      if (misses >= S.fails || E < 1e-6) stop = true;
      E_ms = E;
      succ = 0;
    }
    T *= S.dt;
    if (!stop && moves >= U.cap) stop = true;
    cur = share(nxt);
  }
  if (sub == 0) {
    ChainOut o;
    o.energy = (double)e_hi + (double)e_lo;
    o.energy_fp64 = smooth_full(P, st, dtn, n, S);
    o.base = 0.0;
    o.best = S.gpu_sched ? best : o.energy;
    o.score = e_hi;
    o.status = status;
    o.moves = moves;
    o.accepted = accepted;
    outs[U.chain_base + chain] = o;
  }
  float *po = pos_out + U.out_off + (long long)chain * n * 3;
  for (int i = sub; i < n; i += kSmoothLanes) {
    const float4 q = P[i * st];
    po[3 * i] = q.x;
    po[3 * i + 1] = q.y;
    po[3 * i + 2] = q.z;
  }
}

}  // namespace pmmc

using namespace pmmc;

namespace {

SmoothDevParams smooth_params(const pmmc_anneal_params *prm, uint64_t seed) {
  SmoothDevParams S{};
  S.max_temp = prm->max_temp;
  S.dt = prm->dt_temp;
  S.inv_scale = prm->jump_scale != 0.0f ? 1.0f / prm->jump_scale : 0.0f;
  S.inv_coef = prm->jump_coef != 0.0f ? 1.0f / prm->jump_coef : 0.0f;
  S.improvement = prm->improvement;
  S.ks = prm->k_stretch;
  S.kq = prm->k_squeeze;
  S.kang = prm->k_angle;
  S.wd = prm->w_dist;
  S.wa = prm->w_angle;
  S.R = prm->sphere_radius;
  S.min_succ = prm->min_successes;
  S.use2d = prm->use2d;
  // the weighted full score equals the running (unweighted-delta) score only
  // at unit weights (the reference's convention): recompute only then
  S.resync = (prm->resync_every > 0 && prm->w_dist == 1.0f && prm->w_angle == 1.0f)
                 ? prm->resync_every : 0;
  S.seed = seed;
  if (prm->schedule == PMMC_SCHEDULE_CPU) {
    S.window = std::max(1, prm->milestone_steps);
    S.fails = 1;
    S.cap = prm->max_moves > 0 ? prm->max_moves : 200ll * S.window;
  } else {
    // MonteCarloSmoothKernelMultiWarp (ParallelMonteCarloSmooth.cu:267-337):
    // blocks of 256 moves while fewer than stop_condition_steps are done.
    // Its milestone test runs only when iterations % steps < 256, which
    // inside that loop is only after the last block: every chain makes
    // exactly the cap's moves, so no milestone is evaluated here.
    S.window = 0;
    S.fails = 1;
    S.gpu_sched = 1;
    long long cap = prm->milestone_steps > 0 ? ((long long)prm->milestone_steps + 255) / 256 * 256
                                             : 0;
    if (prm->max_moves > 0) cap = std::min(cap, (long long)prm->max_moves);
    S.cap = cap;
  }
  return S;
}

}  // namespace

// Smoothing of many regions (and/or many chains per region) in one pass.
extern "C" pmmc_status pmmc_smooth_batch_anneal(pmmc_ctx *ctx, int n_units,
                                               const pmmc_smooth_problem *units,
                                               const pmmc_anneal_params *prm,
                                               const float *steps, int chains,
                                               float *pos_out, pmmc_result *res,
                                               double *kernel_ms, void *trace_out,
                                               int trace_cap) {
  if (!ctx || n_units < 1 || !units || !prm || !steps)
    return fail(ctx, PMMC_ERR_INVALID, "smooth batch: bad arguments");
  if (chains < 1) chains = 1;
  SmoothDevParams S = smooth_params(prm, next_key(ctx));
  std::vector<SmoothUnit> hu(n_units);
  std::vector<float4> hpos;
  std::vector<float2> hdtn;
  std::vector<int> hmov;
  long long out_off = 0, work_off = 0;
  int chain_base = 0, max_n = 0;
  for (int u = 0; u < n_units; ++u) {
    const pmmc_smooth_problem &pr = units[u];
    if (pr.n < 1 || !pr.pos || !pr.dist_to_next)
      return fail(ctx, PMMC_ERR_INVALID, "smooth region %d: n, pos, dist_to_next required", u);
    SmoothUnit U{};
    U.n = pr.n;
    U.pos_off = (int)hpos.size();
    U.dtn_off = (int)hdtn.size();
    for (int i = 0; i < pr.n; ++i) {
      hpos.push_back(make_float4(pr.pos[3 * i], pr.pos[3 * i + 1], pr.pos[3 * i + 2], 0.0f));
      // clamp as calcScoreStructureSmooth does (LooperSolver.hpp:3470-3471)
      const float d0 = pr.dist_to_next[i] < 1e-6f ? 1e-6f : pr.dist_to_next[i];
      hdtn.push_back(make_float2(d0, 1.0f / d0));
    }
    std::vector<int> mv;
    for (int i = 0; i < pr.n; ++i)
      if (!pr.fixed || !pr.fixed[i]) mv.push_back(i);
    U.n_mov = (int)mv.size();
    if (U.n_mov < pr.n) {
      U.mov_off = (int)hmov.size();
      hmov.insert(hmov.end(), mv.begin(), mv.end());
    } else {
      U.mov_off = -1;
    }
    U.chains = chains;
    U.chain_base = chain_base;
    U.out_off = out_off;
    U.work_off = work_off;
    U.step = steps[u];
    // max_moves < 0: -max_moves sweeps (one proposal per movable bead each)
    U.cap = prm->max_moves < 0 ? std::max(1LL, (long long)(-prm->max_moves) * U.n_mov) : S.cap;
    chain_base += chains;
    out_off += (long long)chains * pr.n * 3;
    work_off += (long long)chains * pr.n;
    max_n = std::max(max_n, pr.n);
    hu[u] = U;
  }
  if (hmov.empty()) hmov.push_back(0);
  // items: largest regions first
  std::vector<int> order(n_units);
  for (int u = 0; u < n_units; ++u) order[u] = u;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return hu[a].n > hu[b].n; });
  std::vector<int2> items;
  items.reserve((size_t)n_units * chains);
  for (int u : order)
    for (int c = 0; c < chains; ++c) items.push_back(make_int2(u, c));

  const int threads = 128;
  // shared-memory slices when a chain's region fits in 1 KB... 4 KB
  int slice = 0;
  if (max_n <= 64) slice = max_n;
  S.slice = slice;
  const bool use_smem = slice > 0;
  const size_t smem =
      use_smem ? (size_t)(threads / kSmoothLanes) * slice * sizeof(float4) : 0;

  cudaStream_t s = ctx->stream;
  DevBuf<SmoothUnit> d_units;
  DevBuf<int2> d_items;
  DevBuf<float4> d_pos, d_work;
  DevBuf<float2> d_dtn;
  DevBuf<float> d_out;
  DevBuf<int> d_mov;
  DevBuf<ChainOut> d_outs;
  DevBuf<MoveTrace> d_trace;
  cudaError_t e = d_units.upload(hu, s);
  if (e == cudaSuccess && trace_cap > 0) e = d_trace.alloc((size_t)trace_cap);
  if (e == cudaSuccess) e = d_items.upload(items, s);
  if (e == cudaSuccess) e = d_pos.upload(hpos, s);
  if (e == cudaSuccess) e = d_dtn.upload(hdtn, s);
  if (e == cudaSuccess) e = d_mov.upload(hmov, s);
  if (e == cudaSuccess) e = d_out.alloc((size_t)out_off);
  if (e == cudaSuccess) e = d_outs.alloc((size_t)chain_base);
  if (e == cudaSuccess && !use_smem) e = d_work.alloc((size_t)work_off);
  if (e != cudaSuccess)
    return fail(ctx, e == cudaErrorMemoryAllocation ? PMMC_ERR_NOMEM : PMMC_ERR_CUDA,
                "smooth batch upload: %s", cudaGetErrorString(e));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  const int n_items = (int)items.size();
  const int grid = (int)(((long long)n_items * kSmoothLanes + threads - 1) / threads);
  cudaEventRecord(e0, s);
  if (use_smem) {
    cudaFuncSetAttribute(smooth_anneal_kernel<true>,
                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    smooth_anneal_kernel<true><<<grid, threads, smem, s>>>(
        d_units.p, d_items.p, n_items, d_pos.p, d_dtn.p, d_mov.p, S, nullptr, d_out.p,
        d_outs.p, trace_cap > 0 ? d_trace.p : nullptr, trace_cap);
  } else {
    smooth_anneal_kernel<false><<<grid, threads, 0, s>>>(
        d_units.p, d_items.p, n_items, d_pos.p, d_dtn.p, d_mov.p, S, d_work.p, d_out.p,
        d_outs.p, trace_cap > 0 ? d_trace.p : nullptr, trace_cap);
  }
  e = cudaGetLastError();
  cudaEventRecord(e1, s);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  if (e == cudaSuccess && kernel_ms) {
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    *kernel_ms = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (e != cudaSuccess)
    return fail(ctx, PMMC_ERR_CUDA, "smooth kernel: %s", cudaGetErrorString(e));

  std::vector<ChainOut> outs(chain_base);
  PMMC_CUDA(ctx, cudaMemcpy(outs.data(), d_outs.p, sizeof(ChainOut) * outs.size(),
                            cudaMemcpyDeviceToHost));
  if (trace_out && trace_cap > 0)
    PMMC_CUDA(ctx, cudaMemcpy(trace_out, d_trace.p, sizeof(MoveTrace) * trace_cap,
                              cudaMemcpyDeviceToHost));
  long long dst = 0;
  for (int u = 0; u < n_units; ++u) {
    const SmoothUnit &U = hu[u];
    // the reported chain: the lowest final running energy; under the
    // reference kernel's schedule, the lowest running energy ever reached
    // (its per-warp best score, ParallelMonteCarloSmooth.cu:299-301,462-472),
    // ties to the lower index
    int best = 0;
    for (int c = 1; c < U.chains; ++c) {
      const ChainOut &oc = outs[U.chain_base + c], &ob = outs[U.chain_base + best];
      if (S.gpu_sched ? oc.best < ob.best : oc.energy < ob.energy) best = c;
    }
    const ChainOut &o = outs[U.chain_base + best];
    if (pos_out) {
      PMMC_CUDA(ctx, cudaMemcpy(pos_out + dst, d_out.p + U.out_off + (long long)best * U.n * 3,
                                sizeof(float) * U.n * 3, cudaMemcpyDeviceToHost));
      // fixed beads are written back unchanged (ParallelMonteCarloSmooth.cu:485-491)
      const pmmc_smooth_problem &pr = units[u];
      if (pr.fixed)
        for (int i = 0; i < U.n; ++i)
          if (pr.fixed[i])
            for (int c = 0; c < 3; ++c) pos_out[dst + 3 * i + c] = pr.pos[3 * i + c];
    }
    dst += (long long)U.n * 3;
    if (res) {
      pmmc_result r{};
      r.score = o.score;
      r.energy = o.energy;
      r.energy_fp64 = o.energy_fp64;
      r.rel_error = std::fabs(o.energy - o.energy_fp64) / std::max(std::fabs(o.energy_fp64), 1e-30);
      r.moves = o.moves;
      r.accepted = o.accepted;
      long long tot = 0;
      for (int c = 0; c < U.chains; ++c) tot += outs[U.chain_base + c].moves;
      r.total_moves = tot;
      r.best_chain = best;
      r.status = o.status;
      res[u] = r;
    }
  }
  return PMMC_OK;
}

extern "C" pmmc_status pmmc_smooth_anneal(pmmc_ctx *ctx, const pmmc_smooth_problem *pr,
                                          const pmmc_anneal_params *prm, float step_size,
                                          int n_chains, float *pos_out, pmmc_result *res) {
  if (!ctx || !pr || !prm) return fail(ctx, PMMC_ERR_INVALID, "smooth anneal: bad arguments");
  if (n_chains <= 0) n_chains = ctx->sm_count;
  return pmmc_smooth_batch_anneal(ctx, 1, pr, prm, &step_size, n_chains, pos_out, res, nullptr,
                                  nullptr, 0);
}
