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
// Two kernels make the same moves and decisions.  The windowed kernel (the
// default wherever a chain fits its shared-memory slice) gives each chain W
// lanes that score the proposals of W consecutive moves at once and resolve
// them in order; genome-scale smoothing splits chromosomes at their fixed
// anchors into ~30k regions of ~10 beads, each chain a few hundred thousand
// moves long, and annealing accepts under 1% of them, so nearly every window
// is whole.  The one-move-at-a-time kernel gives each chain two lanes; a
// chain's positions sit in shared memory when the region is small, else in a
// per-chain working copy in global memory (the reference's per-warp copies,
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

// A smoothing move draws one Philox block: x picks the bead (the high word
// of x * n_mov) and the low word of the same product -- x's fractional part
// within the bead's interval, uniform and independent of which bead -- is the
// Metropolis uniform; y, z, w are the displacement.  (The other levels draw
// the uniform from a second block, tag 1.)
__device__ __forceinline__ uint32_t bead_fraction(uint32_t x, int n_mov) {
  return x * (uint32_t)n_mov;
}

// Bond term with the clamped target d0 and its reciprocal precomputed:
// ((|a - b| - d0) / d0)^2 * (stretch | squeeze).
__device__ __forceinline__ float bond_e(float4 a, float4 b, float2 d, float ks,
                                        float kq) {
  const float len = ref_len(__fsub_rn(a.x, b.x), __fsub_rn(a.y, b.y), __fsub_rn(a.z, b.z));
  const float f = __fmul_rn(__fsub_rn(len, d.x), d.y);
  return __fmul_rn(__fmul_rn(f, f), f >= 0.0f ? ks : kq);
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
  const float m = (s1 > 0.0f && s2 > 0.0f) ? __fmul_rn(rsqrtf(s1), rsqrtf(s2)) : 0.0f;
  const float dot = __fmul_rn(fmaf(x1, x2, fmaf(y1, y2, z1 * z2)), m);
  const float ang = fmaf(-0.5f, dot, 0.5f);
  return __fmul_rn(__fmul_rn(__fmul_rn(ang, ang), ang), kang);
}

// Local score of bead p at position q (calcScoreStructureSmooth(p,true,true)
// plus the bead's sphere term).  Every operation is rounded explicitly (no
// contraction left to the compiler), so the score of a bead is the same bits
// in every kernel and call site that evaluates it.
// P[i * st]: bead i of the chain (st = 32 when a warp's chains interleave).
// The five terms are evaluated unconditionally (a missing neighbour at a
// chain end reads the bead itself and its term is then dropped), so they
// have no branches between them and schedule side by side; with a branch
// per term a lone chain ran them one after another, ~5x the latency.
// SPH = false leaves out the sphere term (no container: the term is 0).
template <bool SPH = true>
__device__ __forceinline__ float smooth_local(const float4 *P, int st, const float2 *dtn,
                                              int n, int p, float4 q,
                                              const SmoothDevParams &S) {
  const bool l1 = p >= 1, l2 = p >= 2, r1 = p + 1 < n, r2 = p + 2 < n;
  const float4 vm2 = P[(l2 ? p - 2 : p) * st], vm1 = P[(l1 ? p - 1 : p) * st];
  const float4 vp1 = P[(r1 ? p + 1 : p) * st], vp2 = P[(r2 ? p + 2 : p) * st];
  const float2 d0 = dtn[l1 ? p - 1 : p], d1 = dtn[p];
  const float4 pm1 = l1 ? vm1 : q;
  const float4 pp1 = r1 ? vp1 : q;
  const float b0 = bond_e(pm1, q, d0, S.ks, S.kq);
  const float b1 = bond_e(q, pp1, d1, S.ks, S.kq);
  const float a0 = angle_e(vm2, pm1, q, S.kang);   // angle at p-1
  const float a1 = angle_e(pm1, q, pp1, S.kang);   // at p
  const float a2 = angle_e(q, pp1, vp2, S.kang);   // at p+1
  float s = 0.0f;
  s = __fadd_rn(s, l1 ? b0 : 0.0f);
  s = __fadd_rn(s, r1 ? b1 : 0.0f);
  s = __fadd_rn(s, l2 ? a0 : 0.0f);
  s = __fadd_rn(s, (l1 && r1) ? a1 : 0.0f);
  s = __fadd_rn(s, r2 ? a2 : 0.0f);
  return SPH ? __fadd_rn(s, sphere_penalty(q.x, q.y, q.z, S.R)) : s;
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

// Bead i's share of the FP64 full score (calcScoreStructureSmooth(true,true)
// + sphere): the bond to bead i+1, the angle at i and the sphere term.
__device__ __forceinline__ double smooth_term(const float4 *P, int st, const float2 *dtn,
                                              int n, int i, const SmoothDevParams &S) {
  const float4 pi = P[i * st];
  double t = (double)sphere_penalty(pi.x, pi.y, pi.z, S.R);
  if (i + 1 < n) {
    const float4 pn = P[(i + 1) * st];
    t += bond_exact(pi, pn, dtn[i].x, S.ks, S.kq) * (double)S.wd;
    if (i > 0) t += angle_exact(P[(i - 1) * st], pi, pn, S.kang) * (double)S.wa;
  }
  return t;
}

// FP64 full score shared by the L lanes of `mask` (consecutive, lane g of
// them) and summed in one fixed order whatever L is: 32 partial sums (bead
// i into partial i mod 32, in ascending order) combined as a 32-lane
// butterfly (offsets 16, 8, 4, 2, 1).  Each lane holds the partials of the
// virtual lanes g, g+L, ...; every lane returns the same bits.  The bead
// terms are spread over the lanes, not repeated on each (FP64 issues at a
// small fraction of the FP32 rate).
template <int L>
__device__ double smooth_full_lanes(const float4 *P, int st, const float2 *dtn, int n,
                                    const SmoothDevParams &S, int g, unsigned mask) {
  constexpr int K = 32 / L;
  double a[K];
#pragma unroll
  for (int k = 0; k < K; ++k) {
    double v = 0.0;
    for (int i = g + L * k; i < n; i += 32) v += smooth_term(P, st, dtn, n, i, S);
    a[k] = v;
  }
#pragma unroll
  for (int m = K / 2; m >= 1; m >>= 1)
#pragma unroll
    for (int k = 0; k < m; ++k) a[k] = a[k] + a[k + m];
  double v = a[0];
#pragma unroll
  for (int o = L / 2; o >= 1; o >>= 1) {
    const int lo = __shfl_xor_sync(mask, __double2loint(v), o);
    const int hi = __shfl_xor_sync(mask, __double2hiint(v), o);
    v = v + __hiloint2double(hi, lo);
  }
  return v;
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

  const double E0 = smooth_full_lanes<kSmoothLanes>(P, st, dtn, n, S, sub, gm);
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
  // scored (one Philox block a move, the same on both lanes).
  struct Draw {
    int b;
    float dx, dy, dz, thr;
  };
  auto draw = [&](long long mv, float Tm) {
    const uint4 r = philox_move(S.seed, chain_id, (uint64_t)mv, 0u);
    const int k = uniform_index(r.x, U.n_mov);
    Draw w;
    w.b = MOV ? MOV[k] : k;
    w.dx = (2.0f * u01(r.y) - 1.0f) * U.step;
    w.dy = (2.0f * u01(r.z) - 1.0f) * U.step;
    w.dz = S.use2d ? 0.0f : (2.0f * u01(r.w) - 1.0f) * U.step;
    w.thr = ratio_threshold(u01(bead_fraction(r.x, U.n_mov)), Tm, S.inv_scale, S.inv_coef);
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
      const double Er = smooth_full_lanes<kSmoothLanes>(P, st, dtn, n, S, sub, gm);
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
  const double Ef = smooth_full_lanes<kSmoothLanes>(P, st, dtn, n, S, sub, gm);
  if (sub == 0) {
    ChainOut o;
    o.energy = (double)e_hi + (double)e_lo;
    o.energy_fp64 = Ef;
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

// One move's draws (windowed kernel): bead, displacement, Metropolis
// threshold and the move's temperature.
struct Draw {
  int b;
  float dx, dy, dz, thr, T;
};

// Windows of W proposals per chain, W lanes each holding one: the proposals
// of moves m .. m+W-1 are drawn and scored at once against the positions at
// the window's start, then resolved in order.  A proposal whose bead lies
// within two beads of an earlier accepted proposal of the window (its local
// score reads the moved bead) closes the window there and is scored again,
// from the updated positions, as the first slot of the next window (with the
// same draws: they depend only on the move's index).  The resolution takes
// the slots in order with the chain's own float-float running score: every
// slot is tested against the current score
// at once, the first slot that passes is accepted (the ones before it failed
// against the score they would have seen) and the score moves on, so every
// decision, score and position is that of the one-move-at-a-time kernel
// above.  Annealing accepts few moves (under 1% at the genome-smoothing
// temperatures), so a window is nearly always whole and resolves in one
// ballot.  The local score of every bead at its current position is kept in
// shared memory and refreshed around each accepted move, so a slot scores
// only its proposed position.
template <int W, bool SPH>
__global__ void __launch_bounds__(128, 6)
smooth_window_kernel(const SmoothUnit *__restrict__ units,
                     const int2 *__restrict__ items, int n_items,
                     const float4 *__restrict__ pos0, const float2 *__restrict__ dtn_all,
                     const int *__restrict__ movable, SmoothDevParams S,
                     float *__restrict__ pos_out, ChainOut *__restrict__ outs,
                     MoveTrace *__restrict__ trace, int trace_cap) {
  static_assert(W == 4 || W == 8 || W == 16 || W == 32, "window of 4, 8, 16 or 32 slots");
  extern __shared__ __align__(16) unsigned char smem[];
  constexpr unsigned FULL = 0xffffffffu;
  constexpr unsigned SLOTS = W == 32 ? 0xffffffffu : (1u << W) - 1u;
  const int lane = threadIdx.x & 31;
  const int g = lane % W;          // slot
  const int gb = lane - g;         // the group's first lane
  const unsigned gmask = SLOTS << gb;
  const int item = (blockIdx.x * blockDim.x + threadIdx.x) / W;
  const bool live = item < n_items;
  const int2 it = live ? items[item] : make_int2(0, 0);
  const SmoothUnit U = units[it.x];
  const int chain = it.y;
  const int n = U.n;
  const uint32_t chain_id = (uint32_t)(U.chain_base + chain);
  // the group's chain in shared memory: positions, bond targets and the
  // local score of every bead, S.slice beads each
  const int groups = blockDim.x / W, grp = threadIdx.x / W;
  float4 *P = reinterpret_cast<float4 *>(smem) + (size_t)grp * S.slice;
  float2 *D = reinterpret_cast<float2 *>(reinterpret_cast<float4 *>(smem) +
                                         (size_t)groups * S.slice) + (size_t)grp * S.slice;
  float *SO = reinterpret_cast<float *>(reinterpret_cast<float2 *>(reinterpret_cast<float4 *>(smem) +
                                                                  (size_t)groups * S.slice) +
                                        (size_t)groups * S.slice) + (size_t)grp * S.slice;
  const int *MOV = U.mov_off >= 0 ? movable + U.mov_off : nullptr;
  if (live)
    for (int i = g; i < n; i += W) {
      P[i] = pos0[U.pos_off + i];
      D[i] = dtn_all[U.dtn_off + i];
    }
  __syncwarp();
  if (live)
    for (int i = g; i < n; i += W) SO[i] = smooth_local<SPH>(P, 1, D, n, i, P[i], S);

  const double E0 = live ? smooth_full_lanes<W>(P, 1, D, n, S, g, gmask) : 0.0;
  float e_hi = (float)E0, e_lo = (float)(E0 - (double)(float)E0);
  double E_ms = E0, best = E0;
  long long moves = 0, accepted = 0;
  int succ = 0, misses = 0, status = kDevOk;
  bool stop = !live || U.n_mov == 0 || U.cap <= 0;
  if (U.n_mov == 0) status = kDevNoMovable;
  long long next_ms = S.window > 0 ? (long long)S.window : 0x7fffffffffffffffLL;
  long long next_rs = S.resync > 0 ? (long long)S.resync : 0x7fffffffffffffffLL;
  const bool tracing = trace != nullptr && chain_id == 0 && live;
  __syncwarp();

  // The draws of a move depend only on its index and temperature.  Each
  // lane holds those of its slot in this window (move moves+g) and, drawn
  // while this window is scored, those of move moves+W+g; the next window's
  // slots (moves+lend+g) are among the two, so a window never waits for a
  // Philox draw.  Temperatures are the one-move-at-a-time sequence of float
  // products, extended W moves at a time.
  const bool has_mov = U.n_mov > 0;
  auto draw = [&](long long mv, float Tm) {
    const uint4 r = philox_move(S.seed, chain_id, (uint64_t)mv, 0u);
    const int k = uniform_index(r.x, U.n_mov);
    Draw w;
    w.b = has_mov ? (MOV ? MOV[k] : k) : 0;
    w.dx = (2.0f * u01(r.y) - 1.0f) * U.step;
    w.dy = (2.0f * u01(r.z) - 1.0f) * U.step;
    w.dz = S.use2d ? 0.0f : (2.0f * u01(r.w) - 1.0f) * U.step;
    w.thr = ratio_threshold(u01(bead_fraction(r.x, U.n_mov)), Tm, S.inv_scale, S.inv_coef);
    w.T = Tm;
    return w;
  };
  // temperatures W moves on: T of move (last + 1 + g) from T of move `last`
  auto ahead = [&](float t_last) {
    float t = t_last;
#pragma unroll
    for (int j = 0; j < W; ++j)
      if (j <= g) t *= S.dt;
    return t;
  };
  Draw cur;
  {
    float t = S.max_temp;
#pragma unroll
    for (int j = 0; j < W - 1; ++j)
      if (j < g) t *= S.dt;
    cur = draw(g, t);
  }

  // the warp's groups step together until the last of its chains stops
  while (__any_sync(FULL, !stop)) {
    const bool run = !stop;
    const long long lim = min(min(next_ms, next_rs), U.cap);
    const int L = run ? (int)min((long long)W, lim - moves) : 0;
    const bool act = g < L;
    // the next window's draws (moves+W+g), independent of this window
    const Draw nxt = draw(moves + W + g, ahead(__shfl_sync(FULL, cur.T, gb + W - 1)));
    const int b = cur.b;
    const float dx = cur.dx, dy = cur.dy, dz = cur.dz, thr = cur.thr, Tg = cur.T;
    float4 nb = P[b];
    const float so = SO[b];
    nb.x += dx;
    nb.y += dy;
    nb.z += dz;
    const float sn = smooth_local<SPH>(P, 1, D, n, b, nb, S);
    const float d = sn - so;
    // ---- resolution ----
    unsigned accm = 0u;
    int lend = L, from = 0;
    bool open = run, hit = false;  // hit: an accepted earlier slot moved a bead this one reads
    while (__any_sync(FULL, open)) {
      const bool cand = open && act && g >= from;
      bool acc = false;
      if (cand) {
        // strict improvement (LooperSolver.hpp:4974), else the ratio test;
        // the reference kernel divides by max(E_prev, 1e-12)
        // (ParallelMonteCarloSmooth.cu:293-294)
        acc = d < 0.0f;
        if (!acc && Tg > 0.0f)
          acc = (S.gpu_sched && e_hi < 1e-12f) ? d < 1e-12f * thr - e_hi
                                               : d < e_hi * (thr - 1.0f);
      }
      const unsigned ab = (__ballot_sync(FULL, cand && acc) >> gb) & SLOTS;
      const unsigned hb = (__ballot_sync(FULL, cand && hit) >> gb) & SLOTS;
      const int ja = ab ? __ffs(ab) - 1 : W;
      const int jh = hb ? __ffs(hb) - 1 : W;
      const int src = gb + (ja < W ? ja : 0);
      const float dj = __shfl_sync(FULL, d, src);
      const int bj = __shfl_sync(FULL, b, src);
      if (open) {
        if (jh <= ja) {  // the window closes at a stale slot, or ends
          lend = jh < W ? jh : L;
          open = false;
        } else {                   // slot ja is accepted
          accm |= 1u << ja;
          ff_add(e_hi, e_lo, dj);
          if (S.gpu_sched) best = fmin(best, (double)e_hi + (double)e_lo);
          hit = hit || (g > ja && abs(b - bj) <= 2);
          from = ja + 1;
        }
      }
    }
    const bool mine = act && g < lend;
    const bool took = mine && ((accm >> g) & 1u);
    if (took) P[b] = nb;
    if (tracing && mine && moves + g < trace_cap) {
      MoveTrace tr;
      tr.bead = b;
      tr.accepted = took ? 1 : 0;
      tr.before = so;
      tr.after = sn;
      tr.dx = dx;
      tr.dy = dy;
      tr.dz = dz;
      tr.pad = d;
      trace[moves + g] = tr;
    }
    __syncwarp();  // accepted positions visible to the group
    // refresh the local scores the accepted moves changed (beads within two
    // of each): accepted slots of one window are at least three beads apart
    for (unsigned m = accm; m != 0u; m &= m - 1u) {
      const int c = __shfl_sync(gmask, b, gb + __ffs(m) - 1);
      for (int i = c - 2 + g; i <= c + 2; i += W)
        if (i >= 0 && i < n) SO[i] = smooth_local<SPH>(P, 1, D, n, i, P[i], S);
    }
    if (!run) continue;
    // the next window's slot g is move moves+lend+g: this window's lane
    // lend+g, or the lane lend+g-W of the draws made ahead
    if (lend == W) {
      cur = nxt;
    } else {
      const int src = lend + g;
      const int sl = gb + (src < W ? src : src - W);
      const bool here = src < W;
      auto pick = [&](auto a, auto z) {  // every lane of the group shuffles both
        const auto u = __shfl_sync(gmask, a, sl);
        const auto v = __shfl_sync(gmask, z, sl);
        return here ? u : v;
      };
      Draw c;
      c.b = pick(cur.b, nxt.b);
      c.dx = pick(cur.dx, nxt.dx);
      c.dy = pick(cur.dy, nxt.dy);
      c.dz = pick(cur.dz, nxt.dz);
      c.thr = pick(cur.thr, nxt.thr);
      c.T = pick(cur.T, nxt.T);
      cur = c;
    }
    const int na = __popc(accm);
    accepted += na;
    succ += na;
    moves += lend;
    if (moves == next_rs) {
      next_rs += S.resync;
      __syncwarp(gmask);
      const double Er = smooth_full_lanes<W>(P, 1, D, n, S, g, gmask);
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
    if (!stop && moves >= U.cap) stop = true;
    __syncwarp(gmask);  // refreshed local scores visible to the group
  }
  if (!live) return;
  __syncwarp(gmask);
  const double Ef = smooth_full_lanes<W>(P, 1, D, n, S, g, gmask);
  if (g == 0) {
    ChainOut o;
    o.energy = (double)e_hi + (double)e_lo;
    o.energy_fp64 = Ef;
    o.base = 0.0;
    o.best = S.gpu_sched ? best : o.energy;
    o.score = e_hi;
    o.status = status;
    o.moves = moves;
    o.accepted = accepted;
    outs[U.chain_base + chain] = o;
  }
  float *po = pos_out + U.out_off + (long long)chain * n * 3;
  for (int i = g; i < n; i += W) {
    const float4 q = P[i];
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
  {
    size_t beads = 0;
    for (int u = 0; u < n_units; ++u) beads += (size_t)std::max(0, units[u].n);
    hpos.reserve(beads);
    hdtn.reserve(beads);
  }
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
    int n_mov = pr.n;
    if (pr.fixed) {
      n_mov = 0;
      for (int i = 0; i < pr.n; ++i) n_mov += pr.fixed[i] ? 0 : 1;
    }
    U.n_mov = n_mov;
    if (n_mov < pr.n) {  // the movable beads' indices
      U.mov_off = (int)hmov.size();
      for (int i = 0; i < pr.n; ++i)
        if (!pr.fixed[i]) hmov.push_back(i);
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
  // Kernel classes: regions whose chain fits a group's shared-memory slice
  // take the windowed kernel, `window_long` slots when they have at least
  // `window_long_min_free` movable beads (the longest chains: the pass's
  // critical path) and `window_short` otherwise; a window size of 0, and a
  // region too large for a slice, take one move at a time.  Each class runs
  // on its own stream, side by side.
  // a windowed chain's shared memory per bead: position, bond target and
  // its reciprocal, local score
  constexpr size_t kWinBytes = sizeof(float4) + sizeof(float2) + sizeof(float);
  const size_t win_smem_cap = std::min<size_t>(ctx->smem_optin, 200 * 1024);
  struct WinClass {
    int W = 0;
    int slice = 0;
    std::vector<int2> items;
    DevBuf<int2> d_items;
  };
  WinClass wc[2];
  wc[0].W = ctx->smooth_window;
  wc[1].W = ctx->smooth_window_long;
  std::vector<signed char> cls(n_units, -1);
  for (int u = 0; u < n_units; ++u) {
    const SmoothUnit &U = hu[u];
    const int c = U.n_mov >= ctx->smooth_window_long_min_free ? 1 : 0;
    const int Wc = wc[c].W;
    if (Wc == 0 || (size_t)(32 / Wc) * U.n * kWinBytes > win_smem_cap) continue;
    cls[u] = (signed char)c;
    wc[c].slice = std::max(wc[c].slice, U.n);
  }
  // items: largest regions first (a warp's chains then have like move caps)
  std::vector<int> order(n_units);
  for (int u = 0; u < n_units; ++u) order[u] = u;
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
    return hu[a].n_mov != hu[b].n_mov ? hu[a].n_mov > hu[b].n_mov : hu[a].n > hu[b].n;
  });
  std::vector<int2> items;
  items.reserve((size_t)n_units * chains);
  int lane_max_n = 0;
  for (int u : order) {
    if (cls[u] < 0) lane_max_n = std::max(lane_max_n, hu[u].n);
    auto &dst = cls[u] < 0 ? items : wc[(int)cls[u]].items;
    for (int c = 0; c < chains; ++c) dst.push_back(make_int2(u, c));
  }

  const int threads = 128;
  // shared-memory slices when a chain's region fits in 1 KB
  int slice = 0;
  if (lane_max_n <= 64) slice = lane_max_n;
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
  if (e == cudaSuccess && !items.empty()) e = d_items.upload(items, s);
  for (auto &w : wc)
    if (e == cudaSuccess && !w.items.empty()) e = w.d_items.upload(w.items, s);
  if (e == cudaSuccess) e = d_pos.upload(hpos, s);
  if (e == cudaSuccess) e = d_dtn.upload(hdtn, s);
  if (e == cudaSuccess) e = d_mov.upload(hmov, s);
  if (e == cudaSuccess) e = d_out.alloc((size_t)out_off);
  if (e == cudaSuccess) e = d_outs.alloc((size_t)chain_base);
  if (e == cudaSuccess && !items.empty() && !use_smem) e = d_work.alloc((size_t)work_off);
  if (e != cudaSuccess)
    return fail(ctx, e == cudaErrorMemoryAllocation ? PMMC_ERR_NOMEM : PMMC_ERR_CUDA,
                "smooth batch upload: %s", cudaGetErrorString(e));
  // the windowed classes on the context's auxiliary streams, joined back
  for (int k = 0; k < 2; ++k) {
    if (wc[k].items.empty() || ctx->aux_stream[k]) continue;
    e = cudaStreamCreateWithFlags(&ctx->aux_stream[k], cudaStreamNonBlocking);
    if (e != cudaSuccess) {
      ctx->aux_stream[k] = nullptr;
      return fail(ctx, PMMC_ERR_CUDA, "smooth batch: %s", cudaGetErrorString(e));
    }
  }
  cudaEvent_t e0, e1, ef;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventCreateWithFlags(&ef, cudaEventDisableTiming);
  cudaEvent_t ej[2] = {nullptr, nullptr};
  MoveTrace *dtr = trace_cap > 0 ? d_trace.p : nullptr;
  cudaEventRecord(e0, s);
  cudaEventRecord(ef, s);
  for (int k : {1, 0}) {  // the long chains' CTAs first: they are the critical path
    WinClass &w = wc[k];
    if (w.items.empty()) continue;
    cudaStream_t ws = ctx->aux_stream[k];
    cudaStreamWaitEvent(ws, ef, 0);
    SmoothDevParams SW = S;
    SW.slice = w.slice;
    int wt = 128;  // 128-thread CTAs while they fit 96 KB
    while (wt > 32 && (size_t)(wt / w.W) * w.slice * kWinBytes > 96 * 1024) wt >>= 1;
    const size_t wsm = (size_t)(wt / w.W) * w.slice * kWinBytes;
    const int nw = (int)w.items.size();
    const int wgrid = (int)(((long long)nw * w.W + wt - 1) / wt);
    auto launch = [&](auto kern) {
      cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)wsm);
      kern<<<wgrid, wt, wsm, ws>>>(d_units.p, w.d_items.p, nw, d_pos.p, d_dtn.p, d_mov.p, SW,
                                  d_out.p, d_outs.p, dtr, trace_cap);
    };
    // no container: the sphere term is left out of the kernel (it is 0)
    const bool sph = S.R > 0.0f;
    if (w.W == 4) sph ? launch(smooth_window_kernel<4, true>) : launch(smooth_window_kernel<4, false>);
    else if (w.W == 8) sph ? launch(smooth_window_kernel<8, true>) : launch(smooth_window_kernel<8, false>);
    else if (w.W == 16) sph ? launch(smooth_window_kernel<16, true>) : launch(smooth_window_kernel<16, false>);
    else sph ? launch(smooth_window_kernel<32, true>) : launch(smooth_window_kernel<32, false>);
    cudaEventCreateWithFlags(&ej[k], cudaEventDisableTiming);
    cudaEventRecord(ej[k], ws);
  }
  const int n_items = (int)items.size();
  if (n_items > 0) {
    S.slice = slice;
    const int grid = (int)(((long long)n_items * kSmoothLanes + threads - 1) / threads);
    if (use_smem) {
      cudaFuncSetAttribute(smooth_anneal_kernel<true>,
                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      smooth_anneal_kernel<true><<<grid, threads, smem, s>>>(
          d_units.p, d_items.p, n_items, d_pos.p, d_dtn.p, d_mov.p, S, nullptr, d_out.p,
          d_outs.p, dtr, trace_cap);
    } else {
      smooth_anneal_kernel<false><<<grid, threads, 0, s>>>(
          d_units.p, d_items.p, n_items, d_pos.p, d_dtn.p, d_mov.p, S, d_work.p, d_out.p,
          d_outs.p, dtr, trace_cap);
    }
  }
  e = cudaGetLastError();
  for (int k = 0; k < 2; ++k)
    if (ej[k]) cudaStreamWaitEvent(s, ej[k], 0);
  cudaEventRecord(e1, s);
  if (e == cudaSuccess) e = cudaEventSynchronize(e1);
  if (e == cudaSuccess && kernel_ms) {
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    *kernel_ms = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaEventDestroy(ef);
  for (int k = 0; k < 2; ++k)
    if (ej[k]) cudaEventDestroy(ej[k]);
  if (e != cudaSuccess)
    return fail(ctx, PMMC_ERR_CUDA, "smooth kernel: %s", cudaGetErrorString(e));

  std::vector<ChainOut> outs(chain_base);
  PMMC_CUDA(ctx, cudaMemcpy(outs.data(), d_outs.p, sizeof(ChainOut) * outs.size(),
                            cudaMemcpyDeviceToHost));
  if (trace_out && trace_cap > 0)
    PMMC_CUDA(ctx, cudaMemcpy(trace_out, d_trace.p, sizeof(MoveTrace) * trace_cap,
                              cudaMemcpyDeviceToHost));
  // every chain's positions in one copy (one per region was a round trip
  // each); with one chain per region the device layout is the caller's
  const bool direct = chains == 1;
  std::vector<float> hout;
  if (pos_out && direct) {
    PMMC_CUDA(ctx, cudaMemcpy(pos_out, d_out.p, sizeof(float) * (size_t)out_off,
                              cudaMemcpyDeviceToHost));
  } else if (pos_out) {
    hout.resize((size_t)out_off);
    PMMC_CUDA(ctx, cudaMemcpy(hout.data(), d_out.p, sizeof(float) * hout.size(),
                              cudaMemcpyDeviceToHost));
  }
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
      if (!direct)
        std::copy_n(hout.data() + U.out_off + (long long)best * U.n * 3, (size_t)U.n * 3,
                    pos_out + dst);
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

// Regions packed back to back: region u is beads [bead_off[u], bead_off[u+1])
// of the packed arrays.
extern "C" pmmc_status pmmc_smooth_batch_anneal_packed(
    pmmc_ctx *ctx, int n_units, const int64_t *bead_off, const float *pos,
    const float *dist_to_next, const unsigned char *fixed, const pmmc_anneal_params *prm,
    const float *step_sizes, int chains, float *pos_out, pmmc_result *res, double *kernel_ms,
    void *trace_out, int trace_cap) {
  if (!ctx || n_units < 1 || !bead_off || !pos || !dist_to_next)
    return fail(ctx, PMMC_ERR_INVALID, "smooth packed batch: bad arguments");
  std::vector<pmmc_smooth_problem> v((size_t)n_units);
  for (int u = 0; u < n_units; ++u) {
    const int64_t a = bead_off[u], b = bead_off[u + 1];
    if (a < 0 || b < a || b - a > (int64_t)INT32_MAX)
      return fail(ctx, PMMC_ERR_INVALID, "smooth packed batch: region %d spans [%lld, %lld)", u,
                  (long long)a, (long long)b);
    v[u].n = (int)(b - a);
    v[u].pos = pos + 3 * a;
    v[u].fixed = fixed ? fixed + a : nullptr;
    v[u].dist_to_next = dist_to_next + a;
  }
  return pmmc_smooth_batch_anneal(ctx, n_units, v.data(), prm, step_sizes, chains, pos_out, res,
                                  kernel_ms, trace_out, trace_cap);
}

extern "C" pmmc_status pmmc_smooth_set_window(pmmc_ctx *ctx, int window_short, int window_long,
                                              int long_min_free) {
  if (!ctx) return PMMC_ERR_INVALID;
  for (int w : {window_short, window_long})
    if (w != 0 && w != 4 && w != 8 && w != 16 && w != 32)
      return fail(ctx, PMMC_ERR_INVALID, "smooth window: %d slots (0, 4, 8, 16 or 32)", w);
  if (long_min_free < 0)
    return fail(ctx, PMMC_ERR_INVALID, "smooth window: long_min_free %d < 0", long_min_free);
  ctx->smooth_window = window_short;
  ctx->smooth_window_long = window_long;
  ctx->smooth_window_long_min_free = long_min_free;
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
