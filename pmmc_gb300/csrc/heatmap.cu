// heatmap.cu -- heatmap-level (chromosome / segment) simulated annealing.
//
// Score (LooperSolver.hpp:3583-3617): for every bead m, the sum over beads i
// of its chromosome block with |i - m| >= diag and h_im >= 1e-6 of
// ((|p_i - p_m| - h_im) / h_im)^2; the full score sums the local scores of
// all beads, so every pair counts twice and a move of bead m changes the full
// score by 2 * (local_after - local_before) (the matrices createDistanceHeatmap
// builds are symmetric, :3042-3085).  The reference CPU annealer re-scores all
// N^2 pairs after every move (:1488); here a move reads one row.
//
// One CTA runs one chain.  Positions (float4) live in shared memory.  The row
// of the bead a move displaces is streamed from HBM into a ring of D
// shared-memory slots with cp.async.bulk (TMA bulk copy, completion counted
// on an mbarrier per slot); because the Philox stream is counter-based the
// beads of future moves are known, so the copy for move k+D is issued while
// move k is scored.  Each thread scores a strided slice of the row, a warp
// shuffle plus one barrier reduces the partial sums, and every warp takes the
// (identical) Metropolis decision itself, so one __syncthreads per move
// suffices; the running score is a float-float pair in every thread.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace pmmc {

struct HeatUnit {
  int n;
  int n_mov;
  int pos_off;
  int mov_off;       // -1: all movable
  long long heat_off;  // float index of row 0
  int pitch;         // floats per row (multiple of 4)
  int diag;
  int blk_off;       // int2 [n]: chromosome block [st, en] of each bead
  int chain_id;
  long long out_off;
  float step;
  int pad;
};

struct HeatDevParams {
  float max_temp;
  float inv_scale;
  float inv_coef;
  float improvement;
  float R;
  int min_succ;
  int window;
  int fails;
  int use2d;
  int depth;        // TMA ring slots
  int trace_cap;
  int pad;
  long long cap;
  uint64_t seed;
  double dtpow[33];
};

constexpr int kHeatMaxThreads = 512;
constexpr long long kSpinLimit = 1ll << 26;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}

// Bounded wait on an mbarrier phase; returns false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  for (long long it = 0; it < kSpinLimit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

__device__ __forceinline__ void tma_row(void *dst, const void *src, uint32_t bytes,
                                        uint64_t *bar) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  mbar_expect_tx(bar, bytes);
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
          smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
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

struct MoveRec {
  int b;
  float dx, dy, dz;
};

__device__ __forceinline__ float hm_term(float4 a, float4 b, float h) {
  const float x = a.x - b.x, y = a.y - b.y, z = a.z - b.z;
  const float c = (sqrtf(x * x + y * y + z * z) - h) / h;
  return c * c;
}

// Change of one pair term when bead b moves from pb to nb: the hardware
// reciprocal square root and one reciprocal of h shared by both terms.
__device__ __forceinline__ float hm_delta(float4 pi, float4 pb, float4 nb, float h) {
  const float rh = __frcp_rn(h);
  const float co =
      (ref_len(__fsub_rn(pi.x, pb.x), __fsub_rn(pi.y, pb.y), __fsub_rn(pi.z, pb.z)) - h) * rh;
  const float cn =
      (ref_len(__fsub_rn(pi.x, nb.x), __fsub_rn(pi.y, nb.y), __fsub_rn(pi.z, nb.z)) - h) * rh;
  return cn * cn - co * co;
}

// FP64 full score plus the sphere penalties of all beads (the reference adds
// the boundary sum to the initial score, LooperSolver.hpp:1451-1457); the
// whole block, every thread returns the total.
__device__ double heat_full(const HeatUnit &U, const float4 *spos, const float *heat,
                            const int2 *blk, double *red, float R) {
  double acc = 0.0;
  for (int i = threadIdx.x; i < U.n; i += blockDim.x)
    acc += sphere_penalty(spos[i].x, spos[i].y, spos[i].z, R);
  for (int m = 0; m < U.n; ++m) {
    const int2 r = blk[m];
    const float *row = heat + U.heat_off + (long long)m * U.pitch;
    const float4 pm = spos[m];
    float part = 0.0f;
    for (int i = r.x + threadIdx.x; i <= r.y; i += blockDim.x) {
      if (abs(i - m) < U.diag || i == m) continue;
      const float h = row[i];
      if (h < 1e-6f) continue;
      part += hm_term(spos[i], pm, h);
    }
    acc += part;
  }
  acc = warp_sum_d(acc);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
  __syncthreads();
  return t;
}

__global__ void __launch_bounds__(kHeatMaxThreads, 1)
heatmap_anneal_kernel(const HeatUnit *__restrict__ units, const float4 *__restrict__ pos0,
                      const float *__restrict__ heat, const int *__restrict__ movable,
                      const int2 *__restrict__ blk_all, HeatDevParams P,
                      float *__restrict__ pos_out, ChainOut *__restrict__ outs,
                      MoveTrace *__restrict__ trace) {
  extern __shared__ __align__(128) unsigned char smem[];
  const HeatUnit U = units[blockIdx.x];
  const int n = U.n;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nthr = blockDim.x, nwarps = nthr >> 5;
  const int D = P.depth;
  // ---- shared-memory carve ----
  unsigned char *p = smem;
  uint64_t *bars = reinterpret_cast<uint64_t *>(p);
  p += 16 * 8;
  double *red = reinterpret_cast<double *>(p);
  p += 32 * 8;
  float *partial = reinterpret_cast<float *>(p);  // [2][kHeatWarps]
  p += 2 * 32 * 4;
  int *tflag = reinterpret_cast<int *>(p);        // [2][kHeatWarps] wait timed out
  p += 2 * 32 * 4;
  MoveRec *recs = reinterpret_cast<MoveRec *>(p); // ring of 64
  p += 64 * sizeof(MoveRec);
  float *thrs = reinterpret_cast<float *>(p);     // ring of 64
  p += 64 * 4;
  p = smem + (((p - smem) + 127) & ~(size_t)127);
  float *slots = reinterpret_cast<float *>(p);    // D * pitch floats
  p += (size_t)D * U.pitch * 4;
  float4 *spos = reinterpret_cast<float4 *>(p);
  p += (size_t)n * 16;
  // per-bead chromosome block and the movable list, read on every move's
  // critical path: staged next to the positions
  int2 *blk = reinterpret_cast<int2 *>(p);
  p += (size_t)n * 8;
  int *smov = reinterpret_cast<int *>(p);

  const int *MOV = U.mov_off >= 0 ? smov : nullptr;
  const float *hrow0 = heat + U.heat_off;

  if (tid == 0) {
    for (int s = 0; s < D; ++s) mbar_init(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int i = tid; i < n; i += blockDim.x) {
    spos[i] = pos0[U.pos_off + i];
    blk[i] = blk_all[U.blk_off + i];
  }
  if (U.mov_off >= 0)
    for (int k = tid; k < U.n_mov; k += blockDim.x) smov[k] = movable[U.mov_off + k];
  __syncthreads();

  const double E0 = heat_full(U, spos, heat, blk, red, P.R);
  double T = P.max_temp;  // temperature of the next batch's first move (warp 0)

  // draws of one batch of 32 moves (warp 0)
  auto fill = [&](long long first) {
    const uint64_t m = (uint64_t)(first + lane);
    const uint4 r = philox_move(P.seed, (uint32_t)U.chain_id, m, 0u);
    const uint4 a = philox_move(P.seed, (uint32_t)U.chain_id, m, 1u);
    const int k = uniform_index(r.x, U.n_mov);
    MoveRec rec;
    rec.b = MOV ? MOV[k] : k;
    rec.dx = (2.0f * u01(r.y) - 1.0f) * U.step;
    rec.dy = (2.0f * u01(r.z) - 1.0f) * U.step;
    rec.dz = P.use2d ? 0.0f : (2.0f * u01(r.w) - 1.0f) * U.step;
    const float Tl = (float)(T * P.dtpow[lane]);
    const int slot = (int)(m & 63);
    recs[slot] = rec;
    thrs[slot] = ratio_threshold(u01(a.x), Tl, P.inv_scale, P.inv_coef);
    T *= P.dtpow[32];
  };
  // row range [st_al, st_al + len) of bead b, 16-byte aligned
  auto row_range = [&](int b, int &st_al, int &len) {
    const int2 r = blk[b];
    st_al = r.x & ~3;
    int en = (r.y + 4) & ~3;
    if (en > U.pitch) en = U.pitch;
    len = en - st_al;
  };

  const bool run = U.n_mov > 0 && E0 >= 1e-6 && E0 == E0;
  long long cap = run ? P.cap : 0;
  long long issued = 0;  // moves whose rows were requested (thread 0)
  if (warp == 0 && cap > 0) {
    fill(0);
    fill(32);
    __syncwarp();
    if (lane == 0) {
      const long long first = std::min((long long)D, cap);
      for (long long k = 0; k < first; ++k) {
        int st, len;
        row_range(recs[k & 63].b, st, len);
        tma_row(slots + (size_t)(k % D) * U.pitch, hrow0 + (long long)recs[k & 63].b * U.pitch + st,
                (uint32_t)len * 4, &bars[k % D]);
      }
      issued = first;
    }
  }
  __syncthreads();

  float e_hi = (float)E0, e_lo = (float)(E0 - (double)(float)E0);
  double E_ms = E0;
  int succ = 0, misses = 0, status = kDevOk;
  long long moves = 0, accepted = 0;
  int prev_b = -1;
  bool prev_acc = false;
  float4 prev_new = make_float4(0.f, 0.f, 0.f, 0.f);
  bool stop = cap == 0;

  while (!stop) {
    const long long k = moves;
    const MoveRec rec = recs[k & 63];
    const float thr = thrs[k & 63];
    const int b = rec.b;
    const int slot = (int)(k % D);
    const bool timed_out = !mbar_wait(&bars[slot], (uint32_t)((k / D) & 1));
    const float4 pb = (b == prev_b && prev_acc) ? prev_new : spos[b];
    const float4 nb = make_float4(pb.x + rec.dx, pb.y + rec.dy, pb.z + rec.dz, 0.0f);
    int st, len;
    row_range(b, st, len);
    const int2 r = blk[b];
    const float *row = slots + (size_t)slot * U.pitch - st;
    float part = 0.0f;
    for (int i = r.x + tid; i <= r.y; i += nthr) {
      if (abs(i - b) < U.diag || i == b) continue;
      const float h = row[i];
      if (h < 1e-6f) continue;
      const float4 pi = (i == prev_b && prev_acc) ? prev_new : spos[i];
      part += hm_delta(pi, pb, nb, h);
    }
    part = warp_sum_f(part);
    const int any_to = __any_sync(0xffffffffu, timed_out) ? 1 : 0;
    if (lane == 0) {
      partial[(k & 1) * 32 + warp] = part;
      tflag[(k & 1) * 32 + warp] = any_to;
    }
    __syncthreads();
    // every thread sees the same timeout flags (double-buffered by parity)
    const bool block_to =
        __any_sync(0xffffffffu, lane < nwarps && tflag[(k & 1) * 32 + lane] != 0);
    // refill the draws of moves k+32..k+63 (their ring slots held moves
    // k-32..k-1) and issue the copy for move k + D (slot k % D is free)
    if (warp == 0) {
      if ((k & 31) == 0 && k > 0) fill(k + 32);
      __syncwarp();
      if (lane == 0 && issued < cap && issued == k + D) {
        const MoveRec rn = recs[issued & 63];
        int s2, l2;
        row_range(rn.b, s2, l2);
        tma_row(slots + (size_t)(issued % D) * U.pitch, hrow0 + (long long)rn.b * U.pitch + s2,
                (uint32_t)l2 * 4, &bars[issued % D]);
        ++issued;
      }
    }
    // every warp reduces the partials in the same order: identical decisions
    float tot = lane < nwarps ? partial[(k & 1) * 32 + lane] : 0.0f;
    tot = warp_sum_f(tot);
    const float d = 2.0f * tot + (sphere_penalty(nb.x, nb.y, nb.z, P.R) -
                                  sphere_penalty(pb.x, pb.y, pb.z, P.R));
    const bool acc = (d <= 0.0f) || (d < e_hi * (thr - 1.0f));
    if (acc) {
      ff_add(e_hi, e_lo, d);
      ++accepted;
      ++succ;
      if (tid == 0) spos[b] = nb;  // visible to all after the next barrier
    }
    if (tid == 0 && trace != nullptr && U.chain_id == 0 && k < P.trace_cap) {
      MoveTrace tr;
      tr.bead = b;
      tr.accepted = acc ? 1 : 0;
      tr.before = 0.0f;
      tr.after = 2.0f * tot;
      tr.dx = rec.dx;
      tr.dy = rec.dy;
      tr.dz = rec.dz;
      tr.pad = d;
      trace[k] = tr;
    }
    prev_b = b;
    prev_acc = acc;
    prev_new = nb;
    moves = k + 1;
    if (moves % P.window == 0) {
      // LooperSolver.hpp:1543-1548 (FP64)
      const double E = (double)e_hi + (double)e_lo;
      const bool miss = (E > (double)P.improvement * E_ms && succ < P.min_succ) || E < 1e-6;
      misses = miss ? misses + 1 : 0;
      if (misses >= P.fails || E < 1e-6) stop = true;
      E_ms = E;
      succ = 0;
    }
    if (moves >= cap) stop = true;
    if (block_to) {  // a row copy never arrived: give up on this chain
      stop = true;
      status = PMMC_ERR_TIMEOUT;
    }
  }
  __syncthreads();
  // drain copies still in flight (rows prefetched past the last move)
  if (tid == 0) {
    for (long long k = moves; k < issued; ++k)
      if (!mbar_wait(&bars[k % D], (uint32_t)((k / D) & 1))) status = PMMC_ERR_TIMEOUT;
  }
  __syncthreads();
  const double Efin = heat_full(U, spos, heat, blk, red, P.R);
  if (tid == 0) {
    ChainOut o;
    const double E = run ? (double)e_hi + (double)e_lo : 0.0;
    o.energy = E;
    o.energy_fp64 = run ? Efin : 0.0;
    o.base = 0.0;
    o.score = (float)E;
    o.status = status;
    o.moves = moves;
    o.accepted = accepted;
    outs[blockIdx.x] = o;
  }
  float *po = pos_out + U.out_off;
  for (int i = tid; i < n; i += blockDim.x) {
    const float4 q = spos[i];
    po[3 * i] = q.x;
    po[3 * i + 1] = q.y;
    po[3 * i + 2] = q.z;
  }
}

}  // namespace pmmc

using namespace pmmc;

namespace {

// getChromosomeHeatmapBoundary (LooperSolver.hpp:6034-6050): beads beyond
// the last boundary, or in no block, keep the whole range.
void bead_blocks(int n, int nb, const int *b, std::vector<int2> &out) {
  for (int p = 0; p < n; ++p) {
    int st = 0, en = n - 1;
    if (nb > 0 && !(p < 0 || p > b[nb - 1])) {
      for (int i = 0; i + 1 < nb; ++i)
        if (b[i] <= p && p < b[i + 1]) {
          st = b[i];
          en = b[i + 1] - 1;
          break;
        }
    }
    st = std::max(st, 0);
    en = std::min(en, n - 1);
    out.push_back(make_int2(st, en));
  }
}

}  // namespace

extern "C" pmmc_status pmmc_heatmap_batch_anneal(pmmc_ctx *ctx, int n_units,
                                                const pmmc_heatmap_problem *units,
                                                const pmmc_anneal_params *prm,
                                                const float *steps, float *pos_out,
                                                pmmc_result *res, double *kernel_ms,
                                                void *trace_out, int trace_cap) {
  if (!ctx || n_units < 1 || !units || !prm || !steps)
    return fail(ctx, PMMC_ERR_INVALID, "heatmap batch: bad arguments");
  std::vector<HeatUnit> hu(n_units);
  std::vector<float4> hpos;
  std::vector<int> hmov;
  std::vector<int2> hblk;
  long long heat_floats = 0, out_off = 0;
  int max_n = 0, max_pitch = 0;
  for (int u = 0; u < n_units; ++u) {
    const pmmc_heatmap_problem &pr = units[u];
    if (pr.n < 2 || !pr.pos || !pr.heat || pr.diag < 0 || pr.n_bounds < 0 ||
        (pr.n_bounds > 0 && !pr.bounds))
      return fail(ctx, PMMC_ERR_INVALID, "heatmap region %d: bad sizes", u);
    HeatUnit U{};
    U.n = pr.n;
    U.pitch = (pr.n + 3) & ~3;
    U.diag = pr.diag;
    U.pos_off = (int)hpos.size();
    for (int i = 0; i < pr.n; ++i)
      hpos.push_back(make_float4(pr.pos[3 * i], pr.pos[3 * i + 1], pr.pos[3 * i + 2], 0.0f));
    std::vector<int> mv;
    for (int i = 0; i < pr.n; ++i)
      if (!pr.fixed || !pr.fixed[i]) mv.push_back(i);
    U.n_mov = (int)mv.size();
    U.mov_off = U.n_mov < pr.n ? (int)hmov.size() : -1;
    if (U.n_mov < pr.n) hmov.insert(hmov.end(), mv.begin(), mv.end());
    U.blk_off = (int)hblk.size();
    bead_blocks(pr.n, pr.n_bounds, pr.bounds, hblk);
    U.heat_off = heat_floats;
    heat_floats += (long long)U.pitch * pr.n;
    U.chain_id = u;
    U.out_off = out_off;
    out_off += (long long)pr.n * 3;
    U.step = steps[u] * 0.5f;  // MonteCarloHeatmap halves the step (:1426)
    max_n = std::max(max_n, pr.n);
    max_pitch = std::max(max_pitch, U.pitch);
    hu[u] = U;
  }
  if (hmov.empty()) hmov.push_back(0);

  HeatDevParams P{};
  P.max_temp = prm->max_temp;
  P.inv_scale = prm->jump_scale != 0.0f ? 1.0f / prm->jump_scale : 0.0f;
  P.inv_coef = prm->jump_coef != 0.0f ? 1.0f / prm->jump_coef : 0.0f;
  P.improvement = prm->improvement;
  P.R = prm->sphere_radius;
  P.min_succ = prm->min_successes;
  P.use2d = prm->use2d;
  P.seed = next_key(ctx);
  P.trace_cap = trace_cap;
  // the reference CPU schedule; milestone_fails > 1 only with PMMC_SCHEDULE_GPU
  P.window = std::max(1, prm->milestone_steps);
  P.fails = prm->schedule == PMMC_SCHEDULE_GPU ? std::max(1, prm->milestone_fails) : 1;
  P.cap = prm->max_moves > 0 ? prm->max_moves : 200ll * P.window;
  double dp = 1.0;
  for (int l = 0; l <= 32; ++l) {
    P.dtpow[l] = dp;
    dp *= (double)prm->dt_temp;
  }
  // shared memory: header + D row slots + positions
  const size_t head = 4096;
  const size_t pos_bytes = (size_t)max_n * (16 + 8 + 4);  // positions, blocks, movable
  const size_t row_bytes = (size_t)max_pitch * 4;
  const size_t avail = ctx->smem_optin;
  if (head + pos_bytes + 2 * row_bytes > avail)
    return fail(ctx, PMMC_ERR_INVALID, "heatmap region of %d beads does not fit shared memory", max_n);
  int depth = (int)std::min<size_t>(16, (avail - head - pos_bytes) / row_bytes);
  depth = std::max(2, depth);
  P.depth = depth;
  const size_t smem = head + (size_t)depth * row_bytes + pos_bytes;

  cudaStream_t s = ctx->stream;
  // the heatmaps, rows padded to a 16-byte pitch
  std::vector<float> hheat((size_t)heat_floats, 0.0f);
  for (int u = 0; u < n_units; ++u) {
    const HeatUnit &U = hu[u];
    const pmmc_heatmap_problem &pr = units[u];
    for (int i = 0; i < pr.n; ++i)
      memcpy(&hheat[(size_t)U.heat_off + (size_t)i * U.pitch], pr.heat + (size_t)i * pr.n,
             sizeof(float) * pr.n);
  }
  DevBuf<HeatUnit> d_units;
  DevBuf<float4> d_pos;
  DevBuf<float> d_heat, d_out;
  DevBuf<int> d_mov;
  DevBuf<int2> d_blk;
  DevBuf<ChainOut> d_outs;
  DevBuf<MoveTrace> d_trace;
  cudaError_t e = d_units.upload(hu, s);
  if (e == cudaSuccess) e = d_pos.upload(hpos, s);
  if (e == cudaSuccess) e = d_heat.upload(hheat, s);
  if (e == cudaSuccess) e = d_mov.upload(hmov, s);
  if (e == cudaSuccess) e = d_blk.upload(hblk, s);
  if (e == cudaSuccess) e = d_out.alloc((size_t)out_off);
  if (e == cudaSuccess) e = d_outs.alloc((size_t)n_units);
  if (e == cudaSuccess && trace_cap > 0) e = d_trace.alloc((size_t)trace_cap);
  if (e != cudaSuccess)
    return fail(ctx, e == cudaErrorMemoryAllocation ? PMMC_ERR_NOMEM : PMMC_ERR_CUDA,
                "heatmap upload: %s", cudaGetErrorString(e));
  PMMC_CUDA(ctx, cudaFuncSetAttribute(heatmap_anneal_kernel,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  // threads per chain: about four row entries per thread, 128..512
  int threads = 128;
  while (threads < kHeatMaxThreads && threads * 4 < max_n) threads *= 2;
  heatmap_anneal_kernel<<<n_units, threads, smem, s>>>(
      d_units.p, d_pos.p, d_heat.p, d_mov.p, d_blk.p, P, d_out.p, d_outs.p,
      trace_cap > 0 ? d_trace.p : nullptr);
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
  if (e != cudaSuccess) return fail(ctx, PMMC_ERR_CUDA, "heatmap kernel: %s", cudaGetErrorString(e));
  std::vector<ChainOut> outs(n_units);
  PMMC_CUDA(ctx, cudaMemcpy(outs.data(), d_outs.p, sizeof(ChainOut) * n_units,
                            cudaMemcpyDeviceToHost));
  if (pos_out)
    PMMC_CUDA(ctx, cudaMemcpy(pos_out, d_out.p, sizeof(float) * out_off, cudaMemcpyDeviceToHost));
  if (trace_out && trace_cap > 0)
    PMMC_CUDA(ctx, cudaMemcpy(trace_out, d_trace.p, sizeof(MoveTrace) * trace_cap,
                              cudaMemcpyDeviceToHost));
  for (int u = 0; u < n_units; ++u) {
    const ChainOut &o = outs[u];
    if (res) {
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
      res[u] = r;
    }
  }
  for (auto &o : outs)
    if (o.status == PMMC_ERR_TIMEOUT)
      return fail(ctx, PMMC_ERR_TIMEOUT, "heatmap: a row copy did not complete");
  return PMMC_OK;
}

extern "C" pmmc_status pmmc_heatmap_anneal(pmmc_ctx *ctx, const pmmc_heatmap_problem *pr,
                                           const pmmc_anneal_params *prm, float step_size,
                                           float *pos_out, pmmc_result *res) {
  return pmmc_heatmap_batch_anneal(ctx, 1, pr, prm, &step_size, pos_out, res, nullptr,
                                   nullptr, 0);
}
