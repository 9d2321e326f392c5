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
// One CTA runs one chain.  Positions (float4) live in shared memory.  The
// device matrix holds r = 1/h, zero wherever the reference skips the pair
// (h < 1e-6, the diagonal band, another chromosome block), so a pair term is
// branch-free and needs no division.  The row of the bead a move displaces is
// streamed from HBM into a ring of D shared-memory slots with cp.async.bulk
// (TMA bulk copy, completion counted on an mbarrier per slot); because the
// Philox stream is counter-based the beads of future moves are known, so rows
// are requested a window or more before they are scored.
//
// Moves are scored in windows of up to 8: every thread takes a slice of the
// beads and accumulates the change of all 8 moves at once against the
// window-start positions; the 8 sums are reduced with warp shuffles and one
// barrier, warp 0 takes the Metropolis decisions in move order (adding, for a
// move after an accepted one, the exact change of the pair between the two
// moved beads), and warp 1 meanwhile draws future moves and requests their
// rows.  A window never holds the same bead twice and ends at milestones, so
// the accepted sequence is the one-move-at-a-time sequence.  The running score
// is a float-float pair; the start and end scores are FP64 recomputes.
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
  int single;        // 1: one chromosome block (every bead's block is [0, n-1])
  int slice;         // cluster mode: beads per CTA (a multiple of 4)
  int pad_;
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
// A row copy that has not landed after this long is reported as a timeout.
constexpr unsigned long long kWaitLimitNs = 2000000000ull;

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

// Bounded wait on an mbarrier phase; returns false when the time limit ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  const uint32_t a = smem_u32(bar);
  unsigned long long t0 = 0;
  for (unsigned it = 0;; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(a), "r"(parity)
        : "memory");
    if (ok) return true;
    if ((it & 255u) == 0u) {
      const unsigned long long t = globaltimer_ns();
      if (it == 0u) t0 = t;
      else if (t - t0 > kWaitLimitNs) return false;
    }
  }
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

// Thread-block cluster: this CTA's rank, the cluster-wide barrier (every
// thread of every CTA of the cluster), and stores into another CTA's shared
// memory at the address of the same variable there.
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
  return r;
}

__device__ __forceinline__ void cluster_sync() {
  asm volatile("barrier.cluster.arrive.release;\n"
               "barrier.cluster.wait.acquire;" ::: "memory");
}

__device__ __forceinline__ uint32_t cluster_addr(const void *p, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(smem_u32(p)), "r"(rank));
  return r;
}

__device__ __forceinline__ void st_cluster(uint32_t a, float v) {
  asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}
__device__ __forceinline__ void st_cluster(uint32_t a, uint32_t v) {
  asm volatile("st.shared::cluster.u32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
__device__ __forceinline__ void st_cluster(uint32_t a, int v) { st_cluster(a, (uint32_t)v); }
__device__ __forceinline__ void st_cluster(uint32_t a, double v) {
  asm volatile("st.shared::cluster.f64 [%0], %1;" ::"r"(a), "d"(v) : "memory");
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

// Approximate reciprocal square root (one special-function operation,
// flush-to-zero; callers keep the argument normal).
__device__ __forceinline__ float rsqrt_approx(float s) {
  float r;
  asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(s));
  return r;
}

// |v| from |v|^2 with one reciprocal square root; |v|^2 is clamped to 1e-30
// so coincident beads give ~1e-15 instead of 0 * inf.
__device__ __forceinline__ float len_from_sq(float s) {
  s = fmaxf(s, 1e-30f);
  return s * rsqrt_approx(s);
}

// A proposed move: old position, -2 * displacement and |displacement|^2.
struct MoveGeo {
  float ox, oy, oz;
  float mx, my, mz;
  float dd;
};

// Change of the pair term (d r - 1)^2 (r = 1/h) between a bead at p and a
// bead that moves from o to o + delta.  With v = p - o, s_o = |v|^2 and
// t = s_n - s_o = |delta|^2 - 2 v.delta (formed directly, no cancellation):
//   (d_n r - 1)^2 - (d_o r - 1)^2 = r (r t - 2 (d_n - d_o)).
// Two special-function operations per pair (one reciprocal square root per
// length); the difference d_n - d_o costs about one ulp of d, a relative
// error of the move's local change below 1e-8.  r = 0 (no target, inside the
// diagonal band, the bead itself, another chromosome block) contributes
// exactly 0.
__device__ __forceinline__ float pair_delta(float px, float py, float pz, const MoveGeo &g,
                                            float r) {
  const float vx = px - g.ox, vy = py - g.oy, vz = pz - g.oz;
  const float so = fmaf(vx, vx, fmaf(vy, vy, vz * vz));
  const float t = fmaf(vx, g.mx, fmaf(vy, g.my, fmaf(vz, g.mz, g.dd)));
  const float dd = len_from_sq(so + t) - len_from_sq(so);
  return r * fmaf(r, t, -2.0f * dd);
}

// Full score in FP64 (FP32 terms (d r - 1)^2 summed per row, rows summed in
// FP64) plus the sphere penalties of all beads -- of rows and beads [m0, m1) (the reference adds the
// boundary sum to the initial score, LooperSolver.hpp:1451-1457).  One warp
// per row of the reciprocal targets (zero outside the bead's block, in the
// diagonal band and where h < 1e-6); lane l takes beads i = l mod 32, so the
// row loads coalesce and the position reads hit 32 distinct banks; a lane
// issues kB loads before it computes.  The whole block calls it and every
// thread returns the total.
__device__ double heat_full(const HeatUnit &U, const float4 *spos, const float *rheat,
                            const int2 *blk, double *red, float R, int m0, int m1) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  constexpr int kB = 32;
  double acc = 0.0;
  for (int i = m0 + threadIdx.x; i < m1; i += blockDim.x)
    acc += sphere_penalty(spos[i].x, spos[i].y, spos[i].z, R);
  for (int m = m0 + warp; m < m1; m += nw) {
    const int2 r = U.single ? make_int2(0, U.n - 1) : blk[m];
    const float *row = rheat + U.heat_off + (long long)m * U.pitch;
    const float4 pm = spos[m];
    float part = 0.0f;
    for (int i0 = r.x; i0 <= r.y; i0 += 32 * kB) {
      float rv[kB];
#pragma unroll
      for (int k = 0; k < kB; ++k) {
        const int i = i0 + lane + 32 * k;
        rv[k] = i <= r.y ? __ldg(row + i) : 0.0f;
      }
#pragma unroll
      for (int k = 0; k < kB; ++k) {
        if (rv[k] > 0.0f) {  // a nonzero entry lies inside the row's block
          const float4 pi = spos[i0 + lane + 32 * k];
          const float x = pi.x - pm.x, y = pi.y - pm.y, z = pi.z - pm.z;
          const float f = fmaf(len_from_sq(fmaf(x, x, fmaf(y, y, z * z))), rv[k], -1.0f);
          part = fmaf(f, f, part);
        }
      }
    }
    acc += (double)part;
  }
  acc = warp_sum_d(acc);
  __syncthreads();
  if (lane == 0) red[warp] = acc;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < nw; ++w) t += red[w];
  __syncthreads();
  return t;
}

constexpr int kWin = 8;  // moves scored per CTA step

// What warp 0 publishes between windows.
struct WinPlan {
  float4 ga[kWin];  // old position, |delta|^2
  float4 gb[kWin];  // -2 delta, row offset of the move's slot (int bits)
  int bw[kWin];     // moved beads
  unsigned accm;    // accepted moves of the window just resolved (bit w)
  int lend;         // moves in the window just resolved
  float pacc;       // sum of its accepted energy changes
  int len;          // moves in the next window
  int same;         // every move of the next window in one chromosome block
  int timeout;      // a row copy of the next window never landed
  int pad[2];
};

// Bytes of the kernel's shared-memory header (barriers, reduction scratch,
// partial sums, pair corrections, window plan, draw ring), as carved below.
constexpr size_t kHeadBytes =
    ((((16 * 8 + 32 * 8 + 16 * kWin * 4 + kWin * kWin * 4 + sizeof(WinPlan)) + 15) / 16 * 16 +
      128 * sizeof(MoveRec) + 128 * 4) + 127) / 128 * 128;

// Exact in-order windows: every thread scores its slice of the rows of up to
// kWin moves against the window-start positions; pair corrections restore the
// terms between two beads of the same window once the earlier one has been
// accepted, and warp 0 takes the Metropolis decisions in move order.  The
// window ends early before a bead that already moves earlier in it, at a
// milestone and at the move cap, so the decisions are those of one move at a
// time.  Two CTA barriers per window; warp 0 does the serial work between
// them (decisions, draws, row copies, the next window's plan and row waits).
// CL > 1 (cluster mode): one chain on a cluster of CL CTAs.  CTA r scores
// beads [r S, r S + S) of every row (S = U.slice), streams only that slice of
// each row and keeps all positions; the CTAs send their sums and pair
// corrections to CTA 0, which takes the decisions and sends them back; every
// CTA then applies them and plans the next window alike (the draws are the
// same everywhere), so all CTAs run the same windows and meet the same two
// cluster barriers per window.
template <int CL>
__global__ void __launch_bounds__(kHeatMaxThreads, 1)
heatmap_anneal_kernel(const HeatUnit *__restrict__ units, const float4 *__restrict__ pos0,
                      const float *__restrict__ rheat, const int *__restrict__ movable,
                      const int2 *__restrict__ blk_all, HeatDevParams P,
                      float *__restrict__ pos_out, ChainOut *__restrict__ outs,
                      MoveTrace *__restrict__ trace) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int chain_ix = blockIdx.x / CL;
  const HeatUnit U = units[chain_ix];
  const int n = U.n;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int nthr = blockDim.x, nwarps = nthr >> 5;
  const int D = P.depth;  // a power of two
  const int dmask = D - 1, dshift = __ffs(D) - 1;
  const int pitch = U.pitch;
  // this CTA's beads [s0, s1) and the floats a ring slot holds
  const uint32_t crank = CL > 1 ? cluster_rank() : 0u;
  const bool leader = crank == 0u;
  const int s0 = CL > 1 ? (int)crank * U.slice : 0;
  const int s1 = CL > 1 ? min(n, s0 + U.slice) : n;
  const int spitch = CL > 1 ? U.slice : pitch;
  // ---- shared-memory carve ----
  unsigned char *p = smem;
  uint64_t *bars = reinterpret_cast<uint64_t *>(p);
  p += 16 * 8;
  double *red = reinterpret_cast<double *>(p);
  p += 32 * 8;
  float *partial = reinterpret_cast<float *>(p);  // [warp][kWin]
  p += 16 * kWin * 4;
  float *corr = reinterpret_cast<float *>(p);     // [w][j], j < w
  p += kWin * kWin * 4;
  WinPlan *plan_s = reinterpret_cast<WinPlan *>(p);
  p += sizeof(WinPlan);
  p = smem + (((p - smem) + 15) & ~(size_t)15);
  // cluster mode: every CTA's window record (kRec floats: its sums of the
  // kWin moves, its kWin * kWin pair corrections, its late-row flag) from
  // every CTA, two buffers by window parity; this CTA's own record and the
  // records' totals; every CTA's part of a full score
  constexpr int kRec = kWin + kWin * kWin + 1;
  constexpr int kRecP = (kRec + 3) & ~3;          // padded to whole float4s
  float4 *g_all = reinterpret_cast<float4 *>(p);  // CTA 0: [CL][kRecP / 4]
  float *own = reinterpret_cast<float *>(g_all + CL * (kRecP / 4));  // [kRecP]
  float *tot = own + kRecP;                       // CTA 0: [kRec]
  float4 *dec = reinterpret_cast<float4 *>(tot + kRecP);  // decisions from CTA 0
  double *g_e = reinterpret_cast<double *>(dec + 1);
  int *g_flag = reinterpret_cast<int *>(g_e + CL);  // [CL]
  if (CL > 1) p = reinterpret_cast<unsigned char *>(g_flag + CL);
  p = smem + (((p - smem) + 15) & ~(size_t)15);
  MoveRec *recs = reinterpret_cast<MoveRec *>(p); // ring of 128 draws
  p += 128 * sizeof(MoveRec);
  float *thrs = reinterpret_cast<float *>(p);     // ring of 128
  p += 128 * 4;
  p = smem + (((p - smem) + 127) & ~(size_t)127);
  float *slots = reinterpret_cast<float *>(p);    // D rows (slices) of 1/h
  p += (size_t)D * spitch * 4;
  float4 *spos = reinterpret_cast<float4 *>(p);
  p += (size_t)n * 16;
  // per-bead chromosome block (maps with boundaries) and the movable list
  // (regions with fixed beads): staged next to the positions
  int2 *blk = reinterpret_cast<int2 *>(p);
  if (!U.single) p += (size_t)n * 8;
  int *smov = reinterpret_cast<int *>(p);
  auto block_of = [&](int b) { return U.single ? make_int2(0, n - 1) : blk[b]; };

  const int *MOV = U.mov_off >= 0 ? smov : nullptr;
  const float *rrow0 = rheat + U.heat_off;

  if (tid == 0) {
    plan_s->pad[1] = 0;  // cluster mode: a row copy of some CTA did not land
    for (int s = 0; s < D; ++s) mbar_init(&bars[s], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  for (int i = tid; i < n; i += nthr) {
    spos[i] = pos0[U.pos_off + i];
    if (!U.single) blk[i] = blk_all[U.blk_off + i];
  }
  if (U.mov_off >= 0)
    for (int k = tid; k < U.n_mov; k += nthr) smov[k] = movable[U.mov_off + k];
  __syncthreads();

  // the start score: in cluster mode each CTA scores its rows and every CTA
  // adds the CL parts in rank order (the same value everywhere)
  double E0 = heat_full(U, spos, rheat, blk, red, P.R, s0, s1);
  if (CL > 1) {
    cluster_sync();  // every CTA of the cluster is running
    if (tid < CL) st_cluster(cluster_addr(&g_e[crank], (uint32_t)tid), E0);
    cluster_sync();
    E0 = 0.0;
    for (int q = 0; q < CL; ++q) E0 += g_e[q];
  }
  double T = P.max_temp;  // temperature of the next filled move (warp 1)
  long long filled = 0;   // records exist for moves [filled - 128, filled) (warp 1)
  long long issued = 0;   // moves whose rows were requested (warp 1)

  // draws of 32 moves [first, first + 32) into the ring (warp 1)
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
    const int slot = (int)(m & 127);
    recs[slot] = rec;
    thrs[slot] = ratio_threshold(u01(a.x), Tl, P.inv_scale, P.inv_coef);
    T *= P.dtpow[32];
  };
  // row copies up to move `upto` (exclusive), one per lane (warp 1)
  auto issue = [&](long long upto) {
    while (issued < upto) {
      const int cnt = (int)min(32ll, upto - issued);
      if (lane < cnt) {
        const long long k = issued + lane;
        const int b = recs[k & 127].b;
        int st, en;
        if (CL > 1) {  // this CTA's slice of the row
          st = s0;
          en = min(s0 + spitch, pitch);
        } else {
          const int2 r = block_of(b);
          st = r.x & ~3;
          en = min((r.y + 4) & ~3, pitch);
        }
        tma_row(slots + (size_t)(k & dmask) * spitch, rrow0 + (long long)b * pitch + st,
                (uint32_t)(en - st) * 4, &bars[k & dmask]);
      }
      issued += cnt;
    }
  };
  const bool run = U.n_mov > 0 && E0 >= 1e-6 && E0 == E0;
  const long long cap = run ? P.cap : 0;
  // The window starting at m0 (warp 0; the draws of [m0, m0 + kWin) are in
  // the ring and its rows were requested): its length, whether its beads share
  // one block, each move's geometry at the current positions, and the wait
  // for its rows.  Slots past the length repeat move 0 (scored, unused).
  // with_pos = false leaves out the moved beads' old positions (cluster
  // mode plans the rest while CTA 0 decides; plan_old_pos adds them after)
  auto plan = [&](long long m0, long long nms, bool with_pos = true) {
    const int lim = (int)max(1ll, min((long long)min(kWin, D), min(nms, cap) - m0));
    const int b = lane < lim ? recs[(m0 + lane) & 127].b : -1 - lane;
    bool rep = false;
#pragma unroll
    for (int j = 0; j < kWin; ++j) {
      const int bj = __shfl_sync(0xffffffffu, b, j);  // every lane takes part
      rep |= j < lane && bj == b;
    }
    const unsigned rm = __ballot_sync(0xffffffffu, rep && lane < lim);
    const int L = rm ? min(lim, __ffs(rm) - 1) : lim;
    const int ww = lane < L ? lane : 0;
    const long long k = m0 + ww;
    const MoveRec rec = recs[k & 127];
    const int2 bk = block_of(rec.b);
    const int bx0 = __shfl_sync(0xffffffffu, bk.x, 0), by0 = __shfl_sync(0xffffffffu, bk.y, 0);
    const unsigned diff = __ballot_sync(0xffffffffu, bk.x != bx0 || bk.y != by0);
    bool late = false;
    if (lane < kWin) {
      if (with_pos) {
        const float4 o = spos[rec.b];
        plan_s->ga[lane] = make_float4(o.x, o.y, o.z,
                                       fmaf(rec.dx, rec.dx, fmaf(rec.dy, rec.dy, rec.dz * rec.dz)));
      }
      const int roff = CL > 1 ? (int)(k & dmask) * spitch - s0
                              : (int)(k & dmask) * pitch - (bk.x & ~3);
      plan_s->gb[lane] =
          make_float4(-2.0f * rec.dx, -2.0f * rec.dy, -2.0f * rec.dz, __int_as_float(roff));
      plan_s->bw[lane] = rec.b;
      if (lane < L) late = !mbar_wait(&bars[k & dmask], (uint32_t)((k >> dshift) & 1));
    }
    const unsigned lm = __ballot_sync(0xffffffffu, late);
    if (lane == 0) {
      plan_s->len = L;
      plan_s->same = diff == 0u;
      plan_s->timeout = lm != 0u;
    }
  };
  auto plan_old_pos = [&](long long m0) {
    const int L = plan_s->len;
    if (lane < kWin) {
      const MoveRec rec = recs[(m0 + (lane < L ? lane : 0)) & 127];
      const float4 o = spos[rec.b];
      plan_s->ga[lane] = make_float4(o.x, o.y, o.z,
                                     fmaf(rec.dx, rec.dx, fmaf(rec.dy, rec.dy, rec.dz * rec.dz)));
    }
  };

  if (warp == 1 && cap > 0) {
    for (int f = 0; f < 4; ++f) {
      fill(filled);
      filled += 32;
    }
    __syncwarp();
    issue(min((long long)D, cap));
  }
  __syncthreads();
  if (warp == 0 && cap > 0) plan(0, P.window);
  __syncthreads();

  float e_hi = (float)E0, e_lo = (float)(E0 - (double)(float)E0);
  double E_ms = E0;
  int succ = 0, misses = 0, status = kDevOk;
  long long moves = 0, accepted = 0;
  long long next_ms = P.window;
  bool stop = cap == 0;
  // (cluster mode: late rows are gathered at the first window and stop every
  // CTA together)
  if (CL == 1 && !stop && plan_s->timeout) {
    status = PMMC_ERR_TIMEOUT;
    stop = true;
  }
  // corrections (w, j) are spread over the warps: thread c * cstride
  const int cstride = nthr / (kWin * kWin);

  while (!stop) {
    const long long m = moves;
    const int L = plan_s->len;
    const bool same = plan_s->same != 0;
    MoveGeo g[kWin];
    int roff[kWin];
#pragma unroll
    for (int w = 0; w < kWin; ++w) {
      const float4 a = plan_s->ga[w], b = plan_s->gb[w];
      g[w].ox = a.x;
      g[w].oy = a.y;
      g[w].oz = a.z;
      g[w].dd = a.w;
      g[w].mx = b.x;
      g[w].my = b.y;
      g[w].mz = b.z;
      roff[w] = __float_as_int(b.w);
    }
    float part[kWin];
#pragma unroll
    for (int w = 0; w < kWin; ++w) part[w] = 0.0f;
    if (same) {
      const int2 r = block_of(plan_s->bw[0]);
      const int i0 = CL > 1 ? max(r.x, s0) : r.x, i1 = CL > 1 ? min(r.y, s1 - 1) : r.y;
      for (int i = i0 + tid; i <= i1; i += nthr) {
        const float4 pi = spos[i];
#pragma unroll
        for (int w = 0; w < kWin; ++w)
          part[w] += pair_delta(pi.x, pi.y, pi.z, g[w], slots[roff[w] + i]);
      }
    } else {
#pragma unroll
      for (int w = 0; w < kWin; ++w) {
        if (w < L) {
          const int2 r = block_of(plan_s->bw[w]);
          const int i0 = CL > 1 ? max(r.x, s0) : r.x, i1 = CL > 1 ? min(r.y, s1 - 1) : r.y;
          for (int i = i0 + tid; i <= i1; i += nthr) {
            const float4 pi = spos[i];
            part[w] += pair_delta(pi.x, pi.y, pi.z, g[w], slots[roff[w] + i]);
          }
        }
      }
    }
    // pair corrections: the (b_w, b_j) term once move j (< w) has moved
    if (tid % cstride == 0 && tid / cstride < kWin * kWin) {
      const int c = tid / cstride, w = c >> 3, j = c & 7;
      float v = 0.0f;
      if (j < w && w < L) {
        const int bw = plan_s->bw[w], bj = plan_s->bw[j];
        const int2 r = block_of(bw);
        // (cluster mode: the CTA whose slice holds column bj)
        if (bj >= r.x && bj <= r.y && (CL == 1 || (bj >= s0 && bj < s1))) {
          const float4 gb = plan_s->gb[w];
          const float rv = slots[__float_as_int(gb.w) + bj];
          const float4 oj = plan_s->ga[j], dj = plan_s->gb[j];
          MoveGeo gw;
          const float4 ow = plan_s->ga[w];
          gw.ox = ow.x;
          gw.oy = ow.y;
          gw.oz = ow.z;
          gw.dd = ow.w;
          gw.mx = gb.x;
          gw.my = gb.y;
          gw.mz = gb.z;
          v = pair_delta(fmaf(-0.5f, dj.x, oj.x), fmaf(-0.5f, dj.y, oj.y),
                         fmaf(-0.5f, dj.z, oj.z), gw, rv) -
              pair_delta(oj.x, oj.y, oj.z, gw, rv);
        }
      }
      corr[c] = v;
    }
#pragma unroll
    for (int w = 0; w < kWin; ++w) {
      const float v = warp_sum_f(part[w]);
      if (lane == 0) partial[warp * kWin + w] = v;
    }
    __syncthreads();
    // draws (moves below m are done, so the records of [filled - 128,
    // filled - 96) are free when filled <= m + 64) and the row copies that
    // the slots freed by this window can take (warp 1)
    auto draws_and_copies = [&]() {
      if (filled <= m + 64) {
        fill(filled);
        filled += 32;
        __syncwarp();
      }
      issue(min(cap, m + L + D));
    };
    if (CL > 1) {
      // this CTA's record (its sums, pair corrections and late-row flag) to
      // CTA 0, in float4 stores
      if (warp == 0) {
        const int wl = lane & (kWin - 1);
        float t = 0.0f;
        for (int k = lane >> 3; k < nwarps; k += 4) t += partial[k * kWin + wl];
        t += __shfl_xor_sync(0xffffffffu, t, 8);
        t += __shfl_xor_sync(0xffffffffu, t, 16);
        if (lane < kWin) own[lane] = t;
        if (lane == 0) {
          own[kRec - 1] = __int_as_float(plan_s->timeout);
          for (int v = kRec; v < kRecP; ++v) own[v] = 0.0f;
        }
      }
      if (tid < kWin * kWin) own[kWin + tid] = corr[tid];
      __syncthreads();
      if (tid < kRecP / 4) {
        const float4 v = reinterpret_cast<const float4 *>(own)[tid];
        const uint32_t a4 = cluster_addr(&g_all[(int)crank * (kRecP / 4) + tid], 0);
        asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(a4), "f"(v.x),
                     "f"(v.y), "f"(v.z), "f"(v.w)
                     : "memory");
      }
      cluster_sync();  // every record is at CTA 0
      if (leader) {    // the records' totals, in rank order
        if (tid < kRec) {
          const float *r0 = reinterpret_cast<const float *>(g_all);
          if (tid == kRec - 1) {
            int late = 0;
            for (int q = 0; q < CL; ++q) late |= __float_as_int(r0[q * kRecP + tid]);
            tot[tid] = __int_as_float(late);
          } else {
            float a = 0.0f;
            for (int q = 0; q < CL; ++q) a += r0[q * kRecP + tid];
            tot[tid] = a;
          }
        }
        __syncthreads();
      }
      // the draws, the row copies and the next window's plan (all but the
      // moved beads' old positions) do not depend on the decisions: they
      // run while CTA 0 takes them
      if (warp == 1) draws_and_copies();
      if (warp == 2 && m + L < cap)
        plan(m + L, m + L == next_ms ? next_ms + P.window : next_ms, false);
    }
    // ---- warp 0 (of CTA 0 in cluster mode): decisions, the next window ----
    if (warp == 0 && leader) {
      const int wl = lane & (kWin - 1);
      float t = 0.0f;
      float cr[kWin];
      if (CL == 1) {
        for (int k = lane >> 3; k < nwarps; k += 4) t += partial[k * kWin + wl];
        t += __shfl_xor_sync(0xffffffffu, t, 8);
        t += __shfl_xor_sync(0xffffffffu, t, 16);
#pragma unroll
        for (int j = 0; j < kWin; ++j) cr[j] = corr[wl * kWin + j];
      } else {
        t = tot[wl];
#pragma unroll
        for (int j = 0; j < kWin; ++j) cr[j] = tot[kWin + wl * kWin + j];
      }
      const int ll = lane < L ? lane : 0;
      const MoveRec rec = recs[(m + ll) & 127];
      const float4 ow = spos[rec.b];
      const float4 nw = make_float4(ow.x + rec.dx, ow.y + rec.dy, ow.z + rec.dz, 0.f);
      const float sph =
          P.R > 0.0f ? sphere_penalty(nw.x, nw.y, nw.z, P.R) - sphere_penalty(ow.x, ow.y, ow.z, P.R)
                     : 0.0f;
      const float thr = thrs[(m + ll) & 127];
      float dloc = t;  // local change of this move given the accepted earlier ones
      unsigned accm = 0u;
      float pacc = 0.0f;
#pragma unroll
      for (int j = 0; j < kWin; ++j) {
        if (j < L) {
          const float dj = __shfl_sync(0xffffffffu, 2.0f * dloc + sph, j);
          const float tj = __shfl_sync(0xffffffffu, thr, j);
          if (dj <= 0.0f || dj < (e_hi + pacc) * (tj - 1.0f)) {
            accm |= 1u << j;
            pacc += dj;
            dloc += cr[j];
          }
        }
      }
      if (CL == 1 && lane < L && ((accm >> lane) & 1u)) spos[rec.b] = nw;
      if (trace != nullptr && U.chain_id == 0 && lane < L && m + lane < P.trace_cap) {
        MoveTrace tr;
        tr.bead = rec.b;
        tr.accepted = (accm >> lane) & 1u;
        tr.before = 0.0f;
        tr.after = 2.0f * dloc;
        tr.dx = rec.dx;
        tr.dy = rec.dy;
        tr.dz = rec.dz;
        tr.pad = 2.0f * dloc + sph;
        trace[m + lane] = tr;
      }
      __syncwarp();
      if (CL == 1) {
        const long long mn = m + L;
        if (lane == 0) {
          plan_s->accm = accm;
          plan_s->lend = L;
          plan_s->pacc = pacc;
          plan_s->timeout = 0;
        }
        if (mn < cap) plan(mn, mn == next_ms ? next_ms + P.window : next_ms);
      } else if (lane < CL) {  // the decisions to every CTA, one float4 each
        const uint32_t a4 = cluster_addr(dec, (uint32_t)lane);
        asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(a4),
                     "f"(__uint_as_float(accm)), "f"(pacc), "f"(tot[kRec - 1]), "f"(0.0f)
                     : "memory");
      }
    } else if (CL == 1 && warp == 1) {
      draws_and_copies();
    }
    if (CL > 1) {
      cluster_sync();  // every CTA has the window's decisions
      if (warp == 0) {
        // apply them (every CTA keeps all positions) and plan the next window
        const float4 dv = *dec;
        const unsigned am = __float_as_uint(dv.x);
        if (lane < L && ((am >> lane) & 1u)) {
          const MoveRec rec = recs[(m + lane) & 127];
          const float4 ow = spos[rec.b];
          spos[rec.b] = make_float4(ow.x + rec.dx, ow.y + rec.dy, ow.z + rec.dz, 0.f);
        }
        __syncwarp();
        const int late = __float_as_int(dv.z);
        if (lane == 0) {
          plan_s->accm = am;
          plan_s->pacc = dv.y;
          plan_s->pad[1] = late;
          plan_s->lend = L;
        }
        const long long mn = m + L;
        if (mn < cap && late == 0) plan_old_pos(mn);
      }
    }
    __syncthreads();
    const unsigned accm = plan_s->accm;
    if (accm) ff_add(e_hi, e_lo, plan_s->pacc);
    const int na = __popc(accm);
    accepted += na;
    succ += na;
    moves = m + plan_s->lend;
    if (moves == next_ms) {
      next_ms += P.window;
      // LooperSolver.hpp:1543-1548 (FP64)
      const double E = (double)e_hi + (double)e_lo;
      const bool miss = (E > (double)P.improvement * E_ms && succ < P.min_succ) || E < 1e-6;
      misses = miss ? misses + 1 : 0;
      if (misses >= P.fails || E < 1e-6) stop = true;
      E_ms = E;
      succ = 0;
    }
    if (moves >= cap) stop = true;
    // a row copy never landed: give up on this chain (cluster mode: any
    // CTA's, the same flag everywhere)
    if (!stop && (CL == 1 ? plan_s->timeout : plan_s->pad[1])) {
      status = PMMC_ERR_TIMEOUT;
      stop = true;
    }
  }
  __syncthreads();
  // drain copies still in flight (rows prefetched past the last move)
  if (warp == 1) {
    bool late = false;
    for (long long k = moves + lane; k < issued; k += 32)
      late |= !mbar_wait(&bars[k & dmask], (uint32_t)((k >> dshift) & 1));
    const bool any_late = __any_sync(0xffffffffu, late);
    if (lane == 0) plan_s->pad[0] = any_late ? 1 : 0;
  }
  __syncthreads();
  if (plan_s->pad[0] != 0) status = PMMC_ERR_TIMEOUT;
  __syncthreads();
  double Efin = heat_full(U, spos, rheat, blk, red, P.R, s0, s1);
  if (CL > 1) {  // CTA 0 adds the parts (and any CTA's late copies)
    if (tid == 0) {
      st_cluster(cluster_addr(&g_e[crank], 0), Efin);
      st_cluster(cluster_addr(&g_flag[crank], 0), status);
    }
    cluster_sync();  // the last access to another CTA's shared memory
    if (leader) {
      Efin = 0.0;
      for (int q = 0; q < CL; ++q) {
        Efin += g_e[q];
        if (status == kDevOk && g_flag[q] != kDevOk) status = g_flag[q];
      }
    }
  }
  if (!leader) return;  // CTA 0 writes the chain's results
  if (tid == 0) {
    ChainOut o;
    const double E = run ? (double)e_hi + (double)e_lo : 0.0;
    o.energy = E;
    o.energy_fp64 = run ? Efin : 0.0;
    o.base = 0.0;
    o.best = E;
    o.score = (float)E;
    o.status = status;
    o.moves = moves;
    o.accepted = accepted;
    outs[chain_ix] = o;
  }
  float *po = pos_out + U.out_off;
  for (int i = tid; i < n; i += nthr) {
    const float4 q = spos[i];
    po[3 * i] = q.x;
    po[3 * i + 1] = q.y;
    po[3 * i + 2] = q.z;
  }
}

constexpr int kPackTile = 32;

// r = 1/h where the score of bead m reads the pair (m, i), else 0.  The
// reciprocal is correctly rounded (the value of 1.0f / h in IEEE single).
__device__ __forceinline__ float packed_r(float h, int m, int i, int2 b, int diag) {
  const bool read = i >= b.x && i <= b.y && abs(i - m) >= diag && i != m && h >= 1e-6f;
  return read ? __frcp_rn(h) : 0.0f;
}

// The device matrix from a chunk of the caller's maps (map u: n x n,
// row-major, at raw_off[u] - raw_base of `raw`): rows of U.pitch floats at
// U.heat_off holding packed_r, the padding columns zero.  The same pass
// checks symmetry over the pairs the score reads (m < i in bead m's block,
// i - m >= diag): h_mi and h_im must both be skipped (< 1e-6) or be equal;
// asym[u] keeps the lowest m * n + i of a pair that is not (all ones: none).
// One 256-thread block per pair of 32 x 32 tiles (bm, bi), bm <= bi, of one
// map (map u's first block is tile_start[u] - tile_base): the tile and its
// mirror are staged in shared memory, so both are read and written along
// rows.
__global__ void __launch_bounds__(256)
heat_pack_kernel(const HeatUnit *__restrict__ units, int n_units,
                 const long long *__restrict__ tile_start, long long tile_base,
                 const long long *__restrict__ raw_off, long long raw_base,
                 const float *__restrict__ raw, const int2 *__restrict__ blk,
                 float *__restrict__ rheat, unsigned long long *__restrict__ asym) {
  __shared__ float A[kPackTile][kPackTile + 1];  // rows m0.., columns i0..
  __shared__ float B[kPackTile][kPackTile + 1];  // rows i0.., columns m0..
  const long long t = tile_base + blockIdx.x;
  int lo = 0, hi = n_units - 1;  // the last map whose first block is <= t
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (tile_start[mid] <= t)
      lo = mid;
    else
      hi = mid - 1;
  }
  const int u = lo;
  const HeatUnit U = units[u];
  const int n = U.n;
  const int nt = (n + kPackTile - 1) / kPackTile;
  const int2 tb = upper_tile(t - tile_start[u], nt);
  const int m0 = tb.x * kPackTile, i0 = tb.y * kPackTile;
  const bool on_diag = tb.x == tb.y;
  const float *H = raw + (raw_off[u] - raw_base);
  float *R = rheat + U.heat_off;
  const int tx = threadIdx.x & 31, ty = threadIdx.x >> 5;
  for (int r = ty; r < kPackTile; r += 8) {
    const int m = m0 + r, i = i0 + tx;
    A[r][tx] = (m < n && i < n) ? H[(size_t)m * n + i] : 0.0f;
    const int m2 = i0 + r, i2 = m0 + tx;
    if (!on_diag) B[r][tx] = (m2 < n && i2 < n) ? H[(size_t)m2 * n + i2] : 0.0f;
  }
  __syncthreads();
  for (int r = ty; r < kPackTile; r += 8) {
    const int m = m0 + r, i = i0 + tx;
    if (m < n && i < n) {
      const int2 b = blk[U.blk_off + m];
      const float a = A[r][tx];
      R[(size_t)m * U.pitch + i] = packed_r(a, m, i, b, U.diag);
      if (i > m && i >= b.x && i <= b.y && i - m >= U.diag) {
        const float c = on_diag ? A[tx][r] : B[tx][r];  // h_im
        const bool ua = a >= 1e-6f, uc = c >= 1e-6f;
        if (ua != uc || (ua && a != c)) atomicMin(&asym[u], (unsigned long long)m * n + i);
      }
    } else if (m < n && i < U.pitch) {
      R[(size_t)m * U.pitch + i] = 0.0f;  // padding (the last column tile)
    }
    const int m2 = i0 + r, i2 = m0 + tx;
    if (!on_diag && m2 < n && i2 < n)
      R[(size_t)m2 * U.pitch + i2] = packed_r(B[r][tx], m2, i2, blk[U.blk_off + m2], U.diag);
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
  size_t max_bead_bytes = 0;
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
    U.single = 1;
    for (int i = 0; i < pr.n; ++i) {
      const int2 b = hblk[(size_t)U.blk_off + i];
      if (b.x != 0 || b.y != pr.n - 1) U.single = 0;
    }
    U.heat_off = heat_floats;
    heat_floats += (long long)U.pitch * pr.n;
    U.chain_id = u;
    U.out_off = out_off;
    out_off += (long long)pr.n * 3;
    U.step = steps[u] * 0.5f;  // MonteCarloHeatmap halves the step (:1426)
    max_n = std::max(max_n, pr.n);
    max_pitch = std::max(max_pitch, U.pitch);
    // staged per bead: position, block (maps with boundaries), movable index
    max_bead_bytes = std::max(max_bead_bytes, (size_t)pr.n * (16 + (U.single ? 0 : 8) +
                                                               (U.mov_off >= 0 ? 4 : 0)));
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
  // Cluster mode for a few chains on a large map: each chain spread over CL
  // CTAs (one per SM), each scoring a slice of every row.
  int CL = ctx->heatmap_cluster;
  if (CL == 0)  // 16 CTAs (beyond the portable size) for up to 4 chains
    CL = (n_units <= 4 && max_n >= 1024 && 16 * n_units <= ctx->sm_count) ? 16
         : (n_units * 8 <= ctx->sm_count && max_n >= 512)                  ? 8
                                                                          : 1;
  if (CL != 1 && CL != 2 && CL != 4 && CL != 8 && CL != 16)
    return fail(ctx, PMMC_ERR_INVALID, "heatmap: cluster of %d CTAs (1, 2, 4, 8 or 16)", CL);
  while (CL > 1) {  // every CTA needs beads of its own
    bool ok = true;
    for (const HeatUnit &U : hu) {
      const int sl = ((U.n + CL - 1) / CL + 3) & ~3;
      if ((long long)sl * (CL - 1) >= U.n) ok = false;
    }
    if (ok) break;
    CL >>= 1;
  }
  int max_slice = 0;
  if (CL > 1)
    for (HeatUnit &U : hu) {
      U.slice = ((U.n + CL - 1) / CL + 3) & ~3;
      max_slice = std::max(max_slice, U.slice);
    }
  // Shared memory: header + D row slots + per-bead arrays.  With at least two
  // chains per SM of work, two CTAs of 256 threads share an SM (one chain's
  // serial decisions overlap the other's row pass) when a ring of 8 rows
  // still fits in half the SM's shared memory; otherwise one CTA per SM.
  const size_t head = kHeadBytes;
  const size_t row_bytes = (size_t)max_pitch * 4;
  int depth = 0, ctas_per_sm = 1;
  size_t smem = 0;
  for (int mode : {2, 1}) {
    if (CL > 1) break;
    if (mode == 2 && n_units < 2 * ctx->sm_count) continue;
    const size_t avail = mode == 2 ? std::min(ctx->smem_optin, ctx->smem_per_sm / 2 - 1024)
                                   : ctx->smem_optin;
    if (head + max_bead_bytes + 2 * row_bytes > avail) continue;
    const size_t fit = (avail - head - max_bead_bytes) / row_bytes;
    int d = 2;
    while (d < 16 && (size_t)d * 2 <= fit) d *= 2;
    if (mode == 2 && d < kWin) continue;
    depth = d;
    ctas_per_sm = mode;
    smem = head + (size_t)d * row_bytes + max_bead_bytes;
    break;
  }
  if (CL > 1) {
    // header with the cluster's gather area, a 16-slot ring of row slices
    const size_t rec = (kWin + kWin * kWin + 1 + 3) & ~(size_t)3;
    const size_t gather = ((size_t)CL * rec + 2 * rec + 4) * 4 + (size_t)CL * 12 + 256;
    depth = 16;
    smem = head + gather + (size_t)depth * max_slice * 4 + max_bead_bytes;
    if (smem > ctx->smem_optin) depth = 0;
  }
  if (depth == 0)
    return fail(ctx, PMMC_ERR_INVALID, "heatmap region of %d beads does not fit shared memory", max_n);
  P.depth = depth;

  cudaStream_t s = ctx->stream;
  // The kernels read r = 1/h, rows padded to a 16-byte pitch, with r = 0
  // wherever the reference skips the pair: h < 1e-6, |i - m| < diag, i == m,
  // and i outside bead m's chromosome block (LooperSolver.hpp:3597-3611).
  // The caller's maps go to the device as they are, in chunks of at most
  // 256 MiB (a larger map alone) through one staging buffer, and
  // heat_pack_kernel writes that matrix chunk by chunk (stream order keeps
  // the next chunk's copy behind the pass that reads the buffer).  A move changes the full score by twice its local
  // change only when the map is symmetric over the pairs the score reads
  // (createDistanceHeatmap mirrors it, LooperSolver.hpp:3062); the same pass
  // finds an asymmetric map, which is refused.
  std::vector<long long> tile_start((size_t)n_units + 1, 0), raw_off((size_t)n_units, 0);
  long long raw_floats = 0;
  for (int u = 0; u < n_units; ++u) {
    const long long nt = (hu[u].n + kPackTile - 1) / kPackTile;
    tile_start[u + 1] = tile_start[u] + nt * (nt + 1) / 2;
    raw_off[u] = raw_floats;
    raw_floats += (long long)hu[u].n * hu[u].n;
  }
  if (tile_start[n_units] > 0x7fffffffll)
    return fail(ctx, PMMC_ERR_INVALID, "heatmap batch: too many map tiles");
  DevBuf<HeatUnit> d_units;
  DevBuf<float4> d_pos;
  DevBuf<float> d_rheat, d_out, d_raw;
  DevBuf<int> d_mov;
  DevBuf<int2> d_blk;
  DevBuf<ChainOut> d_outs;
  DevBuf<MoveTrace> d_trace;
  DevBuf<long long> d_tile_start, d_raw_off;
  DevBuf<unsigned long long> d_asym;
  cudaError_t e = d_units.upload(hu, s);
  if (e == cudaSuccess) e = d_pos.upload(hpos, s);
  if (e == cudaSuccess) e = d_mov.upload(hmov, s);
  if (e == cudaSuccess) e = d_blk.upload(hblk, s);
  if (e == cudaSuccess) e = d_tile_start.upload(tile_start, s);
  if (e == cudaSuccess) e = d_raw_off.upload(raw_off, s);
  long long stage = 64ll << 20;  // floats (256 MiB)
  for (int u = 0; u < n_units; ++u) stage = std::max(stage, (long long)hu[u].n * hu[u].n);
  stage = std::min(stage, raw_floats);
  if (e == cudaSuccess) e = d_rheat.alloc((size_t)heat_floats);
  if (e == cudaSuccess) e = d_raw.alloc((size_t)stage);
  if (e == cudaSuccess) e = d_asym.alloc((size_t)n_units);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(d_asym.p, 0xff, sizeof(unsigned long long) * n_units, s);
  std::vector<unsigned long long> asym((size_t)n_units, ~0ull);
  for (int u0 = 0; u0 < n_units && e == cudaSuccess;) {
    int u1 = u0 + 1;  // the chunk [u0, u1): whole maps within the buffer
    while (u1 < n_units && raw_off[u1] - raw_off[u0] + (long long)hu[u1].n * hu[u1].n <= stage)
      ++u1;
    for (int u = u0; u < u1 && e == cudaSuccess; ++u)
      e = cudaMemcpyAsync(d_raw.p + (raw_off[u] - raw_off[u0]), units[u].heat,
                          sizeof(float) * (size_t)units[u].n * units[u].n,
                          cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
      heat_pack_kernel<<<(unsigned)(tile_start[u1] - tile_start[u0]), 256, 0, s>>>(
          d_units.p + u0, u1 - u0, d_tile_start.p + u0, tile_start[u0], d_raw_off.p + u0,
          raw_off[u0], d_raw.p, d_blk.p, d_rheat.p, d_asym.p + u0);
      e = cudaGetLastError();
    }
    u0 = u1;
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(asym.data(), d_asym.p, sizeof(unsigned long long) * n_units,
                        cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  d_raw.release();
  if (e == cudaSuccess) e = d_out.alloc((size_t)out_off);
  if (e == cudaSuccess) e = d_outs.alloc((size_t)n_units);
  if (e == cudaSuccess && trace_cap > 0) e = d_trace.alloc((size_t)trace_cap);
  if (e != cudaSuccess)
    return fail(ctx, e == cudaErrorMemoryAllocation ? PMMC_ERR_NOMEM : PMMC_ERR_CUDA,
                "heatmap upload: %s", cudaGetErrorString(e));
  for (int u = 0; u < n_units; ++u)
    if (asym[u] != ~0ull)
      return fail(ctx, PMMC_ERR_INVALID,
                  "heatmap region %d: the map is not symmetric at (%lld, %lld)", u,
                  (long long)(asym[u] / (unsigned long long)units[u].n),
                  (long long)(asym[u] % (unsigned long long)units[u].n));
  auto kernel_of = [](int cl) {
    return cl == 16  ? heatmap_anneal_kernel<16>
           : cl == 8 ? heatmap_anneal_kernel<8>
           : cl == 4 ? heatmap_anneal_kernel<4>
           : cl == 2 ? heatmap_anneal_kernel<2>
                     : heatmap_anneal_kernel<1>;
  };
  const auto kern = kernel_of(CL);
  if (CL > 8)  // clusters above 8 CTAs are opt-in
    PMMC_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  PMMC_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smem));
  PMMC_CUDA(ctx, cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, s);
  // threads per chain: about four row entries per thread, 128..512 (at most
  // 256 when two chains share an SM)
  int threads = 128;
  const int max_threads = ctas_per_sm == 2 ? 256 : kHeatMaxThreads;
  if (CL > 1) {
    threads = max_slice >= 256 ? 256 : 128;
  } else {
    while (threads < max_threads && threads * 4 < max_n) threads *= 2;
  }
  MoveTrace *dtr = trace_cap > 0 ? d_trace.p : nullptr;
  if (CL == 1) {
    heatmap_anneal_kernel<1><<<n_units, threads, smem, s>>>(d_units.p, d_pos.p, d_rheat.p,
                                                            d_mov.p, d_blk.p, P, d_out.p,
                                                            d_outs.p, dtr);
    e = cudaGetLastError();
  } else {
    cudaLaunchConfig_t cfg{};
    cfg.gridDim = dim3((unsigned)(n_units * CL));
    cfg.blockDim = dim3((unsigned)threads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)CL;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    e = cudaLaunchKernelEx(&cfg, kern, (const HeatUnit *)d_units.p, (const float4 *)d_pos.p,
                           (const float *)d_rheat.p, (const int *)d_mov.p,
                           (const int2 *)d_blk.p, P, d_out.p, d_outs.p, dtr);
  }
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

extern "C" pmmc_status pmmc_heatmap_set_cluster(pmmc_ctx *ctx, int ctas) {
  if (!ctx) return PMMC_ERR_INVALID;
  if (ctas != 0 && ctas != 1 && ctas != 2 && ctas != 4 && ctas != 8 && ctas != 16)
    return fail(ctx, PMMC_ERR_INVALID, "heatmap cluster: %d CTAs (0, 1, 2, 4, 8 or 16)", ctas);
  ctx->heatmap_cluster = ctas;
  return PMMC_OK;
}

extern "C" pmmc_status pmmc_heatmap_anneal(pmmc_ctx *ctx, const pmmc_heatmap_problem *pr,
                                           const pmmc_anneal_params *prm, float step_size,
                                           float *pos_out, pmmc_result *res) {
  return pmmc_heatmap_batch_anneal(ctx, 1, pr, prm, &step_size, pos_out, res, nullptr,
                                   nullptr, 0);
}
