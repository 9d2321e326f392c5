// targets.cu -- expected distances of an anchor-level region, built as CSR.
//
// LooperSolver::calcAnchorExpectedDistancesHeatmap (LooperSolver.hpp:
// 5494-5627) fills a dense n x n matrix (-1 everywhere, 0 on the diagonal)
// on one host core before every anchor-level annealing: the arcs of the
// active clusters, then the genomic-position long arcs, each resolved to an
// anchor by a linear scan over the chromosome's anchors (:5564-5568), then
// optionally the anchor heatmap's influence.  The annealer only reads the
// pairs that hold a distance, so the matrix is never formed here:
//
//   host    the arcs of the active clusters (a few per cluster; the last
//           write of a pair wins), with the reference's std::map slot lookup;
//   long_map       one thread per long arc: both positions to anchors
//                  through a bucket table over the anchor starts (sorted,
//                  disjoint anchors; a bucket per anchor at most, the starts
//                  and buckets in shared memory; otherwise the reference's
//                  first-match scan), anchors to active slots, the pair key
//                  (low slot * n + high slot);
//   radix sort     (pair key, index) over the pairs the host wrote followed
//                  by the long arcs: the stable sort puts each pair's own
//                  value first, then its long arcs in the reference's order;
//   long_resolve   (every distance >= 0: long_resolve_first, one thread per
//                  entry: the first long arc of a pair off the diagonal is
//                  written unless an arc of the active clusters wrote the
//                  pair, every other collides) otherwise
//                  one thread per pair: the reference's sequence of writes
//                  and collisions replayed from the pair's own value, so the
//                  first long arc with a distance >= 0 wins unless an arc of
//                  the active clusters already holds one (a long arc's
//                  distance is computed only when it is written);
//   heat_diag / heat_max  Heatmap::getDiagonalSize / getRange of the anchor
//                  heatmap (only with the influence on);
//   pair_emit      influence, both directions of every pair;
//   radix sort     (row * n + col): rows in order, columns sorted;
//   csr_finish     columns and row pointers by binary search.
// Keys are sorted on the bits n * n needs only (24 for 4096 slots: three
// radix passes instead of eight).
// Per long arc in long_map: 8 bytes of positions read, two bucket lookups,
// 12 bytes of key and index written.
#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <climits>
#include <cmath>
#include <unordered_map>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace pmmc {

namespace {

struct CountToDist {
  float a, scale, shift, base;
};

// freqToDistance(freq, memo = true) (LooperSolver.hpp:3949-3967).  The
// reference adds the float shift to the int count in float, truncates for
// the power-law branch, and evaluates the rest in FP64.
__device__ float freq_to_distance_dev(int freq, const float *__restrict__ memo,
                                      const CountToDist c) {
  if (freq >= 1 && freq <= 100) return memo[freq];
  const float fs = __fadd_rn(__int2float_rn(freq), c.shift);
  if (c.a < 0.0f) {
    int fi = __float2int_rz(fs);
    if (fi < 1) fi = 1;
    return __double2float_rn(
        __dadd_rn((double)c.base, __dmul_rn((double)c.scale, pow((double)fi, (double)c.a))));
  }
  return __double2float_rn(__dadd_rn(
      (double)c.base, __ddiv_rn((double)c.scale, exp(__dmul_rn((double)c.a, (double)fs)))));
}

float freq_to_distance_host(int freq, const float *memo, const CountToDist c) {
  if (freq >= 1 && freq <= 100) return memo[freq];
  return count_to_distance(freq, c.a, c.scale, c.shift, c.base);
}

// Anchor::contains(pos) (Anchor.hpp:87): start <= pos <= end; the first
// anchor that holds the position, by the reference's scan (unsorted or
// overlapping anchors).
__device__ int find_anchor_scan(const int *__restrict__ st, const int *__restrict__ en,
                                int n_anc, int pos) {
  for (int i = 0; i < n_anc; ++i)
    if (pos >= st[i] && pos <= en[i]) return i;
  return -1;
}

// Sorted, disjoint anchors (each start above the previous end) through a
// bucket table: first[b] is the last anchor starting at or before
// pos0 + (b << shift) (-1: none), so the last anchor starting at or before
// pos is first[b] or a few anchors after it.
__device__ __forceinline__ int find_anchor_bucket(const int *__restrict__ st,
                                                  const int *__restrict__ en,
                                                  const int *__restrict__ first, int n_anc,
                                                  int nb, int pos0, int shift, int pos) {
  if (pos < pos0) return -1;
  const long long b = min(((long long)pos - pos0) >> shift, (long long)nb - 1);
  int i = first[b];
  while (i + 1 < n_anc && st[i + 1] <= pos) ++i;
  return (i >= 0 && pos <= en[i]) ? i : -1;
}

// Unordered pair of slots; n * n marks "no pair" and sorts last.
__host__ __device__ __forceinline__ uint64_t pair_key(int a, int b, int n) {
  const int lo = a < b ? a : b, hi = a < b ? b : a;
  return (uint64_t)lo * (uint64_t)n + (uint64_t)hi;
}

int key_bits(int n) {
  const uint64_t top = (uint64_t)n * (uint64_t)n;  // the "no pair" key
  int b = 1;
  while (b < 64 && (top >> b) != 0) ++b;
  return b;
}

enum { kCntApplied = 0, kCntOor = 1, kCntInactive = 2, kCntCollision = 3, kCntPairs = 4 };

// Entries of the sort: [0, n_short) the pairs the arcs of the active clusters
// wrote (index kShort | s), then the long arcs (index k).  The stable sort
// puts a pair's own value first, then its long arcs in order.
constexpr uint32_t kShort = 0x80000000u;

constexpr int kThreads = 256;  // block size of the long-arc kernels

// Adds each thread's count into *dst once per block: thread totals stay in
// registers over the grid-stride loop, a single atomic per block and counter
// (one same-address atomic per warp and iteration was the bottleneck).
__device__ __forceinline__ void block_count(unsigned v, unsigned long long *dst) {
  __shared__ unsigned s_part[kThreads / 32];
  v = __reduce_add_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0) s_part[threadIdx.x >> 5] = v;
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned long long t = 0;
    for (int w = 0; w < kThreads / 32; ++w) t += s_part[w];
    if (t) atomicAdd(dst, t);
  }
  __syncthreads();
}

// Slot of this thread's item in the list counted by *counter (every thread
// of the block calls it; one atomic per block and call).
__device__ __forceinline__ unsigned long long block_append(bool emit,
                                                         unsigned long long *counter) {
  __shared__ unsigned s_off[kThreads / 32];
  __shared__ unsigned long long s_base;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned m = __ballot_sync(0xffffffffu, emit);
  if (lane == 0) s_off[w] = __popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    unsigned tot = 0;
    for (int i = 0; i < kThreads / 32; ++i) {
      const unsigned c = s_off[i];
      s_off[i] = tot;
      tot += c;
    }
    s_base = tot ? atomicAdd(counter, (unsigned long long)tot) : 0ull;
  }
  __syncthreads();
  const unsigned long long slot = s_base + s_off[w] + __popc(m & ((1u << lane) - 1u));
  __syncthreads();  // s_off / s_base are reused by the next call
  return slot;
}

// anc_st / anc_en / anc_slot: the anchors' starts, ends and active slots,
// staged in shared memory when kSmem (n_anc * 12 bytes).
// Sorted anchors: the starts and the bucket table (first, nb entries) are
// staged in shared memory when kSmem ((n_anc + nb) * 4 bytes); ends and
// slots are read once per lookup through L1.  Unsorted anchors (first ==
// NULL): the reference's scan.
template <bool kSmem>
__global__ void __launch_bounds__(kThreads)
long_map(int n, int n_long, const int *__restrict__ ls, const int *__restrict__ le,
         const int *__restrict__ anc_st, const int *__restrict__ anc_en,
         const int *__restrict__ anc_slot, int n_anc, const int *__restrict__ bucket_first,
         int nb, int pos0, int shift, int base_idx, uint64_t *__restrict__ keys,
         uint32_t *__restrict__ idx, unsigned long long *__restrict__ cnt) {
  extern __shared__ int s_anc[];
  const int *st = anc_st, *first = bucket_first;
  if (kSmem) {
    for (int i = threadIdx.x; i < n_anc; i += blockDim.x) s_anc[i] = anc_st[i];
    for (int i = threadIdx.x; i < nb; i += blockDim.x) s_anc[n_anc + i] = bucket_first[i];
    __syncthreads();
    st = s_anc;
    first = s_anc + n_anc;
  }
  const uint64_t none = (uint64_t)n * (uint64_t)n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  unsigned oor = 0, inactive = 0;
  // every thread of a block runs the same iterations (block-wide counts)
  for (long long base = (long long)blockIdx.x * blockDim.x; base < n_long; base += stride) {
    const long long k = base + threadIdx.x;
    if (k < n_long) {
      uint64_t key = none;
      const int pa = ls[k], pb = le[k];
      const int ia = bucket_first ? find_anchor_bucket(st, anc_en, first, n_anc, nb, pos0, shift, pa)
                                  : find_anchor_scan(st, anc_en, n_anc, pa);
      const int ib = bucket_first ? find_anchor_bucket(st, anc_en, first, n_anc, nb, pos0, shift, pb)
                                  : find_anchor_scan(st, anc_en, n_anc, pb);
      if (ia < 0 || ib < 0 || ia == ib) {
        ++oor;
      } else {
        const int a = anc_slot[ia], b = anc_slot[ib];
        if (a < 0 || b < 0) {
          ++inactive;
        } else {
          key = pair_key(a, b, n);
        }
      }
      keys[base_idx + k] = key;
      idx[base_idx + k] = (uint32_t)k;
    }
  }
  block_count(oor, cnt + kCntOor);
  block_count(inactive, cnt + kCntInactive);
}

// One thread per pair (its first sorted entry): the value the arcs of the
// active clusters left there (-1: none; 0 on the diagonal unless an arc
// wrote it), then the pair's long arcs in order: a value >= 0 is a
// collision, anything else is overwritten (:5575-5585).
__global__ void __launch_bounds__(kThreads)
long_resolve(int n, int n_items, const uint64_t *__restrict__ keys,
             const uint32_t *__restrict__ idx, const int *__restrict__ lsc,
             const float *__restrict__ memo, CountToDist c, const float *__restrict__ sval,
             int pair_base, uint64_t *__restrict__ pkey, float *__restrict__ pval,
             unsigned long long *__restrict__ cnt) {
  const uint64_t none = (uint64_t)n * (uint64_t)n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  unsigned applied = 0, collided = 0;
  // every thread of a block runs the same iterations (block-wide appends)
  for (long long base = (long long)blockIdx.x * blockDim.x; base < n_items; base += stride) {
    const long long p = base + threadIdx.x;
    bool emit = false;
    uint64_t k = 0;
    float cur = 0.0f;
    if (p < n_items) {
      k = keys[p];
      if (k != none && (p == 0 || keys[p - 1] != k)) {
        const int a = (int)(k / (uint64_t)n), b = (int)(k % (uint64_t)n);
        cur = a == b ? 0.0f : -1.0f;
        long long q = p;
        bool held = false;  // an arc of the active clusters holds a distance >= 0
        const uint32_t i0 = idx[q];
        if (i0 & kShort) {
          cur = sval[i0 & ~kShort];
          held = cur >= 0.0f;
          ++q;
        }
        for (; q < n_items && keys[q] == k; ++q) {
          if (cur >= 0.0f) {
            ++collided;
          } else {
            cur = freq_to_distance_dev(lsc[idx[q]], memo, c);  // only when applied
            ++applied;
          }
        }
        emit = !held && a != b && cur >= 0.0f;
      }
    }
    // one append per block and iteration
    if (__syncthreads_or(emit)) {
      const unsigned long long slot = block_append(emit, cnt + kCntPairs);
      if (emit) {
        pkey[pair_base + slot] = k;
        pval[pair_base + slot] = cur;
      }
    }
  }
  block_count(applied, cnt + kCntApplied);
  block_count(collided, cnt + kCntCollision);
}

// long_resolve when every distance is >= 0 (memo entries and
// countToDistBaseLevel >= 0, countToDistScale > 0): the first value written
// to a pair stays, so a long arc is written exactly when it is the first
// entry of its pair off the diagonal, and every other long arc collides.
// One entry per thread, no walk.
__global__ void __launch_bounds__(kThreads)
long_resolve_first(int n, int n_items, const uint64_t *__restrict__ keys,
                   const uint32_t *__restrict__ idx, const int *__restrict__ lsc,
                   const float *__restrict__ memo, CountToDist c, int pair_base,
                   uint64_t *__restrict__ pkey, float *__restrict__ pval,
                   unsigned long long *__restrict__ cnt) {
  const uint64_t none = (uint64_t)n * (uint64_t)n;
  const long long stride = (long long)gridDim.x * blockDim.x;
  unsigned applied = 0, collided = 0;
  // every thread of a block runs the same iterations (block-wide appends)
  for (long long base = (long long)blockIdx.x * blockDim.x; base < n_items; base += stride) {
    const long long p = base + threadIdx.x;
    bool emit = false;
    uint64_t k = 0;
    float cur = 0.0f;
    if (p < n_items) {
      k = keys[p];
      const uint32_t i = idx[p];
      if (k != none && !(i & kShort)) {
        const bool first = p == 0 || keys[p - 1] != k;
        if (first && k % (uint64_t)(n + 1) != 0) {  // not the diagonal (k = a * (n + 1))
          ++applied;
          cur = freq_to_distance_dev(lsc[i], memo, c);
          emit = true;
        } else {
          ++collided;
        }
      }
    }
    if (__syncthreads_or(emit)) {
      const unsigned long long slot = block_append(emit, cnt + kCntPairs);
      if (emit) {
        pkey[pair_base + slot] = k;
        pval[pair_base + slot] = cur;
      }
    }
  }
  block_count(applied, cnt + kCntApplied);
  block_count(collided, cnt + kCntCollision);
}

// Heatmap::getDiagonalSize: the smallest j - i (j >= i) with heat > 1e-6.
// One block per row at a time, the row's columns across the threads.
__global__ void heat_diag(int n, const float *__restrict__ heat, int *__restrict__ w) {
  int best = INT_MAX;
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const float *row = heat + (size_t)i * n;
    for (int j = i + threadIdx.x; j < n; j += blockDim.x)
      if (row[j] > __uint_as_float(0x358637bdu)) {
        best = min(best, j - i);
        break;  // later columns of this thread are further out
      }
  }
  best = __reduce_min_sync(0xffffffffu, best);
  if ((threadIdx.x & 31) == 0 && best != INT_MAX) atomicMin(w, best);
}

// Heatmap::getRange: the largest value over j >= i + w, from 0.  Positive
// floats order as their bit patterns.
__global__ void heat_max(int n, const float *__restrict__ heat, const int *__restrict__ w,
                         int *__restrict__ max_bits) {
  const int d = *w == INT_MAX ? 0 : *w;
  int best = 0;
  for (int i = blockIdx.x; i < n; i += gridDim.x) {
    const float *row = heat + (size_t)i * n;
    for (long long j = (long long)i + d + threadIdx.x; j < n; j += blockDim.x) {
      const float v = row[j];
      if (v > 0.0f) best = max(best, __float_as_int(v));
    }
  }
  best = __reduce_max_sync(0xffffffffu, best);
  if ((threadIdx.x & 31) == 0 && best) atomicMax(max_bits, best);
}

// Both directions of every pair; with the anchor heatmap, the reference's
// v *= 1 - min(1, heat / max * influence) on the upper entry (:5611-5622).
__global__ void pair_emit(int n_pairs, const uint64_t *__restrict__ pkey,
                          const float *__restrict__ pval, int n, const float *__restrict__ heat,
                          const int *__restrict__ max_bits, float influence,
                          uint64_t *__restrict__ dkey, float *__restrict__ dval) {
  float mx = 0.0f;
  bool use = false;
  if (heat) {
    mx = __int_as_float(*max_bits);
    use = mx > __uint_as_float(0x358637bdu);
  }
  for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < n_pairs; f += gridDim.x * blockDim.x) {
    const uint64_t k = pkey[f];
    const uint64_t a = k / (uint64_t)n, b = k % (uint64_t)n;
    float v = pval[f];
    if (use) {
      float s = __fmul_rn(__fdiv_rn(heat[(size_t)a * n + b], mx), influence);
      if (s > 1.0f) s = 1.0f;
      v = __fmul_rn(v, __fsub_rn(1.0f, s));
    }
    dkey[2 * f] = k;
    dval[2 * f] = v;
    dkey[2 * f + 1] = b * (uint64_t)n + a;
    dval[2 * f + 1] = v;
  }
}

__global__ void csr_finish(int n, int nnz, const uint64_t *__restrict__ dkey,
                           int *__restrict__ row_ptr, int *__restrict__ col) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, stride = gridDim.x * blockDim.x;
  for (int p = tid; p < nnz; p += stride) col[p] = (int)(dkey[p] % (uint64_t)n);
  for (int r = tid; r <= n; r += stride) {
    const uint64_t want = (uint64_t)r * (uint64_t)n;
    int lo = 0, hi = nnz;
    while (lo < hi) {
      const int mid = (lo + hi) >> 1;
      if (dkey[mid] < want) lo = mid + 1;
      else hi = mid;
    }
    row_ptr[r] = lo;
  }
}

// Stream-ordered allocations released together.
struct Arena {
  cudaStream_t s;
  std::vector<void *> ptrs;
  cudaError_t err = cudaSuccess;
  explicit Arena(cudaStream_t st) : s(st) {}
  template <typename T> T *get(size_t count) {
    if (err != cudaSuccess) return nullptr;
    void *p = nullptr;
    err = cudaMallocAsync(&p, std::max<size_t>(count, 1) * sizeof(T), s);
    if (err != cudaSuccess) return nullptr;
    ptrs.push_back(p);
    return static_cast<T *>(p);
  }
  template <typename T> T *put(const T *host, size_t count) {
    T *d = get<T>(count);
    if (d && count) err = cudaMemcpyAsync(d, host, count * sizeof(T), cudaMemcpyHostToDevice, s);
    return d;
  }
  ~Arena() {
    for (void *p : ptrs) cudaFreeAsync(p, s);
  }
};

int grid_for(long long items, int threads, int sm_count) {
  const long long want = (items + threads - 1) / threads;
  return (int)std::max<long long>(1, std::min<long long>(want, 8LL * sm_count));
}

}  // namespace

}  // namespace pmmc

using namespace pmmc;

extern "C" pmmc_status pmmc_anchor_targets(pmmc_ctx *ctx, const pmmc_anchor_targets_problem *pr,
                                           int *row_ptr, int *col, float *target, int64_t cap,
                                           int64_t *nnz, pmmc_anchor_targets_stats *stats,
                                           double *kernel_ms) {
  if (!ctx || !pr || !nnz || pr->n < 0 || pr->n_arcs < 0 || pr->n_long < 0 ||
      pr->n_anchors < 0 || !pr->freq_memo)
    return fail(ctx, PMMC_ERR_INVALID, "anchor targets: bad arguments");
  const int n = pr->n;
  if (n > 0 && (!pr->active || !pr->arc_ptr))
    return fail(ctx, PMMC_ERR_INVALID, "anchor targets: active region without arrays");
  const int n_sarcs = n > 0 ? pr->arc_ptr[n] : 0;
  if (n_sarcs > 0 && (!pr->arc_idx || !pr->arc_start || !pr->arc_end || !pr->arc_score))
    return fail(ctx, PMMC_ERR_INVALID, "anchor targets: arcs without arrays");
  const bool use_long = pr->n_long > 0 && pr->n_anchors > 0;
  if (use_long && (!pr->long_start || !pr->long_end || !pr->long_score || !pr->anchor_start ||
                   !pr->anchor_end))
    return fail(ctx, PMMC_ERR_INVALID, "anchor targets: long arcs without arrays");
  const CountToDist c2d{pr->count_a, pr->count_scale, pr->count_shift, pr->count_base};

  // slot of every cluster (the last position of a repeated cluster wins)
  std::unordered_map<int, int> slot;
  slot.reserve((size_t)n * 2 + 16);
  for (int i = 0; i < n; ++i) slot[pr->active[i]] = i;

  // arcs of the active clusters, in the reference's order (:5512-5539)
  struct Write {
    uint64_t key;
    int order;
    float v;
  };
  std::vector<Write> writes;
  for (int i = 0; i < n; ++i) {
    const int ai = pr->active[i];
    for (int k = pr->arc_ptr[i]; k < pr->arc_ptr[i + 1]; ++k) {
      const int arc = pr->arc_idx[k];
      if (arc < 0 || arc >= pr->n_arcs)
        return fail(ctx, PMMC_ERR_INVALID, "anchor targets: arc index %d out of range", arc);
      int other = -1;
      if (pr->arc_start[arc] == ai) other = pr->arc_end[arc];
      else if (pr->arc_end[arc] == ai) other = pr->arc_start[arc];
      if (other == -1)
        return fail(ctx, PMMC_ERR_INVALID, "anchor targets: arc %d does not touch cluster %d",
                    arc, ai);
      if (other < ai) continue;
      const float e = freq_to_distance_host(pr->arc_score[arc], pr->freq_memo, c2d);
      const int a = slot[ai];
      const int b = slot[other];  // inserted as slot 0 when not active
      const uint64_t key = pair_key(a, b, n);
      writes.push_back({key, (int)writes.size(), e});
    }
  }
  std::sort(writes.begin(), writes.end(), [](const Write &x, const Write &y) {
    return x.key != y.key ? x.key < y.key : x.order < y.order;
  });
  std::vector<uint64_t> skey;  // every pair an arc wrote (diagonal too), its last value
  std::vector<uint32_t> sidx;
  std::vector<float> sval;
  for (size_t w = 0; w < writes.size(); ++w) {
    if (w + 1 < writes.size() && writes[w + 1].key == writes[w].key) continue;
    sidx.push_back(kShort | (uint32_t)skey.size());
    skey.push_back(writes[w].key);
    sval.push_back(writes[w].v);
  }
  std::vector<uint64_t> pkey_h;  // the ones that hold a distance
  std::vector<float> pval_h;
  for (size_t w = 0; w < skey.size(); ++w)
    if (sval[w] >= 0.0f && skey[w] / (uint64_t)n != skey[w] % (uint64_t)n) {
      pkey_h.push_back(skey[w]);
      pval_h.push_back(sval[w]);
    }

  // every distance >= 0 (and none NaN): no value written to a pair is ever
  // replaced.  scale > 0 keeps 0 / exp(..) = 0 / 0 out.
  bool nonneg = pr->count_base >= 0.0f && pr->count_scale > 0.0f &&
                pr->count_a == pr->count_a && pr->count_shift == pr->count_shift;
  for (int f = 1; f <= 100; ++f) nonneg = nonneg && pr->freq_memo[f] >= 0.0f;

  // anchor index -> active slot through the same map (:5556-5561)
  std::vector<int> anc_slot, bucket;
  int sorted = 1, nb = 0, abase = 0, shift = 0;
  if (use_long) {
    anc_slot.assign(pr->n_anchors, -1);
    for (const auto &kv : slot)
      if (kv.first >= pr->first_cluster && kv.first - pr->first_cluster < pr->n_anchors)
        anc_slot[kv.first - pr->first_cluster] = kv.second;
    for (int i = 1; i < pr->n_anchors; ++i)
      if (!(pr->anchor_start[i] > pr->anchor_start[i - 1] &&
            pr->anchor_start[i] > pr->anchor_end[i - 1]))
        sorted = 0;
    if (sorted) {
      // buckets of 2^shift bp over the starts, at most one per anchor
      abase = pr->anchor_start[0];
      const long long span = (long long)pr->anchor_start[pr->n_anchors - 1] - abase;
      while ((span >> shift) + 1 > pr->n_anchors) ++shift;
      nb = (int)((span >> shift) + 1);
      bucket.assign(nb, -1);
      int i = -1;
      for (int b = 0; b < nb; ++b) {
        const long long at = (long long)abase + ((long long)b << shift);
        while (i + 1 < pr->n_anchors && pr->anchor_start[i + 1] <= at) ++i;
        bucket[b] = i;
      }
    }
  }

  cudaStream_t s = ctx->stream;
  const int T = kThreads;
  const int bits = key_bits(n);
  Arena ar(s);
  const int n_long = use_long ? pr->n_long : 0;
  const size_t n_pair_cap = pkey_h.size() + (size_t)n_long;
  unsigned long long *d_cnt = ar.get<unsigned long long>(5);
  uint64_t *d_pkey = ar.get<uint64_t>(n_pair_cap);
  float *d_pval = ar.get<float>(n_pair_cap);
  if (ar.err == cudaSuccess) ar.err = cudaMemsetAsync(d_cnt, 0, 5 * sizeof(unsigned long long), s);
  if (ar.err == cudaSuccess && !pkey_h.empty()) {
    ar.err = cudaMemcpyAsync(d_pkey, pkey_h.data(), pkey_h.size() * 8, cudaMemcpyHostToDevice, s);
    if (ar.err == cudaSuccess)
      ar.err = cudaMemcpyAsync(d_pval, pval_h.data(), pval_h.size() * 4, cudaMemcpyHostToDevice, s);
  }
  const int *d_ls = nullptr, *d_le = nullptr, *d_lsc = nullptr, *d_ast = nullptr,
            *d_aen = nullptr, *d_aslot = nullptr, *d_first = nullptr;
  const float *d_memo = nullptr, *d_sval = nullptr;
  uint64_t *d_keys = nullptr, *d_keys2 = nullptr;
  uint32_t *d_idx = nullptr, *d_idx2 = nullptr;
  const int n_short = (int)skey.size();
  const int n_items = n_short + n_long;  // sorted entries: pairs written, then long arcs
  if (n_long > 0) {
    d_ls = ar.put(pr->long_start, n_long);
    d_le = ar.put(pr->long_end, n_long);
    d_lsc = ar.put(pr->long_score, n_long);
    d_ast = ar.put(pr->anchor_start, pr->n_anchors);
    d_aen = ar.put(pr->anchor_end, pr->n_anchors);
    d_aslot = ar.put(anc_slot.data(), anc_slot.size());
    if (sorted) d_first = ar.put(bucket.data(), bucket.size());
    d_memo = ar.put(pr->freq_memo, 101);
    d_sval = ar.put(sval.data(), sval.size());
    d_keys = ar.get<uint64_t>(n_items);
    d_keys2 = ar.get<uint64_t>(n_items);
    d_idx = ar.get<uint32_t>(n_items);
    d_idx2 = ar.get<uint32_t>(n_items);
    if (ar.err == cudaSuccess && n_short > 0) {
      ar.err = cudaMemcpyAsync(d_keys, skey.data(), 8 * (size_t)n_short, cudaMemcpyHostToDevice,
                               s);
      if (ar.err == cudaSuccess)
        ar.err = cudaMemcpyAsync(d_idx, sidx.data(), 4 * (size_t)n_short,
                                 cudaMemcpyHostToDevice, s);
    }
  }
  const float *d_heat = nullptr;
  int *d_hstat = nullptr;  // diagonal size, max bits
  if (pr->anchor_heat && n > 0) {
    d_heat = ar.put(pr->anchor_heat, (size_t)n * n);
    d_hstat = ar.get<int>(2);
    const int init[2] = {INT_MAX, 0};
    if (ar.err == cudaSuccess)
      ar.err = cudaMemcpyAsync(d_hstat, init, sizeof(init), cudaMemcpyHostToDevice, s);
  }
  size_t tmp1 = 0;
  if (n_long > 0)
    cub::DeviceRadixSort::SortPairs(nullptr, tmp1, d_keys, d_keys2, d_idx, d_idx2, n_items, 0,
                                    bits, s);
  void *d_tmp1 = ar.get<unsigned char>(tmp1);
  if (ar.err != cudaSuccess)
    return fail(ctx, ar.err == cudaErrorMemoryAllocation ? PMMC_ERR_NOMEM : PMMC_ERR_CUDA,
                "anchor targets: %s", cudaGetErrorString(ar.err));

  // ev: phase one (map, sort, resolve, heatmap passes), phase two (assembly)
  cudaEvent_t ev[6];
  for (auto &x : ev) cudaEventCreate(&x);
  struct EvGuard {
    cudaEvent_t *e;
    ~EvGuard() {
      for (int i = 0; i < 6; ++i) cudaEventDestroy(e[i]);
    }
  } evg{ev};
  cudaEventRecord(ev[0], s);
  cudaError_t e = cudaSuccess;
  if (n_long > 0) {
    // starts and buckets in shared memory up to 96 KB, else through L1/L2
    const size_t smem = 4 * ((size_t)pr->n_anchors + (size_t)nb);
    if (sorted && smem <= 96 * 1024) {
      // set on every call: the attribute belongs to the current device
      cudaFuncSetAttribute(long_map<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           96 * 1024);
      int per_sm = 0;
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, long_map<true>, T, smem);
      const int grid = (int)std::min<long long>((n_long + T - 1) / T,
                                                (long long)std::max(1, per_sm) * ctx->sm_count);
      long_map<true><<<std::max(grid, 1), T, smem, s>>>(
          n, n_long, d_ls, d_le, d_ast, d_aen, d_aslot, pr->n_anchors, d_first, nb, abase,
          shift, n_short, d_keys, d_idx, d_cnt);
    } else {
      long_map<false><<<grid_for(n_long, T, ctx->sm_count), T, 0, s>>>(
          n, n_long, d_ls, d_le, d_ast, d_aen, d_aslot, pr->n_anchors,
          sorted ? d_first : nullptr, nb, abase, shift, n_short, d_keys, d_idx, d_cnt);
    }
  }
  cudaEventRecord(ev[1], s);
  if (n_long > 0)
    e = cub::DeviceRadixSort::SortPairs(d_tmp1, tmp1, d_keys, d_keys2, d_idx, d_idx2, n_items,
                                        0, bits, s);
  cudaEventRecord(ev[2], s);
  if (n_long > 0 && e == cudaSuccess)
  {
    if (nonneg)
      long_resolve_first<<<grid_for(n_items, T, ctx->sm_count), T, 0, s>>>(
          n, n_items, d_keys2, d_idx2, d_lsc, d_memo, c2d, (int)pkey_h.size(), d_pkey, d_pval,
          d_cnt);
    else
      long_resolve<<<grid_for(n_items, T, ctx->sm_count), T, 0, s>>>(
          n, n_items, d_keys2, d_idx2, d_lsc, d_memo, c2d, d_sval, (int)pkey_h.size(), d_pkey,
          d_pval, d_cnt);
  }
  cudaEventRecord(ev[3], s);
  if (d_heat && e == cudaSuccess) {
    const int rows = std::max(1, std::min(n, 8 * ctx->sm_count));
    heat_diag<<<rows, T, 0, s>>>(n, d_heat, d_hstat);
    heat_max<<<rows, T, 0, s>>>(n, d_heat, d_hstat, d_hstat + 1);
  }
  cudaEventRecord(ev[4], s);
  unsigned long long cnt[5] = {0, 0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaGetLastError();
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(cnt, d_cnt, sizeof(cnt), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(ctx, PMMC_ERR_CUDA, "anchor targets: %s", cudaGetErrorString(e));
  float t_map = 0.0f, t_sort = 0.0f, t_res = 0.0f, t_heat = 0.0f;
  cudaEventElapsedTime(&t_map, ev[0], ev[1]);
  cudaEventElapsedTime(&t_sort, ev[1], ev[2]);
  cudaEventElapsedTime(&t_res, ev[2], ev[3]);
  cudaEventElapsedTime(&t_heat, ev[3], ev[4]);
  const long long n_pairs = (long long)pkey_h.size() + (long long)cnt[kCntPairs];
  const long long total = 2 * n_pairs;
  *nnz = total;
  if (stats) {
    stats->applied = (int64_t)cnt[kCntApplied];
    stats->out_of_range = (int64_t)cnt[kCntOor];
    stats->inactive = (int64_t)cnt[kCntInactive];
    stats->collision = (int64_t)cnt[kCntCollision];
    stats->ms_map = t_map;
    stats->ms_sort = t_sort;
    stats->ms_resolve = t_res;
    stats->ms_assemble = t_heat;
  }
  if (!row_ptr || !col || !target || cap < total || total > INT_MAX) {
    if (total > INT_MAX)
      return fail(ctx, PMMC_ERR_INVALID, "anchor targets: %lld entries overflow int", total);
    return PMMC_OK;  // size query
  }
  uint64_t *d_dkey = ar.get<uint64_t>(total), *d_dkey2 = ar.get<uint64_t>(total);
  float *d_dval = ar.get<float>(total), *d_dval2 = ar.get<float>(total);
  int *d_row = ar.get<int>((size_t)n + 1), *d_col = ar.get<int>(total);
  size_t tmp2 = 0;
  if (total > 0)
    cub::DeviceRadixSort::SortPairs(nullptr, tmp2, d_dkey, d_dkey2, d_dval, d_dval2, (int)total,
                                    0, bits, s);
  void *d_tmp2 = ar.get<unsigned char>(tmp2);
  e = ar.err;
  cudaEventRecord(ev[4], s);
  if (e == cudaSuccess && n_pairs > 0) {
    pair_emit<<<grid_for(n_pairs, T, ctx->sm_count), T, 0, s>>>(
        (int)n_pairs, d_pkey, d_pval, n, d_heat, d_hstat ? d_hstat + 1 : nullptr,
        pr->anchor_influence, d_dkey, d_dval);
    e = cub::DeviceRadixSort::SortPairs(d_tmp2, tmp2, d_dkey, d_dkey2, d_dval, d_dval2,
                                        (int)total, 0, bits, s);
  }
  if (e == cudaSuccess) {
    csr_finish<<<grid_for(std::max<long long>(total, n + 1), T, ctx->sm_count), T, 0, s>>>(
        n, (int)total, d_dkey2, d_row, d_col);
    e = cudaGetLastError();
  }
  cudaEventRecord(ev[5], s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(row_ptr, d_row, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && total > 0)
    e = cudaMemcpyAsync(col, d_col, sizeof(int) * total, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && total > 0)
    e = cudaMemcpyAsync(target, d_dval2, sizeof(float) * total, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess)
    return fail(ctx, e == cudaErrorMemoryAllocation ? PMMC_ERR_NOMEM : PMMC_ERR_CUDA,
                "anchor targets: %s", cudaGetErrorString(e));
  float t_asm = 0.0f;
  cudaEventElapsedTime(&t_asm, ev[4], ev[5]);
  if (stats) stats->ms_assemble = t_heat + t_asm;
  if (kernel_ms) *kernel_ms = (double)t_map + t_sort + t_res + t_heat + t_asm;
  return PMMC_OK;
}
