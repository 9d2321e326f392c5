// distmap.cu -- expected-distance heatmap from a contact heatmap.
//
// LooperSolver::createDistanceHeatmap (LooperSolver.hpp:3042-3085) turns the
// contact map of a level into the expected-distance map the heatmap annealer
// fits: for i <= j, d = scale * c^power when c >= 1e-6 (0 below, -1 inside
// the diagonal band |i - j| < diag), mirrored to the lower triangle; then
// every value above avg * stretching is clamped to it, avg being
// Heatmap::getAvg of the distance map (the mean over j >= i + w, w the first
// diagonal holding a value above 1e-6, Heatmap.hpp:356-367, 440-451).  The
// reference does this on one host core in O(n^2) before every heatmap level.
//
// Two passes over the upper triangle, 64 x 64 tiles (coalesced rows):
//   pass 1  per tile: the distances (written unclamped to the upper
//           triangle), the sum of the positive ones (FP64 per warp), the
//           number of band entries, the smallest diagonal offset holding a
//           positive distance; one partial per tile, reduced in a fixed order
//           by a single block (deterministic), which derives avg and the clamp;
//   pass 2  per tile: the upper triangle read back, clamped in place and
//           written, through shared memory, to its mirror tile.
// Per upper-triangle entry: 4 bytes of contact read and 4 bytes written in
// pass 1, 4 bytes read in pass 2; per lower-triangle entry 4 bytes written;
// the power function runs once per entry.
#include <cmath>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace pmmc {

constexpr int kTile = 64;     // tile edge
constexpr int kRows = 4;      // thread rows of a 256-thread block (64 x 4)

// (double)c < 1e-6 and (double)d > 1e-6, as the reference compares a float
// with the double constant, in float: 1e-6 lies between the floats
// 0x358637bd and 0x358637be.
__device__ __forceinline__ bool below_1e6(float c) {
  return c < __uint_as_float(0x358637beu);
}
__device__ __forceinline__ bool above_1e6(float d) {
  return d > __uint_as_float(0x358637bdu);
}

__device__ __forceinline__ float contact_to_dist(float c, int i, int j, int diag, float scale,
                                                 float power) {
  if (below_1e6(c)) return 0.0f;
  if (abs(i - j) < diag) return -1.0f;
  return scale * powf(c, power);
}

struct DistPartial {
  double sum_pos;   // positive distances of the tile (upper triangle)
  long long n_neg;  // band entries (-1) of the tile (upper triangle)
  int min_off;      // smallest j - i with a distance above 1e-6 (INT_MAX: none)
  int pad;
};

// Tile blockIdx.x of the upper triangle; its partial goes to part[blockIdx.x].
__global__ void __launch_bounds__(kTile * kRows)
distmap_pass1(const float *__restrict__ c, int n, int nt, int diag, float scale, float power,
              DistPartial *__restrict__ part, float *__restrict__ dist) {
  __shared__ double s_sum[kTile * kRows / 32];
  __shared__ long long s_neg[kTile * kRows / 32];
  __shared__ int s_min[kTile * kRows / 32];
  const int2 tb = upper_tile(blockIdx.x, nt);
  const int bi = tb.x, bj = tb.y;
  const int tx = threadIdx.x % kTile, ty = threadIdx.x / kTile;
  const int j = bj * kTile + tx;
  float sum = 0.0f;   // at most 16 terms per thread; widened to FP64 below
  int neg = 0;
  int mo = 0x7fffffff;
#pragma unroll 4
  for (int r = ty; r < kTile; r += kRows) {
    const int i = bi * kTile + r;
    if (i < n && j < n && j >= i) {
      const float d = contact_to_dist(c[(size_t)i * n + j], i, j, diag, scale, power);
      dist[(size_t)i * n + j] = d;  // unclamped; pass 2 clamps and mirrors
      sum += d > 0.0f ? d : 0.0f;
      neg += d == -1.0f ? 1 : 0;
      if (above_1e6(d)) mo = min(mo, j - i);
    }
  }
  double ds = warp_sum_d((double)sum);
  long long ng = neg;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    ng += __shfl_xor_sync(0xffffffffu, ng, o);
    mo = min(mo, __shfl_xor_sync(0xffffffffu, mo, o));
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    s_sum[w] = ds;
    s_neg[w] = ng;
    s_min[w] = mo;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    DistPartial p{0.0, 0, 0x7fffffff, 0};
    for (int k = 0; k < kTile * kRows / 32; ++k) {
      p.sum_pos += s_sum[k];
      p.n_neg += s_neg[k];
      p.min_off = min(p.min_off, s_min[k]);
    }
    part[blockIdx.x] = p;
  }
}

// One block: the partials of the upper-triangle tiles (thread t takes every
// blockDim-th one from t, then a fixed-order combination: deterministic),
// avg = Heatmap::getAvg of the map and the clamp value.
__global__ void distmap_finish(const DistPartial *__restrict__ part, int nt, int n,
                               float stretching, float *__restrict__ out2) {
  __shared__ double s_sum[32];
  __shared__ long long s_neg[32];
  __shared__ int s_min[32];
  const long long total = (long long)nt * (nt + 1) / 2;
  double sum = 0.0;
  long long neg = 0;
  int mo = 0x7fffffff;
  for (long long k = threadIdx.x; k < total; k += blockDim.x) {
    sum += part[k].sum_pos;
    neg += part[k].n_neg;
    mo = min(mo, part[k].min_off);
  }
  for (int o = 16; o > 0; o >>= 1) {
    sum += shfl_xor_d(sum, o);
    neg += __shfl_xor_sync(0xffffffffu, neg, o);
    mo = min(mo, __shfl_xor_sync(0xffffffffu, mo, o));
  }
  if ((threadIdx.x & 31) == 0) {
    s_sum[threadIdx.x >> 5] = sum;
    s_neg[threadIdx.x >> 5] = neg;
    s_min[threadIdx.x >> 5] = mo;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    long long ng = 0;
    int m = 0x7fffffff;
    for (int k = 0; k < (int)(blockDim.x >> 5); ++k) {
      t += s_sum[k];
      ng += s_neg[k];
      m = min(m, s_min[k]);
    }
    // getDiagonalSize is 0 when no entry exceeds 1e-6; the average then also
    // takes the band entries (-1) on and above the diagonal
    int w = m;
    double sm = t;
    if (m == 0x7fffffff) {
      w = 0;
      sm = -(double)ng;
    }
    const double cnt = (double)(n - w) * (double)(n - w + 1) * 0.5;
    const float avg = (float)(sm / cnt);
    out2[0] = avg;
    out2[1] = avg * stretching;
  }
}

__global__ void __launch_bounds__(kTile * kRows)
distmap_pass2(int n, int nt, const float *__restrict__ stats, float *__restrict__ dist) {
  __shared__ float tile[kTile][kTile + 1];
  const int2 tb = upper_tile(blockIdx.x, nt);
  const int bi = tb.x, bj = tb.y;
  const float maxd = stats[1];
  const int tx = threadIdx.x % kTile, ty = threadIdx.x / kTile;
  const int j = bj * kTile + tx;
#pragma unroll 4
  for (int r = ty; r < kTile; r += kRows) {
    const int i = bi * kTile + r;
    float d = 0.0f;
    // the upper triangle defines both halves; below the diagonal of a
    // diagonal tile the mirror writes the value
    if (i < n && j < n && j >= i) {
      d = dist[(size_t)i * n + j];
      if (d > maxd) {
        d = maxd;
        dist[(size_t)i * n + j] = d;
      }
    }
    tile[r][tx] = d;
  }
  __syncthreads();
  // mirror: element (i, j) -> (j, i); thread tx now walks i within the tile
  const int i2 = bi * kTile + tx;
#pragma unroll 4
  for (int r = ty; r < kTile; r += kRows) {
    const int j2 = bj * kTile + r;
    if (i2 < n && j2 < n && j2 > i2) dist[(size_t)j2 * n + i2] = tile[tx][r];
  }
}

}  // namespace pmmc

using namespace pmmc;

namespace {

pmmc_status distmap_run(pmmc_ctx *ctx, int n, const float *d_c, int diag, float scale,
                        float power, float stretching, float *d_dist, float *d_stats,
                        cudaStream_t s) {
  const int nt = (n + kTile - 1) / kTile;
  if (nt > 65535) return fail(ctx, PMMC_ERR_INVALID, "distance heatmap: n too large");
  // (nt x (nt + 1) / 2 tiles stay below the 2^31 - 1 blocks of a 1-D grid)
  DistPartial *d_part = nullptr;
  const long long tiles = (long long)nt * (nt + 1) / 2;
  PMMC_CUDA(ctx, cudaMallocAsync(&d_part, sizeof(DistPartial) * (size_t)tiles, s));
  const unsigned grid = (unsigned)tiles;
  distmap_pass1<<<grid, kTile * kRows, 0, s>>>(d_c, n, nt, diag, scale, power, d_part, d_dist);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    distmap_finish<<<1, 1024, 0, s>>>(d_part, nt, n, stretching, d_stats);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    distmap_pass2<<<grid, kTile * kRows, 0, s>>>(n, nt, d_stats, d_dist);
    e = cudaGetLastError();
  }
  cudaFreeAsync(d_part, s);
  if (e != cudaSuccess)
    return fail(ctx, PMMC_ERR_CUDA, "distance heatmap: %s", cudaGetErrorString(e));
  return PMMC_OK;
}

}  // namespace

extern "C" pmmc_status pmmc_distance_heatmap_device(pmmc_ctx *ctx, int n, const float *contact,
                                                    int diag, float scale, float power,
                                                    float stretching, float *dist,
                                                    float *stats, void *stream) {
  if (!ctx || n < 1 || !contact || !dist || !stats || diag < 0)
    return fail(ctx, PMMC_ERR_INVALID, "distance heatmap: bad arguments");
  return distmap_run(ctx, n, contact, diag, scale, power, stretching, dist, stats,
                     stream ? (cudaStream_t)stream : ctx->stream);
}

extern "C" pmmc_status pmmc_distance_heatmap(pmmc_ctx *ctx, int n, const float *contact,
                                             int diag, float scale, float power,
                                             float stretching, float *dist_out,
                                             float *avg_out, float *max_out,
                                             double *kernel_ms) {
  if (!ctx || n < 1 || !contact || !dist_out || diag < 0)
    return fail(ctx, PMMC_ERR_INVALID, "distance heatmap: bad arguments");
  cudaStream_t s = ctx->stream;
  const size_t bytes = sizeof(float) * (size_t)n * n;
  float *d_c = nullptr, *d_d = nullptr, *d_st = nullptr;
  cudaError_t e = cudaMallocAsync(&d_c, bytes, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_d, bytes, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_st, 2 * sizeof(float), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_c, contact, bytes, cudaMemcpyHostToDevice, s);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  pmmc_status st = PMMC_OK;
  if (e == cudaSuccess) {
    cudaEventRecord(e0, s);
    st = distmap_run(ctx, n, d_c, diag, scale, power, stretching, d_d, d_st, s);
    cudaEventRecord(e1, s);
  }
  float stats[2] = {0.0f, 0.0f};
  if (e == cudaSuccess && st == PMMC_OK)
    e = cudaMemcpyAsync(dist_out, d_d, bytes, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess && st == PMMC_OK)
    e = cudaMemcpyAsync(stats, d_st, sizeof(stats), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && st == PMMC_OK && kernel_ms) {
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    *kernel_ms = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (d_c) cudaFreeAsync(d_c, s);
  if (d_d) cudaFreeAsync(d_d, s);
  if (d_st) cudaFreeAsync(d_st, s);
  if (st != PMMC_OK) return st;
  if (e != cudaSuccess)
    return fail(ctx, e == cudaErrorMemoryAllocation ? PMMC_ERR_NOMEM : PMMC_ERR_CUDA,
                "distance heatmap: %s", cudaGetErrorString(e));
  if (avg_out) *avg_out = stats[0];
  if (max_out) *max_out = stats[1];
  return PMMC_OK;
}
