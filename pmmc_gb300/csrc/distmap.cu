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
// Two passes over the upper triangle, 32 x 32 tiles (coalesced rows):
//   pass 1  per tile: the sum of the positive distances (FP64), the number
//           of band entries, the smallest diagonal offset holding a positive
//           distance; one partial per tile, reduced in a fixed order by a
//           single block (deterministic), which derives avg and the clamp;
//   pass 2  per tile: the distances again, clamped, written to the tile and,
//           through shared memory, to its mirror tile.
// HBM bound: 4 bytes read per upper-triangle entry in each pass, 4 bytes
// written per entry of the full map.
#include <cmath>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace pmmc {

constexpr int kTile = 32;

__device__ __forceinline__ float contact_to_dist(float c, int i, int j, int diag, float scale,
                                                 float power) {
  if ((double)c < 1e-6) return 0.0f;
  if (abs(i - j) < diag) return -1.0f;
  return scale * powf(c, power);
}

struct DistPartial {
  double sum_pos;   // positive distances of the tile (upper triangle)
  long long n_neg;  // band entries (-1) of the tile (upper triangle)
  int min_off;      // smallest j - i with a distance above 1e-6 (INT_MAX: none)
  int pad;
};

// Tile (bi, bj), bi <= bj, of the upper triangle: blockIdx.x enumerates them
// row by row.
__device__ __forceinline__ void tile_of(int t, int nt, int &bi, int &bj) {
  // row bi holds nt - bi tiles; invert the prefix count
  int r = 0, base = 0;
  while (base + (nt - r) <= t) {
    base += nt - r;
    ++r;
  }
  bi = r;
  bj = r + (t - base);
}

__global__ void __launch_bounds__(kTile * 8)
distmap_pass1(const float *__restrict__ c, int n, int nt, int diag, float scale, float power,
              DistPartial *__restrict__ part) {
  __shared__ double s_sum[8];
  __shared__ long long s_neg[8];
  __shared__ int s_min[8];
  int bi, bj;
  tile_of(blockIdx.x, nt, bi, bj);
  const int tx = threadIdx.x & (kTile - 1), ty = threadIdx.x / kTile;  // 32 x 8
  const int j = bj * kTile + tx;
  double sum = 0.0;
  long long neg = 0;
  int mo = 0x7fffffff;
  for (int r = ty; r < kTile; r += 8) {
    const int i = bi * kTile + r;
    if (i < n && j < n && j >= i) {
      const float d = contact_to_dist(c[(size_t)i * n + j], i, j, diag, scale, power);
      if (d > 0.0f) sum += (double)d;
      if (d == -1.0f) ++neg;
      if ((double)d > 1e-6) mo = min(mo, j - i);
    }
  }
  sum = warp_sum_d(sum);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    neg += __shfl_xor_sync(0xffffffffu, neg, o);
    mo = min(mo, __shfl_xor_sync(0xffffffffu, mo, o));
  }
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    s_sum[w] = sum;
    s_neg[w] = neg;
    s_min[w] = mo;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    DistPartial p{0.0, 0, 0x7fffffff, 0};
    for (int k = 0; k < 8; ++k) {
      p.sum_pos += s_sum[k];
      p.n_neg += s_neg[k];
      p.min_off = min(p.min_off, s_min[k]);
    }
    part[blockIdx.x] = p;
  }
}

// One block: the partials in tile order, avg = Heatmap::getAvg of the map and
// the clamp value.
__global__ void distmap_finish(const DistPartial *__restrict__ part, int n_part, int n,
                               float stretching, float *__restrict__ out2) {
  __shared__ double s_sum[32];
  __shared__ long long s_neg[32];
  __shared__ int s_min[32];
  double sum = 0.0;
  long long neg = 0;
  int mo = 0x7fffffff;
  // each thread a contiguous chunk, then a fixed-order combination
  const int per = (n_part + blockDim.x - 1) / blockDim.x;
  for (int k = threadIdx.x * per; k < min(n_part, (int)(threadIdx.x + 1) * per); ++k) {
    sum += part[k].sum_pos;
    neg += part[k].n_neg;
    mo = min(mo, part[k].min_off);
  }
  // fixed-order tree over the block
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
    double s = t;
    if (m == 0x7fffffff) {
      w = 0;
      s = -(double)ng;
    }
    const double cnt = (double)(n - w) * (double)(n - w + 1) * 0.5;
    const float avg = (float)(s / cnt);
    out2[0] = avg;
    out2[1] = avg * stretching;
  }
}

__global__ void __launch_bounds__(kTile * 8)
distmap_pass2(const float *__restrict__ c, int n, int nt, int diag, float scale, float power,
              const float *__restrict__ stats, float *__restrict__ dist) {
  __shared__ float tile[kTile][kTile + 1];
  int bi, bj;
  tile_of(blockIdx.x, nt, bi, bj);
  const float maxd = stats[1];
  const int tx = threadIdx.x & (kTile - 1), ty = threadIdx.x / kTile;
  const int j = bj * kTile + tx;
  for (int r = ty; r < kTile; r += 8) {
    const int i = bi * kTile + r;
    float d = 0.0f;
    if (i < n && j < n) {
      // the upper triangle defines both halves; below the diagonal of a
      // diagonal tile the mirror writes the value
      if (j >= i) {
        d = contact_to_dist(c[(size_t)i * n + j], i, j, diag, scale, power);
        if (d > maxd) d = maxd;
        dist[(size_t)i * n + j] = d;
      }
    }
    tile[r][tx] = d;
  }
  __syncthreads();
  // mirror: element (i, j) -> (j, i); thread tx now walks i within the tile
  const int i2 = bi * kTile + tx;
  for (int r = ty; r < kTile; r += 8) {
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
  const long long n_tiles = (long long)nt * (nt + 1) / 2;
  if (n_tiles > 0x7fffffffLL) return fail(ctx, PMMC_ERR_INVALID, "distance heatmap: n too large");
  DistPartial *d_part = nullptr;
  PMMC_CUDA(ctx, cudaMallocAsync(&d_part, sizeof(DistPartial) * n_tiles, s));
  distmap_pass1<<<(unsigned)n_tiles, kTile * 8, 0, s>>>(d_c, n, nt, diag, scale, power, d_part);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) {
    distmap_finish<<<1, 1024, 0, s>>>(d_part, (int)n_tiles, n, stretching, d_stats);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) {
    distmap_pass2<<<(unsigned)n_tiles, kTile * 8, 0, s>>>(d_c, n, nt, diag, scale, power,
                                                          d_stats, d_dist);
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
