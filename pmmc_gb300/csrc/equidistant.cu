// equidistant.cu -- equidistant model: points every res bp along a level.
//
// HierarchicalChromosome::createEqidistantModel (src/HierarchicalChromosome.cu:
// 466-519) resamples a chromosome's current level at a fixed genomic step:
// before the end of the first cluster the first cluster's position, from the
// start of the last cluster on the last one's, otherwise the Catmull-Rom
// spline (interpolateSpline, thirdparty/common.cpp:453-462) through the two
// clusters around the point and their neighbours (mirrored at the ends).
// The reference's kernel (parallelFind3DSmoothPosition, :420-464) scans the
// level linearly per point and leaves the thread after its first point, so
// outputs past its grid are never written; its host CPU path (gpuHelper,
// :1380-1447) defines the result, restated here.
//
// One thread per point; a binary search over the level's genomic positions
// (sorted along a chromosome; an unsorted level takes the linear scan of the
// reference); the spline in unfused FP32 as the reference rounds it.
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace pmmc {

__global__ void equidistant_kernel(int n, const int *__restrict__ gpos,
                                   const float *__restrict__ pos, int first_end, int last_start,
                                   int pos_start, int res, long long out_size, int sorted,
                                   float *__restrict__ out) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < out_size;
       idx += stride) {
    const long long p = pos_start + (long long)res * idx;
    float *o = out + 3 * idx;
    int src = -1;  // copy a cluster's position
    int i = -1;    // interpolate between clusters i - 1 and i
    if (p < first_end) {
      src = 0;
    } else if (p >= last_start) {
      src = n - 1;
    } else if (sorted) {
      // the first i >= 1 with p < gpos[i]
      int lo = 1, hi = n;
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (p < gpos[mid]) hi = mid;
        else lo = mid + 1;
      }
      if (lo < n) i = lo;
      else src = n - 1;
    } else {
      for (int k = 1; k < n && i < 0; ++k)
        if (p < gpos[k]) i = k;
      if (i < 0) src = n - 1;
    }
    if (src >= 0) {
      o[0] = pos[3 * src];
      o[1] = pos[3 * src + 1];
      o[2] = pos[3 * src + 2];
      continue;
    }
    const float t = __fdiv_rn((float)(p - gpos[i - 1]), (float)(gpos[i] - gpos[i - 1]));
    const float t2 = __fmul_rn(t, t), t3 = __fmul_rn(t2, t);
    const float b1 = __fmul_rn(0.5f, __fsub_rn(__fadd_rn(-t3, __fmul_rn(2.0f, t2)), t));
    const float b2 =
        __fmul_rn(0.5f, __fadd_rn(__fsub_rn(__fmul_rn(3.0f, t3), __fmul_rn(5.0f, t2)), 2.0f));
    const float b3 =
        __fmul_rn(0.5f, __fadd_rn(__fadd_rn(__fmul_rn(-3.0f, t3), __fmul_rn(4.0f, t2)), t));
    const float b4 = __fmul_rn(0.5f, __fsub_rn(t3, t2));
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      const float v1 = pos[3 * (i - 1) + c], v2 = pos[3 * i + c];
      const float v0 = i > 1 ? pos[3 * (i - 2) + c] : __fsub_rn(__fmul_rn(2.0f, v1), v2);
      const float v3 = i + 1 < n ? pos[3 * (i + 1) + c] : __fsub_rn(__fmul_rn(2.0f, v2), v1);
      o[c] = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(v0, b1), __fmul_rn(v1, b2)), __fmul_rn(v2, b3)),
                       __fmul_rn(v3, b4));
    }
  }
}

}  // namespace pmmc

using namespace pmmc;

extern "C" pmmc_status pmmc_equidistant_model(pmmc_ctx *ctx, int n, const int *gpos,
                                              const float *pos, int first_end, int last_start,
                                              int pos_start, int pos_stop, int res,
                                              float *out, int64_t cap, int64_t *n_out,
                                              double *kernel_ms) {
  if (!ctx || n < 1 || !gpos || !pos || res < 1 || pos_stop < pos_start || !n_out)
    return fail(ctx, PMMC_ERR_INVALID, "equidistant model: bad arguments");
  const long long out_size = (long long)((pos_stop - pos_start + 1) / res + 1);
  *n_out = out_size;
  if (!out || cap < out_size) return PMMC_OK;  // size query
  int sorted = 1;
  for (int k = 1; k < n; ++k)
    if (gpos[k] < gpos[k - 1]) sorted = 0;
  cudaStream_t s = ctx->stream;
  int *d_g = nullptr;
  float *d_p = nullptr, *d_o = nullptr;
  cudaError_t e = cudaMallocAsync(&d_g, sizeof(int) * n, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_p, sizeof(float) * 3 * n, s);
  if (e == cudaSuccess) e = cudaMallocAsync(&d_o, sizeof(float) * 3 * out_size, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_g, gpos, sizeof(int) * n, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_p, pos, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, s);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  if (e == cudaSuccess) {
    const long long want = (out_size + 255) / 256;
    const int blocks = (int)std::min<long long>(want, 16LL * ctx->sm_count);
    cudaEventRecord(e0, s);
    equidistant_kernel<<<std::max(blocks, 1), 256, 0, s>>>(n, d_g, d_p, first_end, last_start,
                                                           pos_start, res, out_size, sorted, d_o);
    e = cudaGetLastError();
    cudaEventRecord(e1, s);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out, d_o, sizeof(float) * 3 * out_size, cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e == cudaSuccess && kernel_ms) {
    float ms = 0.0f;
    cudaEventElapsedTime(&ms, e0, e1);
    *kernel_ms = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (d_g) cudaFreeAsync(d_g, s);
  if (d_p) cudaFreeAsync(d_p, s);
  if (d_o) cudaFreeAsync(d_o, s);
  if (e != cudaSuccess)
    return fail(ctx, e == cudaErrorMemoryAllocation ? PMMC_ERR_NOMEM : PMMC_ERR_CUDA,
                "equidistant model: %s", cudaGetErrorString(e));
  return PMMC_OK;
}
