// capi.cu -- context, parameters and format conversions of the C ABI.
#include <vector>
#include <cstring>

#include "common.cuh"
#include "internal.h"

using namespace pmmc;

extern "C" const char *pmmc_status_string(pmmc_status s) {
  switch (s) {
    case PMMC_OK: return "ok";
    case PMMC_ERR_INVALID: return "invalid argument";
    case PMMC_ERR_NO_DEVICE: return "no usable CUDA device";
    case PMMC_ERR_CUDA: return "CUDA error";
    case PMMC_ERR_NOMEM: return "device out of memory";
    case PMMC_ERR_TIMEOUT: return "device wait timed out";
    case PMMC_ERR_BUDGET: return "device-memory budget exceeded";
    case PMMC_ERR_FIXED: return "every bead is fixed";
    case PMMC_ERR_BUSY: return "no free slot";
    case PMMC_ERR_NOT_FOUND: return "unknown request";
    case PMMC_ERR_CANCELLED: return "request cancelled";
  }
  return "unknown status";
}

extern "C" pmmc_status pmmc_ctx_create(pmmc_ctx **out, int device) {
  if (!out) return PMMC_ERR_INVALID;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
    cudaGetLastError();
    return PMMC_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= count) return PMMC_ERR_INVALID;
  if (cudaSetDevice(device) != cudaSuccess) return PMMC_ERR_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return PMMC_ERR_NO_DEVICE;
  auto *c = new pmmc_ctx();
  c->device = device;
  c->sm_count = prop.multiProcessorCount;
  c->smem_optin = prop.sharedMemPerBlockOptin;
  c->smem_per_sm = prop.sharedMemPerMultiprocessor;
  if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) {
    delete c;
    return PMMC_ERR_CUDA;
  }
  *out = c;
  return PMMC_OK;
}

extern "C" void pmmc_ctx_destroy(pmmc_ctx *ctx) {
  if (!ctx) return;
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  for (cudaStream_t a : ctx->aux_stream)
    if (a) cudaStreamDestroy(a);
  delete ctx;
}

extern "C" const char *pmmc_last_error(const pmmc_ctx *ctx) {
  return ctx ? ctx->last_error : "";
}

extern "C" void pmmc_set_seed(pmmc_ctx *ctx, uint64_t seed) {
  if (!ctx) return;
  ctx->seed = seed;
  ctx->calls = 0;
}

extern "C" int pmmc_sm_count(const pmmc_ctx *ctx) { return ctx ? ctx->sm_count : 0; }

// Settings::init defaults (src/include/Settings.hpp:397-505).
extern "C" void pmmc_default_params(int level, pmmc_anneal_params *o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->max_temp = 20.0f;
  o->dt_temp = 0.99995f;
  o->jump_scale = 50.0f;
  o->jump_coef = 20.0f;
  o->improvement = 0.995f;
  o->min_successes = 5;
  o->milestone_steps = 10000;
  o->k_angle = 0.1f;
  o->w_dist = 1.0f;
  o->w_angle = 1.0f;
  o->sphere_radius = 0.0f;
  o->use2d = 0;
  o->milestone_fails = 3;
  o->schedule = PMMC_SCHEDULE_GPU;
  o->resync_every = 0;
  o->max_moves = 0;
  o->bond_target = 1.0f;
  o->k_stretch_bond = 0.1f;
  o->k_squeeze_bond = 0.1f;
  o->k_angle_ext = 0.1f;
  if (level == PMMC_LEVEL_ARCS) {
    o->k_stretch = 1.0f;  // springConstantStretchArcs
    o->k_squeeze = 1.0f;  // springConstantSqueezeArcs
  } else {
    o->k_stretch = 0.1f;  // springConstantStretch
    o->k_squeeze = 0.1f;  // springConstantSqueeze
  }
}

namespace {

// CSR over both directions from the reference's matrix given as rows
// (row(j)[i] = v[j][i]): entry (i, j) holds v[j][i], the column the
// reference's local score reads (LooperSolver.hpp:3262), kept when i != j
// and v >= 0.  Two row-major passes: the counts of every CSR row, then the
// entries, columns in increasing order.  With col/target NULL only row_ptr
// and the count; a capacity below the count returns PMMC_ERR_INVALID with
// *nnz set.
template <class RowFn>
pmmc_status csr_from_rows(int n, RowFn row, int *row_ptr, int *col, float *target,
                          int64_t cap, int64_t *nnz) {
  std::vector<int64_t> cnt((size_t)n + 1, 0);
  for (int j = 0; j < n; ++j) {
    const float *r = row(j);
    if (!r) return PMMC_ERR_INVALID;
    for (int i = 0; i < n; ++i) cnt[i] += (i != j && r[i] >= 0.0f) ? 1 : 0;
  }
  int64_t k = 0;
  row_ptr[0] = 0;
  for (int i = 0; i < n; ++i) {
    const int64_t c = cnt[i];
    cnt[i] = k;  // cursor of row i
    k += c;
    if (k > 0x7fffffff) return PMMC_ERR_INVALID;
    row_ptr[i + 1] = (int)k;
  }
  if (nnz) *nnz = k;
  if (!col || !target) return PMMC_OK;
  if (k > cap) return PMMC_ERR_INVALID;
  for (int j = 0; j < n; ++j) {
    const float *r = row(j);
    for (int i = 0; i < n; ++i) {
      const float v = r[i];
      if (i != j && v >= 0.0f) {
        const int64_t e = cnt[i]++;
        col[e] = j;
        target[e] = v;
      }
    }
  }
  return PMMC_OK;
}

}  // namespace

extern "C" pmmc_status pmmc_arcs_dense_to_csr(int n, const float *dense, int *row_ptr,
                                              int *col, float *target, int64_t cap,
                                              int64_t *nnz) {
  if (n < 0 || !dense || !row_ptr) return PMMC_ERR_INVALID;
  return csr_from_rows(n, [&](int j) { return dense + (size_t)j * n; }, row_ptr, col, target,
                       cap, nnz);
}

extern "C" pmmc_status pmmc_arcs_rows_to_csr(int n, const float *const *rows, int *row_ptr,
                                             int *col, float *target, int64_t cap,
                                             int64_t *nnz) {
  if (n < 0 || !rows || !row_ptr) return PMMC_ERR_INVALID;
  return csr_from_rows(n, [&](int j) { return rows[j]; }, row_ptr, col, target, cap, nnz);
}

// ---------------------------------------------------------------------------
// Self-test of the kernels' square root: sqrt_rn against the IEEE routine
// on the float bit patterns [lo, lo + count).
// ---------------------------------------------------------------------------
namespace {
__global__ void selftest_sqrt_kernel(uint32_t lo, uint32_t count, unsigned long long *bad,
                                     unsigned int *first) {
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < count; k += stride) {
    const uint32_t bits = lo + k;
    const float s = __uint_as_float(bits);
    const float a = pmmc::sqrt_rn(s), b = __fsqrt_rn(s);
    if (__float_as_uint(a) != __float_as_uint(b) && !(a != a && b != b)) {
      atomicAdd(bad, 1ull);
      atomicMin(first, bits);
    }
  }
}
}  // namespace

extern "C" pmmc_status pmmc_selftest_sqrt(pmmc_ctx *ctx, uint32_t lo, uint32_t count,
                                          uint64_t *mismatches, uint32_t *first_bad) {
  if (!ctx || !mismatches || !first_bad) return PMMC_ERR_INVALID;
  unsigned long long *d_bad = nullptr;
  unsigned int *d_first = nullptr;
  PMMC_CUDA(ctx, cudaMalloc(&d_bad, sizeof(unsigned long long)));
  PMMC_CUDA(ctx, cudaMalloc(&d_first, sizeof(unsigned int)));
  const unsigned int init_first = 0xFFFFFFFFu;
  cudaError_t e = cudaMemset(d_bad, 0, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMemcpy(d_first, &init_first, sizeof(init_first), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    selftest_sqrt_kernel<<<ctx->sm_count * 8, 256, 0, ctx->stream>>>(lo, count, d_bad, d_first);
    e = cudaGetLastError();
  }
  unsigned long long nb = 0;
  unsigned int fb = 0;
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e == cudaSuccess) e = cudaMemcpy(&nb, d_bad, sizeof(nb), cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(&fb, d_first, sizeof(fb), cudaMemcpyDeviceToHost);
  cudaFree(d_bad);
  cudaFree(d_first);
  if (e != cudaSuccess) return fail(ctx, PMMC_ERR_CUDA, "sqrt self-test: %s", cudaGetErrorString(e));
  *mismatches = nb;
  *first_bad = fb;
  return PMMC_OK;
}
