// internal.h -- host-side internals shared by the library's translation units.
#pragma once
#include <cuda_runtime.h>

#include <cmath>
#include <condition_variable>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <functional>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "pmmc_gb300.h"

namespace pmmc {

// Host worker threads kept for the life of a context: a call that splits
// its host work (validating and packing many regions) hands it to the same
// threads every time instead of starting and joining new ones, which costs
// tens of microseconds per thread.  run(n, fn) calls fn(t) for t = 0..n-1,
// t = 0 on the calling thread, and returns when all are done; one run at a
// time.
class HostPool {
 public:
  explicit HostPool(int size) : size_(size < 1 ? 1 : size) {
    for (int t = 1; t < size_; ++t) th_.emplace_back([this, t] { work(t); });
  }
  ~HostPool() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_.notify_all();
    for (auto &t : th_) t.join();
  }
  HostPool(const HostPool &) = delete;
  HostPool &operator=(const HostPool &) = delete;
  int size() const { return size_; }
  void run(int n, const std::function<void(int)> &fn) {
    std::lock_guard<std::mutex> one(run_mu_);
    n = n < 1 ? 1 : (n > size_ ? size_ : n);
    {
      std::lock_guard<std::mutex> lk(mu_);
      job_ = &fn;
      n_job_ = n;
      pending_ = size_ - 1;
      ++gen_;
    }
    cv_.notify_all();
    fn(0);
    std::unique_lock<std::mutex> lk(mu_);
    done_.wait(lk, [this] { return pending_ == 0; });
    job_ = nullptr;
  }

 private:
  void work(int t) {
    unsigned long long seen = 0;
    std::unique_lock<std::mutex> lk(mu_);
    for (;;) {
      cv_.wait(lk, [&] { return stop_ || gen_ != seen; });
      if (stop_) return;
      seen = gen_;
      const std::function<void(int)> *f = job_;
      const int n = n_job_;
      lk.unlock();
      if (t < n) (*f)(t);
      lk.lock();
      if (--pending_ == 0) done_.notify_one();
    }
  }
  const int size_;
  std::vector<std::thread> th_;
  std::mutex run_mu_, mu_;
  std::condition_variable cv_, done_;
  const std::function<void(int)> *job_ = nullptr;
  int n_job_ = 0, pending_ = 0;
  unsigned long long gen_ = 0;
  bool stop_ = false;
};

}  // namespace pmmc

struct pmmc_ctx {
  int device = 0;
  // host-side state a module keeps per context (e.g. packing buffers that
  // are reused, already paged in, by the next call), made once
  std::shared_ptr<void> arcs_host_cache;
  std::once_flag arcs_host_cache_once;
  // host worker threads (made at the first call that splits its host work)
  std::unique_ptr<pmmc::HostPool> host_pool;
  std::once_flag host_pool_once;
  int sm_count = 0;
  size_t smem_optin = 0;       // max dynamic shared memory per block (opt-in)
  size_t smem_per_sm = 0;
  uint64_t seed = 0;
  uint64_t calls = 0;          // advanced by every annealing call
  cudaStream_t stream = nullptr;
  // further kernels of one call beside the first
  cudaStream_t aux_stream[2] = {nullptr, nullptr};
  // smoothing: slots per chain of the windowed kernel (0 = one move at a
  // time), for regions with fewer / at least smooth_window_long_min_free
  // movable beads
  int smooth_window = 8;
  int smooth_window_long = 32;
  int smooth_window_long_min_free = 20;
  // heatmap: CTAs of the cluster that runs one chain (0 = by the batch: 16
  // or 8 for a few chains on large maps, else 1)
  int heatmap_cluster = 0;
  // message of the last failing call; a fixed buffer written under a lock,
  // so failures on several host threads at once (server submits) never
  // touch freed memory (the last byte is always the terminator)
  char last_error[512] = {0};
  std::mutex error_mu;
};

namespace pmmc {

inline int __float_as_int_host(float f) {
  int i;
  memcpy(&i, &f, 4);
  return i;
}
inline float __int_as_float_host(int i) {
  float f;
  memcpy(&f, &i, 4);
  return f;
}

// freqToDistance(freq, memo = false) (LooperSolver.hpp:3949-3967) on the
// host: the int count plus the float shift is a float, the rest FP64 (this
// code is built with -ffp-contract=off, so it rounds as the reference does).
inline float count_to_distance(int freq, float a, float scale, float shift, float base) {
  const float fs = (float)freq + shift;
  if (a < 0.0f) {
    int fi = (int)fs;
    if (fi < 1) fi = 1;
    return (float)((double)base + (double)scale * std::pow((double)fi, (double)a));
  }
  return (float)((double)base + (double)scale / std::exp((double)a * (double)fs));
}

// Records a message on the context and returns the status.
inline pmmc_status fail(pmmc_ctx *ctx, pmmc_status s, const char *fmt, ...) {
  if (ctx) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    static_assert(sizeof(buf) == sizeof(ctx->last_error), "message buffer sizes");
    const size_t len = strnlen(buf, sizeof(buf) - 1);
    std::lock_guard<std::mutex> lk(ctx->error_mu);
    memcpy(ctx->last_error, buf, len);
    ctx->last_error[len] = '\0';
  }
  return s;
}

#define PMMC_CUDA(ctx, call)                                                   \
  do {                                                                         \
    cudaError_t e_ = (call);                                                   \
    if (e_ != cudaSuccess)                                                     \
      return ::pmmc::fail((ctx), e_ == cudaErrorMemoryAllocation               \
                                     ? PMMC_ERR_NOMEM                          \
                                     : PMMC_ERR_CUDA,                          \
                          "%s: %s (%s:%d)", #call, cudaGetErrorString(e_),     \
                          __FILE__, __LINE__);                                 \
  } while (0)

// The Philox key of the next annealing call: the context seed for the first
// call after pmmc_set_seed, then a fresh key per call.
inline uint64_t next_key(pmmc_ctx *ctx) {
  uint64_t k = ctx->seed + ctx->calls * 0x9E3779B97F4A7C15ull;
  ctx->calls++;
  return k;
}

// RAII device buffer.
template <typename T> struct DevBuf {
  T *p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf &) = delete;
  DevBuf &operator=(const DevBuf &) = delete;
  ~DevBuf() { release(); }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count) {
    release();
    n = count;
    if (count == 0) return cudaSuccess;
    return cudaMalloc(&p, count * sizeof(T));
  }
  cudaError_t upload(const std::vector<T> &v, cudaStream_t s) {
    cudaError_t e = alloc(v.size());
    if (e != cudaSuccess || v.empty()) return e;
    return cudaMemcpyAsync(p, v.data(), v.size() * sizeof(T),
                           cudaMemcpyHostToDevice, s);
  }
};

}  // namespace pmmc
