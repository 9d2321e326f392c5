// Host-side thread safety of a context (pmmc_gb300/csrc/internal.h).  The
// worker pool (pmmc::HostPool): every run calls fn(t) exactly once for each
// t < n, on distinct threads for t > 0, returns only after all have
// finished, and the split of a range into per-thread parts covers every
// index once.  Failure messages (pmmc::fail) recorded by many threads at
// once leave one whole message.  Built and run by
// tests/test_host_pool_cpu.py.
#include <atomic>
#include <cstdio>
#include <set>
#include <thread>

#include "internal.h"

int main() {
  constexpr int kSize = 8;
  pmmc::HostPool pool(kSize);
  for (int rep = 0; rep < 3000; ++rep) {
    const int n = 1 + rep % (kSize + 2);  // above the size: clamped to it
    std::atomic<int> hits[kSize];
    for (auto &h : hits) h = 0;
    std::mutex mu;
    std::set<std::thread::id> ids;
    pool.run(n, [&](int t) {
      hits[t] += 1;
      std::lock_guard<std::mutex> lk(mu);
      ids.insert(std::this_thread::get_id());
    });
    const int m = n < kSize ? n : kSize;
    for (int t = 0; t < kSize; ++t)
      if (hits[t] != (t < m ? 1 : 0)) {
        std::printf("run %d: slice %d ran %d times\n", rep, t, (int)hits[t]);
        return 1;
      }
    if ((int)ids.size() != m) {
      std::printf("run %d: %d slices on %zu threads\n", rep, m, ids.size());
      return 1;
    }
  }
  // the partition the batch packing uses: parts of ceil(units / threads)
  for (int units = 1; units < 200; ++units) {
    std::vector<std::atomic<int>> seen(units);
    for (auto &s : seen) s = 0;
    const int per = (units + kSize - 1) / kSize;
    pool.run(kSize, [&](int t) {
      const int a = t * per, z = std::min(units, a + per);
      for (int u = a; u < z; ++u) seen[u] += 1;
    });
    for (int u = 0; u < units; ++u)
      if (seen[u] != 1) {
        std::printf("units %d: unit %d seen %d times\n", units, u, (int)seen[u]);
        return 1;
      }
  }
  // failures recorded on one context by several threads at once
  {
    auto *ctx = new pmmc_ctx();
    std::vector<std::thread> th;
    for (int t = 0; t < 8; ++t)
      th.emplace_back([ctx, t] {
        for (int k = 0; k < 2000; ++k)
          pmmc::fail(ctx, PMMC_ERR_INVALID, "thread %d failure %d %s", t, k,
                     k % 2 ? "with a longer tail to vary the length" : "");
      });
    for (auto &x : th) x.join();
    int t = -1, k = -1;
    if (std::sscanf(ctx->last_error, "thread %d failure %d", &t, &k) != 2 || t < 0 ||
        t >= 8 || k < 0 || k >= 2000) {
      std::printf("last message: %s\n", ctx->last_error);
      return 1;
    }
    delete ctx;
  }
  std::printf("ok\n");
  return 0;
}
