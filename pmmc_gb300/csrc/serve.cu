// serve.cu -- request loop for arc-level region reconstructions.
//
// The reference runs reconstructions one after another inside a host memory
// budget (-M, Settings::maxMemoryMB, checked by checkMemoryBudget in the
// ensemble loop, main_reconstruct.cpp:423).  Here a server object accepts
// regions of any size from any host thread and keeps the GPU busy with them:
//
//   submit   packs the region on the caller's thread (the same layout the
//            batched path uses) and queues it; a region whose device
//            footprint alone exceeds the budget is refused.
//   admit    a scheduler thread forms a wave from the head of the queue:
//            regions of one shared-memory class, in arrival order, while the
//            device bytes of everything resident stay within the budget and a
//            launch slot is free.  The wave's inputs go up in one copy from a
//            pinned staging buffer, the frozen repulsion of its regions is
//            computed (one block each), one persistent launch anneals all of
//            them (one warp per region, plus a drawing warp for one-lane
//            regions; work-stealing), and the results come back in one copy,
//            all on the slot's own stream.
//   overlap  up to max_waves waves are in flight at once on separate streams,
//            so regions that arrive while others run start as soon as a slot
//            and memory free up, without waiting for the running waves.
//   finish   the scheduler polls the waves' events, hands the results to the
//            waiting callers and releases the wave's memory and slot.
//
// Each region carries its own Philox key (the caller's seed, chain 0), and a
// region's class (arc lists staged in shared memory or not) and its lanes per
// proposal (chosen from its size) depend only on the region, so its result is
// bit-identical whether it runs alone or in any mix.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "arcs_impl.h"

using namespace pmmc;

namespace {

using Clock = std::chrono::steady_clock;

constexpr size_t kAlign = 256;
inline size_t align_up(size_t x) { return (x + kAlign - 1) & ~(kAlign - 1); }

// Byte offsets of one wave's device blob: inputs first (one H2D copy), then
// the zero-initialised counters, then the outputs (one D2H copy).
struct BlobLayout {
  size_t units, items, pos0, rp, nbr, inv, nulls, mov, lrp, lent, lst;
  size_t in_bytes;        // [0, in_bytes) is copied up
  size_t head, done;      // cleared before the launch
  size_t bases;           // frozen repulsion per region
  size_t pos_out, outs;   // [pos_out, total) is copied back
  size_t total;
};

BlobLayout layout_of(const ArcsPack &pk) {
  BlobLayout L{};
  size_t o = 0;
  auto take = [&](size_t bytes) {
    const size_t at = o;
    o = align_up(o + std::max<size_t>(bytes, 1));
    return at;
  };
  L.units = take(sizeof(ArcsUnit) * pk.units.size());
  L.items = take(sizeof(int2) * pk.units.size());
  L.pos0 = take(sizeof(float4) * pk.pos.size());
  L.rp = take(sizeof(int) * pk.rp.size());
  L.nbr = take(sizeof(int2) * pk.nbr.size());
  L.inv = take(sizeof(float) * pk.inv.size());
  L.nulls = take(sizeof(int2) * std::max<size_t>(pk.nulls.size(), 1));
  L.mov = take(sizeof(int) * pk.mov.size());
  L.lrp = take(sizeof(int) * pk.lrp.size());
  L.lent = take(sizeof(float4) * pk.lent.size());
  L.lst = take(sizeof(int4) * std::max<size_t>(pk.lst.size(), 1));
  L.in_bytes = o;
  L.head = take(sizeof(int));
  L.done = take(sizeof(int) * pk.units.size());
  L.bases = take(sizeof(double) * pk.units.size());
  L.pos_out = take(sizeof(float) * (size_t)pk.out_floats);
  L.outs = take(sizeof(ChainOut) * (size_t)pk.chains);
  L.total = o;
  return L;
}

enum class ReqState { Queued, Running, Done, Failed, Cancelled };

struct Request {
  long long ticket = 0;
  ArcsPack pack;           // one region, one chain, packed at submit
  int n = 0;
  bool nb_smem = true;     // arc lists staged in shared memory
  int lanes = 2;           // lanes per proposal (depends on the region only)
  int smem_need = 0;       // bytes of the chain's shared-memory slice
  size_t dev_bytes = 0;    // device footprint alone (budget accounting)
  Clock::time_point t_submit, t_done;
  ReqState state = ReqState::Queued;
  pmmc_status error = PMMC_OK;
  std::vector<float> pos_out;
  pmmc_result res{};
};
using ReqPtr = std::shared_ptr<Request>;

struct Slot {
  cudaStream_t stream = nullptr;
  cudaEvent_t ev = nullptr;
  void *h_in = nullptr;    // pinned staging of the inputs
  size_t h_in_cap = 0;
  void *h_out = nullptr;   // pinned landing of the outputs
  size_t h_out_cap = 0;
  bool busy = false;
  std::vector<ReqPtr> wave;
  ArcsPack pack;           // the wave's merged pack (offsets of its results)
  BlobLayout lay{};
  void *d_blob = nullptr;
  size_t bytes = 0;        // budget charged for the wave
};

cudaError_t ensure_pinned(void *&p, size_t &cap, size_t need) {
  if (cap >= need) return cudaSuccess;
  if (p) cudaFreeHost(p);
  p = nullptr;
  cap = 0;
  size_t c = 1 << 20;
  while (c < need) c <<= 1;
  cudaError_t e = cudaHostAlloc(&p, c, cudaHostAllocDefault);
  if (e == cudaSuccess) cap = c;
  return e;
}

}  // namespace

struct pmmc_server {
  pmmc_ctx *ctx = nullptr;
  ArcsDevParams P{};
  int lanes = 0;           // 0: by region size
  size_t budget = 0;
  int max_wave = 0;
  size_t cap_smem = 0;
  std::vector<Slot> slots;

  std::mutex mu;
  std::condition_variable cv_sched, cv_done;
  std::deque<ReqPtr> queue;
  std::unordered_map<long long, ReqPtr> table;
  long long next_ticket = 1;
  size_t bytes_in_use = 0;
  bool stopping = false;
  std::thread th;

  // statistics (under mu)
  long long n_submitted = 0, n_completed = 0, n_rejected = 0, n_waves = 0, n_failed = 0;
  size_t bytes_peak = 0;
  int running_requests = 0, running_peak = 0, waves_peak = 0;

  void run();
  void launch(Slot &sl, std::vector<ReqPtr> wave);
  void finish(Slot &sl, cudaError_t e);
};

void pmmc_server::finish(Slot &sl, cudaError_t e) {
  const auto now = Clock::now();
  std::vector<ReqPtr> wave;
  wave.swap(sl.wave);
  if (e == cudaSuccess) {
    const unsigned char *out = static_cast<const unsigned char *>(sl.h_out);
    const float *pos = reinterpret_cast<const float *>(out);
    const ChainOut *outs =
        reinterpret_cast<const ChainOut *>(out + (sl.lay.outs - sl.lay.pos_out));
    for (size_t k = 0; k < wave.size(); ++k) {
      Request &r = *wave[k];
      const ArcsUnit &U = sl.pack.units[k];
      r.pos_out.assign(pos + U.out_off, pos + U.out_off + (size_t)U.n * 3);
      const ChainOut &o = outs[U.chain_base];
      pmmc_result q{};
      q.score = o.score;
      q.energy = o.energy;
      q.energy_fp64 = o.energy_fp64;
      q.rel_error = std::fabs(o.energy - o.energy_fp64) / std::max(std::fabs(o.energy_fp64), 1e-30);
      q.moves = o.moves;
      q.accepted = o.accepted;
      q.total_moves = o.moves;
      q.best_chain = 0;
      q.status = o.status;
      r.res = q;
    }
  }
  if (sl.d_blob) cudaFreeAsync(sl.d_blob, sl.stream);
  sl.d_blob = nullptr;
  std::lock_guard<std::mutex> lock(mu);
  for (auto &r : wave) {
    r->t_done = now;
    r->state = e == cudaSuccess ? ReqState::Done : ReqState::Failed;
    r->error = e == cudaSuccess ? PMMC_OK : PMMC_ERR_CUDA;
    if (e == cudaSuccess) ++n_completed;
    else ++n_failed;
  }
  bytes_in_use -= sl.bytes;
  running_requests -= (int)wave.size();
  sl.bytes = 0;
  sl.busy = false;
  cv_done.notify_all();
}

void pmmc_server::launch(Slot &sl, std::vector<ReqPtr> wave) {
  // merged pack, largest regions first in the work queue
  ArcsPack pk;
  bool nbs = true;
  int smem_need = 0, lanes = 2;
  for (auto &r : wave) {
    pk.append(r->pack);
    nbs = r->nb_smem;
    lanes = r->lanes;
    smem_need = std::max(smem_need, r->smem_need);
  }
  pk.finish();
  std::vector<int2> items(pk.units.size());
  for (size_t u = 0; u < items.size(); ++u) items[u] = make_int2((int)u, 0);
  std::stable_sort(items.begin(), items.end(), [&](const int2 &a, const int2 &b) {
    return pk.units[a.x].n > pk.units[b.x].n;
  });
  const BlobLayout L = layout_of(pk);
  sl.wave = std::move(wave);
  sl.lay = L;
  cudaError_t e = ensure_pinned(sl.h_in, sl.h_in_cap, L.in_bytes);
  if (e == cudaSuccess) e = ensure_pinned(sl.h_out, sl.h_out_cap, L.total - L.pos_out);
  if (e == cudaSuccess) {
    unsigned char *h = static_cast<unsigned char *>(sl.h_in);
    auto put = [&](size_t off, const void *src, size_t bytes) {
      if (bytes) memcpy(h + off, src, bytes);
    };
    put(L.units, pk.units.data(), sizeof(ArcsUnit) * pk.units.size());
    put(L.items, items.data(), sizeof(int2) * items.size());
    put(L.pos0, pk.pos.data(), sizeof(float4) * pk.pos.size());
    put(L.rp, pk.rp.data(), sizeof(int) * pk.rp.size());
    put(L.nbr, pk.nbr.data(), sizeof(int2) * pk.nbr.size());
    put(L.inv, pk.inv.data(), sizeof(float) * pk.inv.size());
    put(L.nulls, pk.nulls.data(), sizeof(int2) * pk.nulls.size());
    put(L.mov, pk.mov.data(), sizeof(int) * pk.mov.size());
    put(L.lrp, pk.lrp.data(), sizeof(int) * pk.lrp.size());
    put(L.lent, pk.lent.data(), sizeof(float4) * pk.lent.size());
    put(L.lst, pk.lst.data(), sizeof(int4) * pk.lst.size());
    e = cudaMallocAsync(&sl.d_blob, L.total, sl.stream);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(sl.d_blob, sl.h_in, L.in_bytes, cudaMemcpyHostToDevice, sl.stream);
  unsigned char *d = static_cast<unsigned char *>(sl.d_blob);
  if (e == cudaSuccess)
    e = cudaMemsetAsync(d + L.head, 0, L.pos_out - L.head, sl.stream);
  if (e == cudaSuccess) {
    int warps = 4;
    const int per_warp = (smem_need + 15) & ~15;
    while (warps > 1 && (size_t)warps * per_warp > cap_smem) warps >>= 1;
    const int n_items = (int)items.size();
    // one lane per proposal (large regions): a drawing warp per chain keeps
    // the proposal draws off the chain's path
    const bool prod = lanes == 1;
    const int per_sm = arcs_ctas_per_sm(nbs, lanes, warps, per_warp, prod);
    const int grid = std::max(1, std::min(per_sm * ctx->sm_count, (n_items + warps - 1) / warps));
    ArcsLaunch a{reinterpret_cast<const ArcsUnit *>(d + L.units),
                 reinterpret_cast<const int2 *>(d + L.items),
                 n_items,
                 reinterpret_cast<int *>(d + L.head),
                 reinterpret_cast<const float4 *>(d + L.pos0),
                 reinterpret_cast<const int *>(d + L.rp),
                 reinterpret_cast<const int2 *>(d + L.nbr),
                 reinterpret_cast<const float *>(d + L.inv),
                 reinterpret_cast<const int *>(d + L.mov),
                 reinterpret_cast<const int *>(d + L.lrp),
                 reinterpret_cast<const float4 *>(d + L.lent),
                 reinterpret_cast<const int4 *>(d + L.lst),
                 reinterpret_cast<const int2 *>(d + L.nulls),
                 reinterpret_cast<float *>(d + L.pos_out),
                 reinterpret_cast<ChainOut *>(d + L.outs),
                 reinterpret_cast<int *>(d + L.done),
                 nullptr,
                 reinterpret_cast<const double *>(d + L.bases)};
    e = arcs_bases(a.units, n_items, a.pos0, a.row_ptr, a.nbr, a.nulls,
                   reinterpret_cast<double *>(d + L.bases), sl.stream);
    if (e == cudaSuccess)
      e = arcs_launch(a, P, nbs, lanes, grid, warps, per_warp, sl.stream, prod);
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(sl.h_out, d + L.pos_out, L.total - L.pos_out, cudaMemcpyDeviceToHost,
                        sl.stream);
  if (e == cudaSuccess) e = cudaEventRecord(sl.ev, sl.stream);
  sl.pack = std::move(pk);
  if (e != cudaSuccess) {
    cudaGetLastError();
    cudaStreamSynchronize(sl.stream);
    finish(sl, e);
  }
}

void pmmc_server::run() {
  cudaSetDevice(ctx->device);
  for (;;) {
    // completed waves
    for (auto &sl : slots) {
      if (!sl.busy) continue;
      const cudaError_t q = cudaEventQuery(sl.ev);
      if (q == cudaErrorNotReady) continue;
      finish(sl, q);
    }
    // admission: waves from the head of the queue while a slot is free
    std::vector<std::pair<Slot *, std::vector<ReqPtr>>> todo;
    bool idle = false;
    {
      std::unique_lock<std::mutex> lock(mu);
      for (;;) {
        Slot *free_slot = nullptr;
        for (auto &sl : slots)
          if (!sl.busy) {
            free_slot = &sl;
            break;
          }
        if (!free_slot || queue.empty()) break;
        const ReqPtr head = queue.front();
        if (bytes_in_use + head->dev_bytes > budget) break;  // wait for memory
        std::vector<ReqPtr> wave;
        size_t bytes = 0;
        for (auto it = queue.begin(); it != queue.end() && (int)wave.size() < max_wave;) {
          const ReqPtr &r = *it;
          if (r->nb_smem == head->nb_smem && r->lanes == head->lanes &&
              (wave.empty() || bytes_in_use + bytes + r->dev_bytes <= budget)) {
            bytes += r->dev_bytes;
            r->state = ReqState::Running;
            wave.push_back(r);
            it = queue.erase(it);
          } else {
            ++it;
          }
        }
        free_slot->busy = true;
        free_slot->bytes = bytes + 16 * kAlign;  // the wave blob's own padding
        bytes_in_use += free_slot->bytes;
        bytes_peak = std::max(bytes_peak, bytes_in_use);
        running_requests += (int)wave.size();
        running_peak = std::max(running_peak, running_requests);
        ++n_waves;
        int busy = 0;
        for (auto &sl : slots) busy += sl.busy ? 1 : 0;
        waves_peak = std::max(waves_peak, busy);
        todo.emplace_back(free_slot, std::move(wave));
      }
      bool inflight = false;
      for (auto &sl : slots) inflight |= sl.busy;
      if (todo.empty()) {
        if (stopping && queue.empty() && !inflight) return;
        if (!inflight) {
          cv_sched.wait(lock, [&] { return stopping || !queue.empty(); });
          continue;
        }
        idle = true;
      }
    }
    for (auto &t : todo) launch(*t.first, std::move(t.second));
    if (idle) std::this_thread::sleep_for(std::chrono::microseconds(20));
  }
}

extern "C" pmmc_status pmmc_server_create(pmmc_ctx *ctx, const pmmc_anneal_params *prm,
                                          const pmmc_server_opts *opts, pmmc_server **out) {
  if (!ctx || !prm || !out) return fail(ctx, PMMC_ERR_INVALID, "server: bad arguments");
  *out = nullptr;
  auto sv = std::make_unique<pmmc_server>();
  sv->ctx = ctx;
  sv->P = arcs_make_params(prm, 0, false);
  sv->P.trace_cap = 0;
  const int lanes = opts ? opts->lanes_per_chain : 0;
  if (lanes != 0 && lanes != 1 && lanes != 2 && lanes != 4 && lanes != 8 && lanes != 32)
    return fail(ctx, PMMC_ERR_INVALID, "server: lanes_per_chain must be 0, 1, 2, 4, 8 or 32");
  sv->lanes = lanes;
  size_t budget = opts ? opts->budget_bytes : 0;
  if (budget == 0) {
    size_t fr = 0, tot = 0;
    PMMC_CUDA(ctx, cudaMemGetInfo(&fr, &tot));
    budget = fr / 2;
  }
  sv->budget = budget;
  const int waves = opts && opts->max_waves > 0 ? opts->max_waves : 8;
  sv->max_wave = opts && opts->max_wave_requests > 0 ? opts->max_wave_requests
                                                      : 4 * ctx->sm_count;
  sv->cap_smem = ctx->smem_optin - kCtaHeader;
  arcs_set_smem_limit((int)ctx->smem_optin);
  sv->slots.resize(waves);
  for (auto &sl : sv->slots) {
    PMMC_CUDA(ctx, cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking));
    PMMC_CUDA(ctx, cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming));
  }
  pmmc_server *p = sv.release();
  p->th = std::thread([p] { p->run(); });
  *out = p;
  return PMMC_OK;
}

extern "C" pmmc_status pmmc_server_submit(pmmc_server *sv, const pmmc_arcs_problem *pr,
                                          float step_size, uint64_t seed, long long *ticket) {
  if (!sv || !pr || !ticket) return PMMC_ERR_INVALID;
  pmmc_status st = arcs_validate(sv->ctx, pr);
  if (st != PMMC_OK) return st;
  auto r = std::make_shared<Request>();
  r->pack.add(*pr, 1, step_size, seed, 0);
  const ArcsUnit &U = r->pack.units[0];
  r->n = pr->n;
  const size_t full = arcs_unit_smem(U.n, U.nnz, U.n_mov, U.mov_off >= 0);
  const size_t minimal = arcs_unit_smem_min(U.n);
  if (minimal > sv->cap_smem)
    return fail(sv->ctx, PMMC_ERR_INVALID,
                "server: region of %d beads exceeds the %zu B shared-memory slice a chain "
                "can hold", U.n, sv->cap_smem);
  r->nb_smem = full <= sv->cap_smem;
  // lanes per proposal from the region's own size (large regions: one lane
  // and 32 proposals per window; small ones: more lanes, fewer conflicts)
  r->lanes = sv->lanes > 0 ? sv->lanes : (pr->n >= 1024 ? 1 : pr->n >= 128 ? 2 : 4);
  r->smem_need = (int)(r->nb_smem ? full : minimal);
  ArcsPack probe = r->pack;
  probe.finish();
  r->dev_bytes = layout_of(probe).total;
  std::lock_guard<std::mutex> lock(sv->mu);
  if (sv->stopping) return PMMC_ERR_INVALID;
  if (r->dev_bytes + 16 * kAlign > sv->budget) {
    ++sv->n_rejected;
    return fail(sv->ctx, PMMC_ERR_BUDGET,
                "server: region of %d beads needs %zu device bytes, over the %zu B budget",
                pr->n, r->dev_bytes, sv->budget);
  }
  r->ticket = sv->next_ticket++;
  r->t_submit = Clock::now();
  sv->table[r->ticket] = r;
  sv->queue.push_back(r);
  ++sv->n_submitted;
  *ticket = r->ticket;
  sv->cv_sched.notify_one();
  return PMMC_OK;
}

extern "C" pmmc_status pmmc_server_poll(pmmc_server *sv, long long ticket, int *done) {
  if (!sv || !done) return PMMC_ERR_INVALID;
  std::lock_guard<std::mutex> lock(sv->mu);
  auto it = sv->table.find(ticket);
  if (it == sv->table.end()) return PMMC_ERR_NOT_FOUND;
  const ReqState s = it->second->state;
  *done = (s == ReqState::Done || s == ReqState::Failed || s == ReqState::Cancelled) ? 1 : 0;
  return PMMC_OK;
}

extern "C" pmmc_status pmmc_server_cancel(pmmc_server *sv, long long ticket) {
  if (!sv) return PMMC_ERR_INVALID;
  std::lock_guard<std::mutex> lock(sv->mu);
  auto it = sv->table.find(ticket);
  if (it == sv->table.end()) return PMMC_ERR_NOT_FOUND;
  ReqPtr r = it->second;
  if (r->state != ReqState::Queued) return PMMC_ERR_BUSY;
  for (auto q = sv->queue.begin(); q != sv->queue.end(); ++q)
    if (q->get() == r.get()) {
      sv->queue.erase(q);
      break;
    }
  r->state = ReqState::Cancelled;
  r->t_done = Clock::now();
  sv->cv_done.notify_all();
  return PMMC_OK;
}

extern "C" pmmc_status pmmc_server_wait(pmmc_server *sv, long long ticket, int timeout_ms,
                                        float *pos_out, pmmc_result *res, double *latency_ms) {
  if (!sv) return PMMC_ERR_INVALID;
  std::unique_lock<std::mutex> lock(sv->mu);
  auto it = sv->table.find(ticket);
  if (it == sv->table.end()) return PMMC_ERR_NOT_FOUND;
  ReqPtr r = it->second;
  auto ready = [&] {
    return r->state == ReqState::Done || r->state == ReqState::Failed ||
           r->state == ReqState::Cancelled;
  };
  if (timeout_ms < 0) {
    sv->cv_done.wait(lock, ready);
  } else if (!sv->cv_done.wait_for(lock, std::chrono::milliseconds(timeout_ms), ready)) {
    return PMMC_ERR_TIMEOUT;
  }
  sv->table.erase(ticket);
  lock.unlock();
  if (r->state == ReqState::Cancelled)
    return fail(sv->ctx, PMMC_ERR_CANCELLED, "server: request %lld was cancelled", ticket);
  if (r->state == ReqState::Failed)
    return fail(sv->ctx, r->error, "server: request %lld failed on the device", ticket);
  if (pos_out) memcpy(pos_out, r->pos_out.data(), sizeof(float) * r->pos_out.size());
  if (res) *res = r->res;
  if (latency_ms)
    *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
  return PMMC_OK;
}

extern "C" pmmc_status pmmc_server_get_stats(pmmc_server *sv, pmmc_server_stats *st) {
  if (!sv || !st) return PMMC_ERR_INVALID;
  std::lock_guard<std::mutex> lock(sv->mu);
  pmmc_server_stats s{};
  s.submitted = sv->n_submitted;
  s.completed = sv->n_completed;
  s.rejected = sv->n_rejected;
  s.failed = sv->n_failed;
  s.waves = sv->n_waves;
  s.queued = (long long)sv->queue.size();
  s.bytes_in_use = (long long)sv->bytes_in_use;
  s.bytes_peak = (long long)sv->bytes_peak;
  s.budget_bytes = (long long)sv->budget;
  s.running_peak = sv->running_peak;
  s.waves_peak = sv->waves_peak;
  *st = s;
  return PMMC_OK;
}

extern "C" void pmmc_server_destroy(pmmc_server *sv) {
  if (!sv) return;
  {
    std::lock_guard<std::mutex> lock(sv->mu);
    sv->stopping = true;
  }
  sv->cv_sched.notify_all();
  if (sv->th.joinable()) sv->th.join();
  for (auto &sl : sv->slots) {
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    if (sl.d_blob) cudaFree(sl.d_blob);
    if (sl.h_in) cudaFreeHost(sl.h_in);
    if (sl.h_out) cudaFreeHost(sl.h_out);
    if (sl.ev) cudaEventDestroy(sl.ev);
    if (sl.stream) cudaStreamDestroy(sl.stream);
  }
  delete sv;
}
