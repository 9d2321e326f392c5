// markarcs.cu -- genomic arcs -> anchor-index arcs (InteractionArcs::markArcs).
//
// For every raw arc the reference scans all anchors and keeps, for each end,
// the LAST anchor of length > 1 that contains the position
// (InteractionArcs.hpp:242-249, ParallelMarkArcs.cu:48-62).  With anchors
// sorted by start that anchor is found by a binary search for the last
// anchor starting at or before the position, followed by a backward scan
// that stops as soon as no earlier eligible anchor can reach the position
// (prefix maximum of the eligible anchors' ends) -- exact also for
// overlapping anchors, and O(log A) for the usual disjoint ones.  One thread
// per raw arc.  The host then merges arcs between the same anchor pair
// exactly as the CPU markArcs does (:263-327).
#include <algorithm>
#include <climits>
#include <map>
#include <vector>

#include "common.cuh"
#include "internal.h"

namespace pmmc {

__device__ __forceinline__ int find_anchor(int pos, int A, const int *__restrict__ st,
                                           const int *__restrict__ en,
                                           const int *__restrict__ pmax) {
  int lo = 0, hi = A - 1, J = -1;
  while (lo <= hi) {
    const int mid = (lo + hi) >> 1;
    if (st[mid] <= pos) {
      J = mid;
      lo = mid + 1;
    } else {
      hi = mid - 1;
    }
  }
  for (int j = J; j >= 0; --j) {
    if (pmax[j] < pos) return -1;
    const int len = (st[j] == 0 && en[j] == 0) ? 0 : en[j] - st[j] + 1;
    if (len > 1 && en[j] >= pos) return j;
  }
  return -1;
}

__global__ void mark_arcs_kernel(int A, const int *__restrict__ a_st,
                                 const int *__restrict__ a_en,
                                 const int *__restrict__ pmax, int R,
                                 const int2 *__restrict__ raw, int2 *__restrict__ out) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < R; i += gridDim.x * blockDim.x) {
    const int2 r = raw[i];
    out[i] = make_int2(find_anchor(r.x, A, a_st, a_en, pmax),
                       find_anchor(r.y, A, a_st, a_en, pmax));
  }
}

}  // namespace pmmc

using namespace pmmc;

namespace {

struct RawArc {
  int start, end, score, factor, order;
};

struct Arc7 {
  int start, end, gstart, gend, score, eff, factor, order;
};

bool raw_less(const RawArc &a, const RawArc &b) {
  if (a.start != b.start) return a.start < b.start;
  if (a.end != b.end) return a.end < b.end;
  if (a.factor != b.factor) return a.factor < b.factor;
  return a.order < b.order;
}

}  // namespace

extern "C" pmmc_status pmmc_mark_arcs(pmmc_ctx *ctx, int n_anchors, const int *a_start,
                                      const int *a_end, int n_raw, const int *r_start,
                                      const int *r_end, const int *r_score,
                                      const int *r_factor, int *out, int cap, int *n_out,
                                      int *n_non_matching) {
  if (!ctx || n_anchors < 0 || n_raw < 0 || (n_anchors > 0 && (!a_start || !a_end)) ||
      (n_raw > 0 && (!r_start || !r_end || !r_score || !r_factor)) || !n_out)
    return fail(ctx, PMMC_ERR_INVALID, "mark arcs: bad arguments");
  for (int j = 1; j < n_anchors; ++j)
    if (a_start[j] < a_start[j - 1])
      return fail(ctx, PMMC_ERR_INVALID, "mark arcs: anchors must be sorted by start");
  // sort raw arcs by (start, end, factor) (InteractionArc::operator<)
  std::vector<RawArc> raw(n_raw);
  for (int i = 0; i < n_raw; ++i) raw[i] = {r_start[i], r_end[i], r_score[i], r_factor[i], i};
  std::sort(raw.begin(), raw.end(), raw_less);
  std::vector<int> pmax(std::max(n_anchors, 1), INT_MIN);
  int m = INT_MIN;
  for (int j = 0; j < n_anchors; ++j) {
    const int len = (a_start[j] == 0 && a_end[j] == 0) ? 0 : a_end[j] - a_start[j] + 1;
    if (len > 1) m = std::max(m, a_end[j]);
    pmax[j] = m;
  }
  std::vector<int2> hraw(std::max(n_raw, 1));
  for (int i = 0; i < n_raw; ++i) hraw[i] = make_int2(raw[i].start, raw[i].end);
  std::vector<int2> idx(std::max(n_raw, 1));
  if (n_raw > 0 && n_anchors > 0) {
    cudaStream_t s = ctx->stream;
    std::vector<int> hs(a_start, a_start + n_anchors), he(a_end, a_end + n_anchors);
    DevBuf<int> d_s, d_e, d_pm;
    DevBuf<int2> d_raw, d_out;
    cudaError_t e = d_s.upload(hs, s);
    if (e == cudaSuccess) e = d_e.upload(he, s);
    pmax.resize(n_anchors);
    if (e == cudaSuccess) e = d_pm.upload(pmax, s);
    hraw.resize(n_raw);
    if (e == cudaSuccess) e = d_raw.upload(hraw, s);
    if (e == cudaSuccess) e = d_out.alloc(n_raw);
    if (e != cudaSuccess)
      return fail(ctx, PMMC_ERR_CUDA, "mark arcs upload: %s", cudaGetErrorString(e));
    const int threads = 256;
    const int grid = std::min((n_raw + threads - 1) / threads, ctx->sm_count * 8);
    mark_arcs_kernel<<<grid, threads, 0, s>>>(n_anchors, d_s.p, d_e.p, d_pm.p, n_raw, d_raw.p,
                                              d_out.p);
    PMMC_CUDA(ctx, cudaGetLastError());
    PMMC_CUDA(ctx, cudaMemcpyAsync(idx.data(), d_out.p, sizeof(int2) * n_raw,
                                   cudaMemcpyDeviceToHost, s));
    PMMC_CUDA(ctx, cudaStreamSynchronize(s));
  } else {
    for (int i = 0; i < n_raw; ++i) idx[i] = make_int2(-1, -1);
  }
  // ---- host merge (InteractionArcs.hpp:238-328) ----
  int cnt = 0, nm = 0, last_start = -1;
  std::map<int, std::vector<Arc7>> tmp;  // keyed by end anchor, ascending
  auto emit = [&](const Arc7 &a) {
    if (cnt < cap && out) {
      int *o = out + 7 * cnt;
      o[0] = a.start;
      o[1] = a.end;
      o[2] = a.gstart;
      o[3] = a.gend;
      o[4] = a.score;
      o[5] = a.eff;
      o[6] = a.factor;
    }
    ++cnt;
  };
  auto flush = [&]() {
    for (auto &kv : tmp) {
      std::vector<Arc7> &el = kv.second;
      if (el.size() == 1) {
        emit(el[0]);
        continue;
      }
      std::stable_sort(el.begin(), el.end(), [](const Arc7 &a, const Arc7 &b) {
        if (a.start != b.start) return a.start < b.start;
        if (a.end != b.end) return a.end < b.end;
        return a.factor < b.factor;
      });
      bool multiple = false;
      for (size_t j = 1; j < el.size(); ++j)
        if (el[j].factor != el[j - 1].factor) multiple = true;
      int total = 0, fscore = 0;
      size_t first = 0;
      for (size_t j = 0; j <= el.size(); ++j) {
        if (j == el.size() || (j > 0 && el[j].factor != el[j - 1].factor)) {
          Arc7 r = el[first];
          r.score = fscore;
          r.eff = multiple ? 0 : fscore;
          emit(r);
          first = j;
          total += fscore;
          fscore = 0;
        }
        if (j < el.size()) fscore += el[j].score;
      }
      if (multiple) {
        Arc7 r{el[0].start, kv.first, -1, -1, 0, total, -1, 0};
        emit(r);
      }
    }
    tmp.clear();
  };
  for (int i = 0; i <= n_raw; ++i) {
    int st = -1, en = -1;
    if (i < n_raw) {
      st = idx[i].x;
      en = idx[i].y;
      if (st == -1 || en == -1) {
        ++nm;
        continue;
      }
      if (st == en) continue;  // looping arc
    }
    if (st != last_start || i == n_raw) {
      flush();
      last_start = st;
    }
    if (i < n_raw) {
      Arc7 a{st, en, raw[i].start, raw[i].end, raw[i].score, raw[i].score, raw[i].factor,
             (int)tmp[en].size()};
      tmp[en].push_back(a);
    }
  }
  *n_out = cnt;
  if (n_non_matching) *n_non_matching = nm;
  if (cnt > cap) return fail(ctx, PMMC_ERR_INVALID, "mark arcs: %d arcs exceed cap %d", cnt, cap);
  return PMMC_OK;
}
