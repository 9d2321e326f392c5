// ref_hc_harness.cpp -- test infrastructure: drives the reference's
// equidistant-model interpolation (HierarchicalChromosome::gpuHelper,
// src/HierarchicalChromosome.cu:1253-1447) through its CPU path (on a host
// without a GPU, gpuHelper takes its own CPU fallback) to record golden
// outputs.  Built from the reference sources where they lie by
// oracle/Makefile into oracle/_ref/libpmmc_ref_hc.so; never shipped.
#include <fcntl.h>
#include <unistd.h>

#include <cstdio>
#include <cstring>
#include <algorithm>
#include <map>
#include <optional>
#include <string>
#include <vector>

#define private public
#include <HierarchicalChromosome.h>
#undef private

namespace {
struct QuietHC {
  int saved = -1;
  QuietHC() {
    fflush(stdout);
    saved = dup(1);
    int dn = open("/dev/null", O_WRONLY);
    if (dn >= 0) {
      dup2(dn, 1);
      close(dn);
    }
  }
  ~QuietHC() {
    fflush(stdout);
    if (saved >= 0) {
      dup2(saved, 1);
      close(saved);
    }
  }
};
}  // namespace

// One chromosome whose current level holds n clusters (genomic position,
// start, end, xyz); writes up to cap points (xyz) and returns their count,
// -1 when gpuHelper returns nothing.
extern "C" int ref_equidistant(int n, const int *gpos, const int *start, const int *end,
                               const float *pos, int pos_start, int pos_stop, int res,
                               float *out, int cap) {
  QuietHC q;
  HierarchicalChromosome hc;
  const std::string chr = "chr1";
  hc.chrs.push_back(chr);
  hc.clusters.resize(n);
  std::vector<int> level(n);
  for (int i = 0; i < n; ++i) {
    Cluster &c = hc.clusters[i];
    c.genomic_pos = gpos[i];
    c.start = start[i];
    c.end = end[i];
    c.pos = vector3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
    level[i] = i;
  }
  hc.current_level[chr] = level;
  auto r = hc.gpuHelper(pos_start, pos_stop, res, chr);
  if (!r.has_value()) return -1;
  const int m = (int)r.value().size();
  // float3 is three packed floats
  static_assert(sizeof(r.value()[0]) == 3 * sizeof(float), "float3 layout");
  if (m > 0) memcpy(out, r.value().data(), sizeof(float) * 3 * (size_t)std::min(m, cap));
  return m;
}
