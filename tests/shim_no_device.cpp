// Test driver (CPU test infrastructure): builds a 4-bead active region in the
// reference's LooperSolver and calls the drop-in parallelMonteCarloArcs on a
// host without a CUDA device.  The drop-in must
// end the program with the library's status and message, as the reference's
// gpuErrchk does on a CUDA error; it must not fall back to a CPU annealer.
// argv[1]: a one-line BED file for Settings::dataSegmentsSplit.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <iostream>
#include <map>
#include <random>
#include <set>
#include <sstream>
#include <vector>

#define private public
#define protected public
#include <AppCommon.hpp>
#include <Static.hpp>
#include <LooperSolver.hpp>
#undef private
#undef protected

int main(int argc, char **argv) {
  if (argc < 2) return 64;
  Settings st;
  st.init();
  Settings::dataSegmentsSplit = argv[1];
  Settings::outputLevel = 0;
  LooperSolver s("drop-in", "/tmp/");
  const int n = 4;
  s.clusters.assign(n, Cluster());
  s.active_region.clear();
  for (int i = 0; i < n; ++i) {
    s.clusters[i].pos.set((float)i, 0.0f, 0.0f);
    s.active_region.push_back(i);
  }
  s.heatmap_exp_dist_anchor.init(n);
  for (int i = 0; i < n; ++i)
    for (int j = 0; j < n; ++j) s.heatmap_exp_dist_anchor.v[i][j] = -1.0f;
  s.heatmap_exp_dist_anchor.v[0][3] = s.heatmap_exp_dist_anchor.v[3][0] = 1.5f;
  const float score = s.parallelMonteCarloArcs(0.5f);
  printf("returned %f\n", score);
  return 0;
}
