// hcm.cu -- writer of the reference's HCM model file (host code).
//
// HierarchicalChromosome::toFile (src/HierarchicalChromosome.cu:530-552):
//   "%d %d %d %d\n"            clusters, factors, -1, chromosomes
//   "%s " per factor, "\n"
//   one line per cluster        Cluster::toFile (Cluster.hpp:175-181):
//                               "%d %d %c %f %f %f %zu" start end orientation
//                               x y z #children, then " %d" per child, "\n"
//   per chromosome              "%s %d %d\n" name root #arcs, then one line
//                               per arc, InteractionArc::toFile
//                               (InteractionArc.hpp:122-125):
//                               "%d %d %d %d %d %d %d\n" start end
//                               genomic_start genomic_end score eff_score
//                               factor
// The annealers write positions into plain arrays; a caller that keeps its
// own tree (the shim keeps the reference's) writes the same file with this.
#include <cstdio>
#include <string>

#include "internal.h"

using namespace pmmc;

extern "C" pmmc_status pmmc_hcm_write(const char *path, int n_clusters, const int *start,
                                      const int *end, const char *orientation,
                                      const float *pos, const int *child_ptr,
                                      const int *children, int n_factors,
                                      const char *const *factors, int n_chrs,
                                      const char *const *chr_names, const int *chr_root,
                                      const int *arc_ptr, const int *arcs) {
  if (!path || n_clusters < 0 || n_factors < 0 || n_chrs < 0 ||
      (n_clusters > 0 && (!start || !end || !orientation || !pos || !child_ptr)) ||
      (n_factors > 0 && !factors) || (n_chrs > 0 && (!chr_names || !chr_root || !arc_ptr)))
    return PMMC_ERR_INVALID;
  if (n_clusters > 0 && child_ptr[n_clusters] > 0 && !children) return PMMC_ERR_INVALID;
  if (n_chrs > 0 && arc_ptr[n_chrs] > 0 && !arcs) return PMMC_ERR_INVALID;
  FILE *f = fopen(path, "w");
  if (!f) return PMMC_ERR_INVALID;
  fprintf(f, "%d %d %d %d\n", n_clusters, n_factors, -1, n_chrs);
  for (int i = 0; i < n_factors; ++i) fprintf(f, "%s ", factors[i]);
  fprintf(f, "\n");
  for (int i = 0; i < n_clusters; ++i) {
    const int c0 = child_ptr[i], c1 = child_ptr[i + 1];
    fprintf(f, "%d %d %c %f %f %f %zu", start[i], end[i], orientation[i], (double)pos[3 * i],
            (double)pos[3 * i + 1], (double)pos[3 * i + 2], (size_t)(c1 - c0));
    for (int k = c0; k < c1; ++k) fprintf(f, " %d", children[k]);
    fprintf(f, "\n");
  }
  for (int c = 0; c < n_chrs; ++c) {
    const int a0 = arc_ptr[c], a1 = arc_ptr[c + 1];
    fprintf(f, "%s %d %d\n", chr_names[c], chr_root[c], a1 - a0);
    for (int k = a0; k < a1; ++k) {
      const int *a = arcs + 7 * (size_t)k;
      fprintf(f, "%d %d %d %d %d %d %d\n", a[0], a[1], a[2], a[3], a[4], a[5], a[6]);
    }
  }
  const bool ok = ferror(f) == 0;
  fclose(f);
  return ok ? PMMC_OK : PMMC_ERR_INVALID;
}
