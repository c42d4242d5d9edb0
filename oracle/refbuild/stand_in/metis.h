/* METIS stand-in for the reference's decomposition program.  Test infrastructure only.
 * The reference calls METIS only when it splits a mesh into more than one
 * partition (ucs/decomp.cpp:581); the single-partition runs built here never
 * reach these entry points, which abort if called. */
#ifndef PCFD_REFBUILD_METIS_H
#define PCFD_REFBUILD_METIS_H

#include <cstdint>
#include <cstdio>
#include <cstdlib>

typedef int32_t idx_t;
typedef float real_t;

#define METIS_NOPTIONS 40
#define METIS_OK 1

static inline int pcfd_metis_unavailable() {
  std::fprintf(stderr, "metis stand-in: partitioning into more than one part is not built\n");
  std::abort();
}
static inline int METIS_SetDefaultOptions(idx_t*) { return METIS_OK; }
static inline int METIS_PartGraphRecursive(idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*,
                                           real_t*, real_t*, idx_t*, idx_t*, idx_t*) {
  return pcfd_metis_unavailable();
}
static inline int METIS_PartGraphKway(idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*,
                                      real_t*, real_t*, idx_t*, idx_t*, idx_t*) {
  return pcfd_metis_unavailable();
}

#endif
