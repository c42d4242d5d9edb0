// Runs include/ucs_shim/pcfd_shim.h's ChemModelFrom on the reference's own
// ChemModel (test infrastructure only): the model is built by the
// reference's constructor from <case dir>/<name>.rxn and the species
// database of chemdb_text.h, converted to pcfd_chem_model by the shim, and
// printed as text ("PCFD key index... value" lines, doubles with 17
// significant digits, among the reference's own messages)
// for tests/test_integration_shim.py to compare with the product's model.
//
// Usage: chem_shim_dump <case dir> <case name>
#include <mpi.h>

#include <cstdio>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>

#include "general.h"
#include "exceptions.h"
#include "bc.h"
#include "mesh.h"
#include "param.h"
#include "eqnset.h"
#include "solutionSpaceBase.h"
#include "solutionSpace.h"
#include "limiters.h"
#include "crs.h"
#include "chem.h"
#include "compressibleFR.h"
#include "h5layer.h"
#include "chemdb_text.h"
#include "pcfd_shim.h"

int main(int argc, char* argv[]) {
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s <case dir> <case name>\n", argv[0]);
    return 1;
  }
  std::string dir = argv[1];
  if (dir.empty() || dir[dir.size() - 1] != '/') dir += "/";
  MPI_Init(&argc, &argv);
  HDF_TurnOffErrorHandling();
  if (write_chem_db(dir) != 0) {
    std::fprintf(stderr, "chemistry database write failed\n");
    return 2;
  }
  ChemModel<double> chem(dir + argv[2], dir + "chemdb.h5");
  pcfd_chem_model m;
  pcfd_shim::ChemModelFrom(&chem, m);
  std::printf("PCFD nspecies %d\nPCFD nreactions %d\n", m.nspecies, m.nreactions);
  for (int k = 0; k < m.nspecies; k++) {
    std::printf("PCFD mw %d %.17g\n", k, m.mw[k]);
    for (int i = 0; i < 7; i++) std::printf("PCFD nasa_lo %d %d %.17g\nPCFD nasa_hi %d %d %.17g\n", k, i, m.nasa_lo[k][i], k, i,
                                            m.nasa_hi[k][i]);
    std::printf("PCFD nmu %d %d\nPCFD nk %d %d\n", k, m.nmu[k], k, m.nk[k]);
    for (int r = 0; r < m.nmu[k]; r++)
      for (int i = 0; i < 6; i++) std::printf("PCFD mu_fit %d %d %d %.17g\n", k, r, i, m.mu_fit[k][r][i]);
    for (int r = 0; r < m.nk[k]; r++)
      for (int i = 0; i < 6; i++) std::printf("PCFD k_fit %d %d %d %.17g\n", k, r, i, m.k_fit[k][r][i]);
  }
  for (int j = 0; j < m.nreactions; j++) {
    const pcfd_chem_reaction& c = m.rx[j];
    std::printf("PCFD type %d %d\nPCFD A %d %.17g\nPCFD EA %d %.17g\nPCFD n %d %.17g\nPCFD third_bodies %d %d\nPCFD nlocal %d %d\n", j, c.type, j,
                c.A, j, c.EA, j, c.n, j, c.third_bodies, j, c.nlocal);
    for (int l = 0; l < c.nlocal; l++)
      std::printf("PCFD global %d %d %d\nPCFD nup %d %d %.17g\nPCFD nupp %d %d %.17g\nPCFD tbeff %d %d %.17g\n", j, l, c.global[l], j, l,
                  c.nup[l], j, l, c.nupp[l], j, l, c.tbeff[l]);
  }
  std::fflush(stdout);
  std::_Exit(0);
}
