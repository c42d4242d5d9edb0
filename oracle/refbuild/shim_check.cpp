// Compiles include/ucs_shim/pcfd_shim.h against the reference's own headers
// and instantiates every function for the solver's Type = double, so that a
// renamed member or a changed signature on either side fails the build.
// Test infrastructure: built by `make shim-check`, nothing links it.
#include <mpi.h>

#include <iostream>
#include <sstream>
#include <string>
#include <vector>

// the reference's own include order (its headers are not self-contained)
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
#include "pcfd_shim.h"

template void pcfd_shim::GatherMesh<double>(Mesh<double>*, pcfd_shim::MeshArrays&);
template pcfd_solver_t pcfd_shim::Create<double>(SolutionSpace<double>*);
template void pcfd_shim::PushState<double>(SolutionSpace<double>*, pcfd_solver_t);
template void pcfd_shim::PullState<double>(SolutionSpace<double>*, pcfd_solver_t);
template std::vector<double> pcfd_shim::ComputeResiduals<double>(SolutionSpace<double>*, pcfd_solver_t);
template void pcfd_shim::UpdateBCsGradientLimiter<double>(SolutionSpace<double>*, pcfd_solver_t);
template double pcfd_shim::ComputeTimesteps<double>(SolutionSpace<double>*, pcfd_solver_t, double*);
template double pcfd_shim::JacobianAndSGS<double>(SolutionSpace<double>*, pcfd_solver_t);
template double pcfd_shim::NewtonIterate<double>(SolutionSpace<double>*, pcfd_solver_t, int, int);
template void pcfd_shim::ChemModelFrom<double>(const ChemModel<double>*, pcfd_chem_model&);
template pcfd_chem_ref pcfd_shim::ChemRefFrom<double>(const Param<double>*);
template pcfd_chem_t pcfd_shim::ChemCreate<double>(SolutionSpace<double>*, CompressibleFREqnSet<double>*,
                                                   pcfd_shim::MeshArrays&);
template void pcfd_shim::ChemBCs<double>(SolutionSpace<double>*, pcfd_shim::ChemBCTables&);
template void pcfd_shim::ReactingSpatialResidual<double>(SolutionSpace<double>*, CompressibleFREqnSet<double>*,
                                                         pcfd_chem_t);
