// Golden-output harness around the reference solver (test infrastructure only).
//
// Built by oracle/refbuild/Makefile from the reference's own sources, unmodified,
// with the stand-ins for MPI, HDF5 and METIS in stand_in/.  It runs the
// reference exactly as its programs do and writes what the GPU path must match:
//
//   1. the decomposition step of udecomp.x (ucs/decomp.cpp main, one partition)
//      on <case>.ugrid, which writes the partitioned mesh <case>.0.h5;
//   2. the solver set-up of ucs.x (ReadParamFile, TemporalControl::Read and
//      the SolutionSpace constructor, ucs/main.cpp:165-190,
//      ucs/create_functions.h:91): mesh read, reverse Cuthill-McKee reorder
//      (reorderMesh), maps, dual metrics, LSQ coefficients, CRS set-up;
//   3. the first Newton step of Solve (ucs/solve.tcc:24-60) stage by stage -
//      PreIterate, PreTimeAdvance (ComputeJacobians, ComputeTimesteps), then
//      NewtonIterate's own sequence (ucs/solutionSpace.tcc:640-818): UpdateBCs,
//      Gradient::Compute, Limiter::Compute, ComputeResiduals, PrepareSGS +
//      SGS, ApplyDQ - dumping each stage's output;
//   4. further whole steps (PostTimeAdvance, PreTimeAdvance, NewtonIterate),
//      recording their residual norms and the final state.
//
// An optional <case>.qinit ([nnode][neqn] doubles of the equation set's stored
// variables, in the file's node order) replaces the freestream initial state
// before step 1, so the gradients, limiters and viscous terms are all active.
// An optional <case>/chemdb.txt is written into <case>/chemdb.h5 first, the
// species database a reacting case names (write_chem_db, chemdb_text.h).
//
// Usage: ref_dump <case directory> <case name> <output directory> <steps>
// Output: one raw little-endian file per array plus index.txt
// ("name dtype n0 n1"), read by tests/golden/make_ref_fixtures.py.
#include <mpi.h>

#include <algorithm>
#include <complex>
#include <deque>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <list>
#include <map>
#include <set>
#include <sstream>
#include <string>
#include <vector>

// The harness reads a few of SolutionSpace's private members (the step's
// minimum time step and residual); only this file sees them as public.
#define private public
#define protected public
#include "general.h"
#include "exceptions.h"
#include "bc.h"
#include "mesh.h"
#include "param.h"
#include "eqnset.h"
#include "create_functions.h"
#include "parallel.h"
#include "timer.h"
#include "solutionSpaceBase.h"
#include "solutionSpace.h"
#include "solve.h"
#include "temporalControl.h"
#include "residual.h"
#include "jacobian.h"
#include "timestep.h"
#include "gradient.h"
#include "limiters.h"
#include "crs.h"
#include "crsmatrix.h"
#include "h5layer.h"
#include "chemdb_text.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <string>
#include <vector>

int pcfd_decomp_main(int argc, char* argv[]);  // ucs/decomp.cpp main, renamed at compile time

namespace {

std::string g_out;
std::ofstream g_index;

template <class T>
const char* dtype_name();
template <>
const char* dtype_name<int>() { return "i4"; }
template <>
const char* dtype_name<double>() { return "f8"; }

template <class T>
void dump(const std::string& name, const T* data, long long n0, long long n1 = 1) {
  std::string path = g_out + "/" + name + ".bin";
  FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) { std::fprintf(stderr, "cannot write %s\n", path.c_str()); std::exit(2); }
  if (n0 * n1 > 0) std::fwrite(data, sizeof(T), (size_t)(n0 * n1), f);
  std::fclose(f);
  g_index << name << " " << dtype_name<T>() << " " << n0 << " " << n1 << "\n";
  g_index.flush();
}

void dump_scalar(const std::string& name, double v) { dump(name, &v, 1, 1); }

// Element list as [nelem][11]: type, factag, node count, then up to 8 node ids (-1 pad).
void dump_elements(const std::string& name, std::vector<Element<Real>*>& list) {
  std::vector<int> out(11 * list.size(), -1);
  for (size_t e = 0; e < list.size(); ++e) {
    Int* nodes;
    Int nn = list[e]->GetNodes(&nodes);
    out[11 * e + 0] = list[e]->GetType();
    out[11 * e + 1] = list[e]->GetFactag();
    out[11 * e + 2] = nn;
    for (int k = 0; k < nn && k < 8; ++k) out[11 * e + 3 + k] = nodes[k];
  }
  dump(name, out.data(), (long long)list.size(), 11);
}
void dump_iscalar(const std::string& name, int v) { dump(name, &v, 1, 1); }


// NewtonIterate's own sequence (ucs/solutionSpace.tcc:640-818) with each
// stage's output dumped under the given prefix.
std::vector<Real> newton_stages(SolutionSpace<Real>* space, const std::string& pre) {
  Param<Real>* param = space->param;
  Mesh<Real>* m = space->m;
  EqnSet<Real>* eqn = space->eqnset;
  const int nnode = m->GetNumNodes();
  const int nrows = nnode + m->GetNumParallelNodes() + m->GetNumBoundaryNodes();
  const int neqn = eqn->neqn;
  const int nvars = neqn + eqn->nauxvars;
  const int iter = space->iter;
  dump_iscalar(pre + "iter", iter);
  UpdateBCs(space);
  dump(pre + "q_bc", space->q, nrows, nvars);
  if ((param->sorder > 1 && iter > param->nFirstOrderSteps) || param->viscous) {
    space->grad->Compute();
    dump(pre + "qgrad", space->qgrad, nnode, space->grad->GetNterms() * 3);
  }
  if ((iter % param->limiterRefresh == 0) && (param->sorder > 1) && param->limiter &&
      (iter > param->nFirstOrderSteps) && (iter < param->limiterFreeze)) {
    space->limiter->Compute(space);
    dump(pre + "limiter", space->limiter->l, nnode, neqn);
  }
  std::vector<Real> norms = ComputeResiduals(space);
  space->residualnm1 = space->residual;
  space->residual = norms[0];
  dump(pre + "b", space->crs->b, nnode, neqn);
  dump(pre + "norms", norms.data(), 1, (long long)norms.size());
  if (param->nSgs > 0) {
    space->crs->A->PrepareSGS();
    space->crs->BlankX();
    Real ddq = space->crs->SGS(param->nSgs, NULL, NULL, NULL);
    dump(pre + "x_sgs", space->crs->x, nnode, neqn);
    dump_scalar(pre + "sgs_delta", real(ddq));
    for (int j = 0; j < nnode; ++j) {
      bool zero = false;
      for (int k = 0; k < neqn; ++k)
        if (std::isnan(real(space->crs->x[(size_t)j * neqn + k])) || std::isinf(real(space->crs->x[(size_t)j * neqn + k])))
          zero = true;
      if (zero)
        for (int k = 0; k < neqn; ++k) space->crs->x[(size_t)j * neqn + k] = 0.0;
    }
    for (int j = 0; j < nnode; ++j)
      eqn->ApplyDQ(&space->crs->x[(size_t)j * neqn], &space->q[(size_t)j * nvars], &m->xyz[j * 3]);
    dump(pre + "q", space->q, nnode, nvars);
  }
  return norms;
}

// The pressure and viscous force on composite body 1 as PostTimeAdvance's
// Forces::Compute left them (FORCE_Kernel, ucs/forces.tcc:124), when the
// case defines a body.
void dump_forces(SolutionSpace<Real>* space, const std::string& pre) {
  Forces<Real>* f = space->forces;
  if (!f || f->num_bodies < 1) return;
  double v[6];
  for (int j = 0; j < 3; ++j) {
    v[j] = real(f->bodies[1].forces[j]);
    v[3 + j] = real(f->bodies[1].vforces[j]);
  }
  dump(pre + "forces", v, 1, 6);
}

}  // namespace

int main(int argc, char* argv[]) {
  if (argc != 5) {
    std::fprintf(stderr, "usage: %s <case dir> <case name> <output dir> <steps>\n", argv[0]);
    return 1;
  }
  std::string dir = argv[1];
  if (dir.empty() || dir[dir.size() - 1] != '/') dir += "/";
  std::string casename = argv[2];
  g_out = argv[3];
  int nsteps = std::atoi(argv[4]);
  g_index.open((g_out + "/index.txt").c_str());

  MPI_Init(&argc, &argv);

  // 1. udecomp.x <case>.ugrid 1
  {
    std::string ugrid = dir + casename + ".ugrid";
    std::vector<char> a0(ugrid.begin(), ugrid.end()), a1;
    a0.push_back('\0');
    const char* one = "1";
    char prog[] = "udecomp.x";
    char* dargv[] = {prog, a0.data(), const_cast<char*>(one), nullptr};
    int rc = pcfd_decomp_main(3, dargv);
    if (rc != 0) { std::fprintf(stderr, "decomposition failed (%d)\n", rc); return 3; }
  }

  // 2. ucs.x set-up
  PObj<Real> pobj;
  std::vector<Param<Real>*> paramList;
  TemporalControl<Real> temporalControl;
  HDF_TurnOffErrorHandling();
  if (write_chem_db(dir) != 0) { std::fprintf(stderr, "chemistry database write failed\n"); return 4; }
  Abort.rootDirectory = dir;
  if (ReadParamFile(paramList, casename, dir)) { std::fprintf(stderr, "param read failed\n"); return 4; }
  if (temporalControl.Read(casename, dir)) { std::fprintf(stderr, "temporal control read failed\n"); return 4; }
  Param<Real>* param = paramList[0];
  {
    // the partitioned mesh as the solver reads it, before its reorder
    Mesh<Real> pre;
    pre.SetParallelPointer(&pobj);
    if (pre.ReadPartedMesh(param->path + param->spacename)) { std::fprintf(stderr, "mesh read failed\n"); return 4; }
    dump("xyz_pre", pre.xyz, pre.GetNumNodes(), 3);
    dump_elements("elements_pre", pre.elementList);
  }
  SolutionSpace<Real>* space = new SolutionSpace<Real>(param, &pobj, param->spacename, temporalControl);

  Mesh<Real>* m = space->m;
  EqnSet<Real>* eqn = space->eqnset;
  const int nnode = m->GetNumNodes();
  const int gnode = m->GetNumParallelNodes();
  const int nbnode = m->GetNumBoundaryNodes();
  const int nedge = m->GetNumEdges();
  const int nbedge = m->GetNumBoundaryEdges();
  const int neqn = eqn->neqn;
  const int nvars = neqn + eqn->nauxvars;
  const int nrows = nnode + gnode + nbnode;

  dump_iscalar("nnode", nnode);
  dump_iscalar("gnode", gnode);
  dump_iscalar("nbnode", nbnode);
  dump_iscalar("nedge", nedge);
  dump_iscalar("nbedge", nbedge);
  dump_iscalar("neqn", neqn);
  dump_iscalar("nvars", nvars);
  dump_scalar("gamma", real(param->gamma));
  dump_scalar("Re", real(param->Re));
  dump_scalar("Pr", real(param->Pr));
  dump_scalar("ref_temperature", real(param->ref_temperature));
  dump_scalar("velocity", real(param->GetVelocity(1)));
  dump_scalar("chi", real(param->chi));
  dump_iscalar("sorder", param->sorder);
  dump_iscalar("param_limiter", param->limiter);
  dump_iscalar("viscous", param->viscous);
  dump("qinf", eqn->Qinf, 1, nvars);
  // the non-dimensional freestream temperature and pressure UpdateQinf forms
  // (ucs/compressible.tcc:835-836)
  dump_scalar("qinf_T", real(param->initialTemperature / param->ref_temperature));
  dump_scalar("qinf_p", real(param->initialPressure / param->ref_pressure));
  // the reference scales (Param::PostCompute, ucs/param.tcc:355) the reacting
  // set's non-dimensional arithmetic uses
  {
    double refs[9] = {real(param->ref_density), real(param->ref_pressure), real(param->ref_temperature),
                      real(param->ref_specific_enthalpy), real(param->ref_velocity), real(param->ref_viscosity),
                      real(param->ref_k), real(param->ref_time), real(param->ref_length)};
    dump("refs", refs, 1, 9);
  }

  // mesh maps and metrics (after the reorder, which ucs.x does at set-up)
  dump_elements("elements", m->elementList);
  dump("xyz", m->xyz, nnode, 3);
  dump("vol", m->vol, nnode, 1);
  dump("ipsp", m->ipsp, nnode + 1, 1);
  dump("psp", m->psp, m->ipsp[nnode], 1);
  if (m->ordering) dump("ordering", m->ordering, nnode, 1);
  {
    std::vector<int> en(2 * (size_t)nedge);
    std::vector<double> ea(4 * (size_t)nedge);
    for (int e = 0; e < nedge; ++e) {
      en[2 * e] = m->edges[e].n[0];
      en[2 * e + 1] = m->edges[e].n[1];
      for (int k = 0; k < 4; ++k) ea[4 * e + k] = m->edges[e].a[k];
    }
    dump("edges", en.data(), nedge, 2);
    dump("edge_area", ea.data(), nedge, 4);
    const int nh = m->GetNumParallelEdges() + nbedge;
    std::vector<int> bn(2 * (size_t)nh), bt(nh), bel(nh);
    std::vector<double> ba(4 * (size_t)nh);
    for (int e = 0; e < nh; ++e) {
      bn[2 * e] = m->bedges[e].n[0];
      bn[2 * e + 1] = m->bedges[e].n[1];
      bt[e] = m->bedges[e].factag;
      bel[e] = m->bedges[e].elem;
      for (int k = 0; k < 4; ++k) ba[4 * e + k] = m->bedges[e].a[k];
    }
    dump("bedges", bn.data(), nh, 2);
    dump("bedge_area", ba.data(), nh, 4);
    dump("bfactag", bt.data(), nh, 1);
    dump("belem", bel.data(), nh, 1);
  }
  dump("sw", m->sw, nnode, 6);
  CRSMatrix<Real>* A = space->crs ? space->crs->A : nullptr;
  if (A) {
    dump("ia", A->ia, nnode + 1, 1);
    dump("ja", A->ja, A->ia[nnode], 1);
    dump("iau", A->iau, nnode, 1);
  }

  // optional seeded initial state
  {
    std::ifstream qi((dir + casename + ".qinit").c_str(), std::ios::binary);
    if (qi.is_open()) {
      std::vector<double> q0((size_t)nnode * neqn);
      qi.read(reinterpret_cast<char*>(q0.data()), sizeof(double) * q0.size());
      if (!qi) { std::fprintf(stderr, "short .qinit file\n"); return 5; }
      // .qinit is in the file's node order; the reorder moved node i to ordering[i]
      for (int i = 0; i < nnode; ++i) {
        int j = m->ordering ? m->ordering[i] : i;
        for (int k = 0; k < neqn; ++k) space->q[(size_t)j * nvars + k] = q0[(size_t)i * neqn + k];
        eqn->ComputeAuxiliaryVariables(&space->q[(size_t)j * nvars]);
      }
    }
  }
  dump("q_init", space->q, nrows, nvars);

  // 3. first step, stage by stage
  space->PreIterate();
  dump("dt_preiterate", space->GetFieldData("timestep", FIELDS::STATE_NONE), nnode, 1);
  space->PreTimeAdvance();
  dump("dt", space->GetFieldData("timestep", FIELDS::STATE_NONE), nnode, 1);
  dump_scalar("dtmin", real(space->dtmin));
  dump_scalar("cfl_step1", real(param->GetCFL()));
  if (A) dump("jacobian", A->M, A->nblocks, (long long)neqn * neqn);

  std::vector<Real> norms = newton_stages(space, "s1_");
  space->PostTimeAdvance();
  dump_forces(space, "s1_");
  // the second step is the first with second-order fluxes and a limiter
  // (NewtonIterate tests iter > nFirstOrderSteps; iter starts at 0)
  if (nsteps >= 2) {
    space->PreTimeAdvance();
    dump("s2_dt", space->GetFieldData("timestep", FIELDS::STATE_NONE), nnode, 1);
    if (A) dump("s2_jacobian", A->M, A->nblocks, (long long)neqn * neqn);
    std::vector<Real> n2 = newton_stages(space, "s2_");
    space->PostTimeAdvance();
    dump_forces(space, "s2_");
  }

  // 4. whole steps
  std::vector<double> hist;
  hist.insert(hist.end(), norms.begin(), norms.end());
  for (int s = 3; s <= nsteps; ++s) {
    space->PreTimeAdvance();
    space->NewtonIterate();
    hist.push_back(real(space->residual));
    space->PostTimeAdvance();
  }
  if (nsteps >= 3) {
    dump("resglobal_steps3on", hist.data() + norms.size(), (long long)hist.size() - (long long)norms.size(), 1);
    dump("q_final", space->q, nnode, nvars);
  }
  g_index.close();
  std::_Exit(0);  // skip the reference's teardown (file writers); everything is dumped
}
