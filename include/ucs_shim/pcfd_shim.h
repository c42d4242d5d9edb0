// The reference-side binding of libpcfd: a header a ProteusCFD maintainer adds
// to ucs/ (compiled only with -DPCFD_GPU) so that the single-partition solver
// runs its hot path through the C ABI of include/pcfd.h.  It keeps the
// reference's types and call sites; each function names the reference
// function it stands in for (ngcurrier/ProteusCFD file:line).
//
// Include after the reference's solutionSpace.h, bc.h, crs.h and param.h.
#ifndef PCFD_SHIM_H__
#define PCFD_SHIM_H__

#include <string>
#include <vector>

#include "pcfd.h"

namespace pcfd_shim {

// Any non-zero status ends the run as the reference ends one (Abort <<,
// ucs/exceptions.h:30), with the library's message.
inline void Check(int status, const char* call)
{
  if (status != PCFD_OK) {
    Abort << std::string(call) + ": " + pcfd_last_error();
  }
}

// The mesh arrays as pcfd_mesh_view expects them.  Edges and HalfEdges are
// structs ({Int n[2]; Type a[4]; ...}, ucs/uns_base.h:13,28), so their node
// pairs, normals and face tags are gathered into flat arrays first.
struct MeshArrays {
  std::vector<int> edges, bedges, factag, ipsp, psp;
  std::vector<double> edge_area, bedge_area;
  pcfd_mesh_view view;
};

template <class Type>
void GatherMesh(Mesh<Type>* m, MeshArrays& a)
{
  const Int nedge = m->GetNumEdges();
  const Int nbedge = m->GetNumBoundaryEdges();
  const Int nnode = m->GetNumNodes();
  a.edges.resize(2 * nedge);
  a.edge_area.resize(4 * nedge);
  a.bedges.resize(2 * nbedge);
  a.bedge_area.resize(4 * nbedge);
  a.factag.resize(nbedge);
  for (Int i = 0; i < nedge; i++) {
    a.edges[2 * i] = m->edges[i].n[0];
    a.edges[2 * i + 1] = m->edges[i].n[1];
    for (int k = 0; k < 4; k++) a.edge_area[4 * i + k] = m->edges[i].a[k];
  }
  for (Int i = 0; i < nbedge; i++) {
    a.bedges[2 * i] = m->bedges[i].n[0];
    a.bedges[2 * i + 1] = m->bedges[i].n[1];
    a.factag[i] = m->bedges[i].factag;
    for (int k = 0; k < 4; k++) a.bedge_area[4 * i + k] = m->bedges[i].a[k];
  }
  // Int is the reference's index type; the ABI takes int
  a.ipsp.assign(m->ipsp, m->ipsp + nnode + 1);
  a.psp.assign(m->psp, m->psp + m->ipsp[nnode]);
  pcfd_mesh_view& v = a.view;
  v.nnode = nnode;
  v.nbnode = m->GetNumBoundaryNodes();
  v.nedge = nedge;
  v.nbedge = nbedge;
  v.edges = a.edges.data();
  v.edge_area = a.edge_area.data();
  v.bedges = a.bedges.data();
  v.bedge_area = a.bedge_area.data();
  v.bfactag = a.factag.data();
  v.xyz = m->xyz;
  v.vol = m->vol;
  v.sw = m->sw;
  v.ipsp = a.ipsp.data();
  v.psp = a.psp.data();
}

// A device solver on the space's mesh and parameters, created after
// SolutionSpace<T>::Init (ucs/solutionSpace.tcc:148); the handle copies the
// mesh to the device once and keeps no pointer into the caller's memory.
template <class Type>
pcfd_solver_t Create(SolutionSpace<Type>* space)
{
  Mesh<Type>* m = space->m;
  Param<Type>* p = space->param;
  MeshArrays a;
  GatherMesh(m, a);
  // the BC table indexed by factag (BoundaryConditions::GetBCType /
  // GetBCObj, ucs/bc.tcc:71,77); the enum values are the reference's
  std::vector<int> bct(space->bc->num_bcs + 1);
  std::vector<double> tw(space->bc->num_bcs + 1);
  for (Int t = 0; t <= space->bc->num_bcs; t++) {
    bct[t] = space->bc->GetBCType(t);
    tw[t] = space->bc->GetBCObj(t)->twall;
  }
  pcfd_params prm = {};
  prm.gamma = p->gamma;
  prm.mach = p->GetVelocity(space->iter);
  for (int k = 0; k < 3; k++) prm.flowdir[k] = p->flowdir[k];
  prm.Re = p->Re;
  prm.Pr = p->Pr;
  prm.PrT = p->PrT;
  prm.ref_temperature = p->ref_temperature;
  prm.sorder = p->sorder;
  prm.chi = p->chi;
  prm.viscous = p->viscous;
  prm.limiter = p->limiter;
  prm.venkat_K = 1.0;  // Kernel_VenkatMod's constant (ucs/limiters.tcc:563)
  prm.no_cvbc = p->no_cvbc;
  prm.jac_boundary_eval = p->boundaryJacEval;
  prm.ntags = (int)bct.size();
  prm.bc_type = bct.data();
  prm.bc_twall = tw.data();
  prm.torder = p->torder;
  prm.time_step = p->dt;
  // CompressibleEqnSet::UpdateQinf's freestream (ucs/compressible.tcc:835-836)
  prm.tinf = p->initialTemperature / p->ref_temperature;
  prm.pinf = p->initialPressure / p->ref_pressure;
  pcfd_solver_t h = nullptr;
  Check(pcfd_create(&a.view, &prm, &h), "pcfd_create");
  return h;
}

// The host state onto the device: q [nnode+nbnode][neqn+naux] in the
// reference's layout (ucs/compressible.tcc:11-22).
template <class Type>
void PushState(SolutionSpace<Type>* space, pcfd_solver_t h)
{
  Mesh<Type>* m = space->m;
  const int nvars = space->eqnset->neqn + space->eqnset->nauxvars;
  Check(pcfd_set_state(h, space->q, nvars, m->GetNumNodes() + m->GetNumBoundaryNodes()), "pcfd_set_state");
}

template <class Type>
void PullState(SolutionSpace<Type>* space, pcfd_solver_t h)
{
  Mesh<Type>* m = space->m;
  const int nvars = space->eqnset->neqn + space->eqnset->nauxvars;
  Check(pcfd_get_state(h, space->q, nvars, m->GetNumNodes() + m->GetNumBoundaryNodes()), "pcfd_get_state");
}

// ComputeResiduals (ucs/residual.tcc:13): b into the CRS right-hand side,
// returned as the reference returns its norms (resGlobal, then per equation).
template <class Type>
std::vector<Type> ComputeResiduals(SolutionSpace<Type>* space, pcfd_solver_t h)
{
  double norms[6];
  Check(pcfd_residual(h, space->crs->b, norms), "pcfd_residual");
  return std::vector<Type>(norms, norms + 1 + space->eqnset->neqn);
}

// UpdateBCs (ucs/bc.tcc:1400), Gradient<T>::Compute (ucs/gradient.tcc:57)
// and Limiter<T>::Compute (ucs/limiters.tcc:53), each with its result copied
// to the reference's array for host code that reads it.
template <class Type>
void UpdateBCsGradientLimiter(SolutionSpace<Type>* space, pcfd_solver_t h)
{
  Check(pcfd_update_bcs(h), "pcfd_update_bcs");
  Check(pcfd_gradient(h, space->qgrad), "pcfd_gradient");
  if (space->param->limiter) Check(pcfd_limiter(h, space->limiter->l), "pcfd_limiter");
}

// ComputeTimesteps (ucs/timestep.tcc:7): local steps into dt, returns dtmin.
template <class Type>
Type ComputeTimesteps(SolutionSpace<Type>* space, pcfd_solver_t h, Type* dt)
{
  double dtmin = 0.0;
  Check(pcfd_timestep(h, space->param->GetCFL(), dt, &dtmin), "pcfd_timestep");
  return dtmin;
}

// ComputeJacobians + CRSMatrix::PrepareSGS (ucs/jacobian.tcc:13,
// ucs/crsmatrix.tcc:840), then CRS<T>::SGS (ucs/crs.tcc:62) into crs->x.
template <class Type>
Type JacobianAndSGS(SolutionSpace<Type>* space, pcfd_solver_t h)
{
  double dq = 0.0;
  Check(pcfd_jacobian(h), "pcfd_jacobian");
  Check(pcfd_sgs(h, space->param->nSgs, space->crs->x, &dq), "pcfd_sgs");
  return dq;
}

// One outer iteration in the reference's order, PreTimeAdvance then
// NewtonIterate (ucs/solutionSpace.tcc:573,640), with q, b, the Jacobian and
// x kept on the device.  Returns resGlobal, the norm the reference keeps for
// its CFL scaling (SolutionSpace::residual).
template <class Type>
Type NewtonIterate(SolutionSpace<Type>* space, pcfd_solver_t h, int linear_solver = 0, int jac_precision = 0)
{
  Param<Type>* p = space->param;
  pcfd_newton_opts o = {};
  o.iter = space->iter;
  o.cfl = p->cfl;
  o.cfl_start = p->cflStart;
  o.cfl_ramp_steps = p->cflRampingSteps;
  o.nsgs = p->nSgs;
  o.jac_update_freq = p->jacobianFreq;
  o.jac_precision = jac_precision;
  o.linear_solver = linear_solver;
  o.fgmres_m = 30;
  o.fgmres_restarts = 1;
  o.fgmres_rtol = 0.1;
  o.limiter_refresh = p->limiterRefresh;
  o.limiter_freeze = p->limiterFreeze;
  o.first_order_steps = p->nFirstOrderSteps;
  pcfd_newton_report r;
  Check(pcfd_newton_step(h, &o, &r), "pcfd_newton_step");
  return r.res[0];
}

}  // namespace pcfd_shim

#endif
