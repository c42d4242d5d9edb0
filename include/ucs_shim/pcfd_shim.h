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

// ---- the reacting equation set (CompressibleFREqnSet) ----------------------
// Include the reference's chem.h and compressibleFR.h too.

// The chemistry the equation set owns (CompressibleFREqnSet::chem,
// ucs/compressibleFR.tcc:39) as pcfd_chem_model: per species the molecular
// weight (kg/mol after Species::GetDBInfo's division, ucs/species.tcc:162-167),
// the NASA-7 fits below and above 1000 K (thermo_coeff[0], [1]; the third
// range repeats the second) and the viscosity and conductivity fits; per
// reaction its rate law and its species with their global indices,
// stoichiometric coefficients and third-body efficiencies (ucs/reaction.h).
template <class Type>
void ChemModelFrom(const ChemModel<Type>* chem, pcfd_chem_model& m)
{
  m = pcfd_chem_model{};
  if (chem->nspecies > PCFD_CHEM_MAX_SPECIES || chem->nreactions > PCFD_CHEM_MAX_REACTIONS) {
    Abort << std::string("pcfd_shim::ChemModelFrom: mechanism larger than the library's limits");
  }
  m.nspecies = chem->nspecies;
  for (Int k = 0; k < chem->nspecies; k++) {
    const Species<Type>& s = chem->species[k];
    m.mw[k] = s.MW;
    for (int i = 0; i < 7; i++) {
      m.nasa_lo[k][i] = s.thermo_coeff[0][i];
      m.nasa_hi[k][i] = s.thermo_coeff[1][i];
    }
    m.nmu[k] = s.mu_coeff_curves;
    m.nk[k] = s.k_coeff_curves;
    for (Int r = 0; r < s.mu_coeff_curves; r++)
      for (int i = 0; i < 6; i++) m.mu_fit[k][r][i] = s.mu_coeff[r][i];
    for (Int r = 0; r < s.k_coeff_curves; r++)
      for (int i = 0; i < 6; i++) m.k_fit[k][r][i] = s.k_coeff[r][i];
  }
  m.nreactions = chem->nreactions;
  for (Int j = 0; j < chem->nreactions; j++) {
    const Reaction<Type>& r = chem->reactions[j];
    pcfd_chem_reaction& c = m.rx[j];
    // the reaction's species, third bodies included (Reaction::GetNspecies)
    const Int nloc = (Int)r.speciesSymbols.size();
    if (nloc > PCFD_CHEM_MAX_LOCAL) {
      Abort << std::string("pcfd_shim::ChemModelFrom: reaction with too many species");
    }
    c.type = r.rxnType;
    c.A = r.A;
    c.EA = r.EA;
    c.n = r.n;
    c.third_bodies = r.thirdBodiesPresent ? 1 : 0;
    c.nlocal = nloc;
    for (Int l = 0; l < nloc; l++) {
      c.global[l] = r.globalIndx[l];
      c.nup[l] = r.Nup[l];
      c.nupp[l] = r.Nupp[l];
      // TBEff is filled only for third-body reactions (Reaction::ParseThirdBodies)
      c.tbeff[l] = (size_t)l < r.TBEff.size() ? r.TBEff[l] : 1.0;
    }
  }
}

// The reference scales the reacting set is non-dimensional in
// (Param::PostCompute, ucs/param.tcc:355).
template <class Type>
pcfd_chem_ref ChemRefFrom(const Param<Type>* p)
{
  pcfd_chem_ref r;
  r.density = p->ref_density;
  r.pressure = p->ref_pressure;
  r.temperature = p->ref_temperature;
  r.specific_enthalpy = p->ref_specific_enthalpy;
  r.velocity = p->ref_velocity;
  r.viscosity = p->ref_viscosity;
  r.conductivity = p->ref_k;
  return r;
}

// A reacting handle with the space's mesh attached; keep `a` alive as long
// as the handle is used with pcfd_chem_attach_mesh's arrays.
template <class Type>
pcfd_chem_t ChemCreate(SolutionSpace<Type>* space, CompressibleFREqnSet<Type>* eqn, MeshArrays& a)
{
  pcfd_chem_model m;
  ChemModelFrom(eqn->chem, m);
  pcfd_chem_t h = nullptr;
  Check(pcfd_chem_create(&m, &h), "pcfd_chem_create");
  GatherMesh(space->m, a);
  Check(pcfd_chem_attach_mesh(h, &a.view), "pcfd_chem_attach_mesh");
  return h;
}

// The boundary tables UpdateBCs reads, per face tag (BoundaryConditions,
// ucs/bc.tcc:71,77; BCObj::Qref, which points at the equation set's Qinf
// unless the .bc file gave one, ucs/bc.tcc:51-58).
struct ChemBCTables {
  std::vector<int> type, sym;
  std::vector<double> twall, qref;
};
template <class Type>
void ChemBCs(SolutionSpace<Type>* space, ChemBCTables& t)
{
  EqnSet<Type>* eqn = space->eqnset;
  const int nvars = eqn->neqn + eqn->nauxvars;
  const int ntags = space->bc->num_bcs + 1;
  t.type.assign(ntags, -1);
  t.twall.assign(ntags, 0.0);
  t.qref.assign((size_t)ntags * nvars, 0.0);
  t.sym.clear();
  for (int tag = 0; tag < ntags; tag++) {
    BCObj<Real>* o = space->bc->GetBCObj(tag);
    t.type[tag] = space->bc->GetBCType(tag);
    t.twall[tag] = o->twall;
    std::vector<Real> q(nvars);
    o->GetQref(q.data());
    for (int i = 0; i < nvars; i++) t.qref[(size_t)tag * nvars + i] = q[i];
    if (t.type[tag] == Proteus_Symmetry) t.sym.push_back(tag);
  }
}

// SpatialResidual (ucs/residual.tcc:66) of the reacting set in the
// reference's NewtonIterate order, with q, the gradient and the limiter on
// the host arrays the reference reads: UpdateBCs, Gradient::Compute,
// Limiter::Compute once past the first-order steps, the inviscid residual
// (first order, or second order with the limiter) with the chemistry source,
// plus the viscous residual (the directional correction once second order
// is on).  b goes to crs->b.  The reference's own TemporalResidual and
// boundary-row hook (ucs/residual.tcc:20-40) then run on crs->b as before.
template <class Type>
void ReactingSpatialResidual(SolutionSpace<Type>* space, CompressibleFREqnSet<Type>* eqn, pcfd_chem_t h)
{
  Param<Type>* p = space->param;
  Mesh<Type>* m = space->m;
  const int nnode = m->GetNumNodes();
  const int neqn = eqn->neqn;
  ChemBCTables t;
  ChemBCs(space, t);
  const pcfd_chem_ref ref = ChemRefFrom(p);
  pcfd_chem_flux_opts o;
  o.beta = 1.0;
  o.pref = eqn->Pref;
  o.symmetry2D = 0;
  Check(pcfd_chem_update_bcs(h, &ref, (int)t.type.size(), t.type.data(), t.twall.data(), t.qref.data(), p->no_cvbc,
                             space->q, 0), "pcfd_chem_update_bcs");
  const bool second = p->sorder > 1 && space->iter > p->nFirstOrderSteps;
  if (second || p->viscous)
    Check(pcfd_chem_gradient(h, space->q, t.sym.data(), (int)t.sym.size(), space->qgrad, 0), "pcfd_chem_gradient");
  if (second && p->limiter && space->iter % p->limiterRefresh == 0 && space->iter < p->limiterFreeze)
    Check(pcfd_chem_limiter(h, p->chi, space->q, space->qgrad, space->limiter->l, 0), "pcfd_chem_limiter");
  double norms[1 + PCFD_CHEM_MAX_SPECIES + 4];
  if (second)
    Check(pcfd_chem_residual_ho(h, &ref, &o, p->chi, p->ref_time, p->rxnOn ? 1 : 0, space->q, space->qgrad,
                                space->limiter->l, space->crs->b, norms, 0), "pcfd_chem_residual_ho");
  else
    Check(pcfd_chem_residual(h, &ref, &o, p->ref_time, p->rxnOn ? 1 : 0, space->q, space->crs->b, norms, 0),
          "pcfd_chem_residual");
  if (p->viscous) {
    std::vector<double> bv((size_t)nnode * neqn);
    Check(pcfd_chem_viscous_residual(h, &ref, &o, p->Re, second ? 1 : 0, space->q, space->qgrad, bv.data(), 0),
          "pcfd_chem_viscous_residual");
    for (size_t i = 0; i < bv.size(); i++) space->crs->b[i] += bv[i];
  }
}

}  // namespace pcfd_shim

#endif
