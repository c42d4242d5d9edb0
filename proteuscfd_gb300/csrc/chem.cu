// Finite-rate chemistry: mass production rates per node (the per-node
// chemistry of the reacting equation set), one thread per node, the
// mechanism staged in shared memory per block.
//   ChemModel<T>::GetMassProductionRates      ucs/chem.tcc:575
//   Reaction<T>::GetForwardReactionRate       ucs/reaction.tcc:608
//   Reaction<T>::GetEquilibriumReactionRate   ucs/reaction.tcc:629
//   Reaction<T>::GetBackwardReactionRate      ucs/reaction.tcc:683
//   Reaction<T>::GetMassProductionRate        ucs/reaction.tcc:763
//   Species<T>::GetThermoCoeff                ucs/species.tcc:96
// and the node state of the reacting equation set (ideal-gas mixture):
//   CompressibleFREqnSet<T>::NewtonFindTGivenP      ucs/compressibleFR.tcc:2343
//   CompressibleFREqnSet<T>::ConservativeToNative   ucs/compressibleFR.tcc:2133
//   CompressibleFREqnSet<T>::NativeToConservative   ucs/compressibleFR.tcc:2117
//   CompressibleFREqnSet<T>::ComputeAuxiliaryVariables ucs/compressibleFR.tcc:755
// and its inviscid edge flux:
//   CompressibleFREqnSet<T>::HLLCFlux               ucs/compressibleFR.tcc:301
// and its first-order inviscid residual (SpatialResidual, ucs/residual.tcc:66).
// The reference evaluates each reaction's rates once per species it
// produces; here each reaction is evaluated once per node and its
// contribution added to every species it changes, in reaction order, which
// is the order each species' sum has in the reference.
#include "../../include/pcfd.h"

#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

void pcfd_set_last_error(const std::string& msg);

namespace {

constexpr double kUnivR = 8.31447215;  // ucs/chem_constants.h:5

// an edge's unit normal and area, one 32-byte load
struct __align__(32) EdgeArea {
  double x, y, z, w;
};
constexpr double kPref = 101325.0;     // ucs/reaction.tcc:665

// Per-species constants of the thermodynamic functions, formed once per
// handle so that no FP64 division is left in the per-node loops: the species
// gas constant R = R_univ / MW (Species::Init, ucs/species.tcc:315), and per
// curve the enthalpy polynomial's coefficients (a5, a0, a1/2, a2/3, a3/4,
// a4/5) and the cp polynomial's (a0..a4).
struct ChemDerived {
  double R[PCFD_CHEM_MAX_SPECIES];
  double h[2][PCFD_CHEM_MAX_SPECIES][6];
  double cp[2][PCFD_CHEM_MAX_SPECIES][5];
};

struct ChemHandle {
  pcfd_chem_model host;
  pcfd_chem_model* dev = nullptr;
  ChemDerived* dder = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double *d_rho = nullptr, *d_T = nullptr, *d_w = nullptr;
  long long cap = 0;
  double* d_buf = nullptr;  // host-array calls of the node-state functions
  size_t buf_cap = 0;
  long long* d_count = nullptr;
  // attached mesh (pcfd_chem_attach_mesh)
  long long nnode = 0, nedge = 0, nbedge = 0;
  int2 *d_en = nullptr, *d_bn = nullptr;
  EdgeArea *d_ea = nullptr, *d_ba = nullptr;
  double* d_vol = nullptr;
  int *d_nptr = nullptr, *d_nedg = nullptr, *d_bptr = nullptr, *d_bhe = nullptr;
  double *d_q = nullptr, *d_ef = nullptr, *d_bf = nullptr, *d_b = nullptr, *d_part = nullptr, *d_norms = nullptr;
  double* d_xyz = nullptr;   // node coordinates (the viscous flux's directional correction)
  double* d_sw = nullptr;    // LSQ normal matrices [nnode][6] (the gradient)
  int* d_btag = nullptr;     // half-edge face tags (the gradient's symmetry fix, the conditions)
  void* d_bctab = nullptr;   // per-tag condition tables of pcfd_chem_update_bcs
  double* d_lim = nullptr;   // host-array limiter of the second-order residual [nnode][ns + 4]
  size_t bc_cap = 0;
  double* d_grad = nullptr;  // host-array gradient of the viscous residual [nnode][2 ns + 4][3]
};

constexpr int kChemNormBlocks = 304;  // fixed grid of the residual gather: a fixed summation order

int cuda_fail(cudaError_t e, const char* what) {
  pcfd_set_last_error(std::string(what) + ": " + cudaGetErrorString(e));
  return e == cudaErrorMemoryAllocation ? PCFD_ERR_NOMEM : PCFD_ERR_CUDA;
}
#define CHEM_TRY(x, what)                   \
  do {                                      \
    cudaError_t e_ = (x);                   \
    if (e_ != cudaSuccess) return cuda_fail(e_, what); \
  } while (0)

__device__ __forceinline__ bool whole(double v) { return v == floor(v); }

// x^a: small whole exponents (the stoichiometric coefficients of the
// mechanisms, 0..3) by multiplication, which FP64 pow would spend ~20
// operations on; anything else through pow
__device__ __forceinline__ double stoich_pow(double x, double a) {
  if (a == 0.0) return 1.0;
  if (a == 1.0) return x;
  if (a == 2.0) return x * x;
  if (a == 3.0) return x * x * x;
  return pow(x, whole(a) ? (double)(int)a : a);
}

__device__ __forceinline__ const double* thermo_coeff(const pcfd_chem_model& m, int s, double T) {
  if (T < 200.0) return m.nasa_lo[s];
  if (T > 6000.0) return m.nasa_hi[s];
  return T > 1000.0 ? m.nasa_hi[s] : m.nasa_lo[s];
}

__device__ double forward_rate(const pcfd_chem_reaction& r, double T) {
  switch (r.type) {
    case 0: return r.A * exp(-r.EA / (kUnivR * T));
    case 1: return r.A * pow(T, r.n) * exp(-r.EA / (kUnivR * T));
    case 2: return r.A * pow(T, r.n) * exp(-r.EA / T);
    case 3: return r.A * pow(T, r.n);
  }
  return -999.0;
}

__device__ double equilibrium_const(const pcfd_chem_model& m, const pcfd_chem_reaction& r, double T, double logT) {
  double nu = 0.0, d0 = 0.0, d1 = 0.0, d2 = 0.0, d3 = 0.0, d4 = 0.0, d5 = 0.0, d6 = 0.0;
  for (int i = 0; i < r.nlocal; i++) {
    const double* a = thermo_coeff(m, r.global[i], T);
    const double dnu = r.nupp[i] - r.nup[i];
    nu += dnu;
    d0 += dnu * a[0];
    d1 += dnu * a[1];
    d2 += dnu * a[2];
    d3 += dnu * a[3];
    d4 += dnu * a[4];
    d5 += dnu * a[5];
    d6 += dnu * a[6];
  }
  double Kp = exp(d0 * (logT - 1.0) + T * (d1 / 2.0 + T * (d2 / 6.0 + T * (d3 / 12.0 + d4 / 20.0 * T))) - d5 / T + d6);
  double Kc = Kp;
  if (!(fabs(nu) < 1.0e-15)) Kc *= pow(kPref / (kUnivR * T), whole(nu) ? (double)(int)nu : nu);
  return Kc;
}

// mass production rates of one node from its molar concentrations X [ns]
// (rhoi / MW) -> wdot [ns], with the rate constants of reaction j given by
// consts(j, Kf, Kb)
template <class Consts>
__device__ __forceinline__ void rates_with(const pcfd_chem_model& m, const double* X, Consts&& consts,
                                          double* wdot) {
  const int ns = m.nspecies;
  double w[PCFD_CHEM_MAX_SPECIES];
  for (int k = 0; k < ns; k++) w[k] = 0.0;
  double Xsum = 0.0;
  for (int k = 0; k < ns; k++) Xsum += X[k];
  for (int j = 0; j < m.nreactions; j++) {
    const pcfd_chem_reaction& r = m.rx[j];
    double Kf, Kb;
    consts(j, Kf, Kb);
    double form = 1.0, dest = 1.0;
    for (int l = 0; l < r.nlocal; l++) {
      const double x = X[r.global[l]];
      const double a = r.nup[l], b = r.nupp[l];
      form *= stoich_pow(x, a);
      dest *= stoich_pow(x, b);
    }
    double Mc = 1.0;
    if (r.third_bodies) {
      Mc = Xsum;
      for (int l = 0; l < r.nlocal; l++) Mc += (r.tbeff[l] - 1.0) * X[r.global[l]];
    }
    const double net = Kf * form - Kb * dest;
    for (int l = 0; l < r.nlocal; l++) {
      const double nu = r.nupp[l] - r.nup[l];
      if (nu == 0.0) continue;
      const int g = r.global[l];
      double t = nu * Mc * net;
      t *= m.mw[g];
      w[g] += t;
    }
  }
  for (int k = 0; k < ns; k++) wdot[k] = w[k];
}

// forward (Arrhenius) and backward (forward / equilibrium constant) rate
// constants of reaction j at T
__device__ __forceinline__ void rate_consts(const pcfd_chem_model& m, int j, double T, double logT, double& Kf,
                                            double& Kb) {
  const pcfd_chem_reaction& r = m.rx[j];
  Kf = forward_rate(r, T);
  Kb = Kf / equilibrium_const(m, r, T, logT);
}

// mass production rates of one node (rhoi [ns] kg/m^3, T K -> wdot [ns])
__device__ void node_rates(const pcfd_chem_model& m, const double* rhoi, const double T, double* wdot) {
  double X[PCFD_CHEM_MAX_SPECIES];
  for (int k = 0; k < m.nspecies; k++) X[k] = rhoi[k] / m.mw[k];
  const double logT = log(T);
  rates_with(m, X, [&](int j, double& Kf, double& Kb) { rate_consts(m, j, T, logT, Kf, Kb); }, wdot);
}

__global__ void __launch_bounds__(128) k_chem_rates(long long n, const pcfd_chem_model* __restrict__ gm,
                                                    const double* __restrict__ rhoi, const double* __restrict__ Tn,
                                                    double* __restrict__ wdot) {
  __shared__ pcfd_chem_model m;
  {
    // stage the mechanism (about 17 KB) with 8-byte copies
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(gm);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(&m);
    for (int k = threadIdx.x; k < (int)(sizeof(pcfd_chem_model) / 8); k += blockDim.x) dst[k] = src[k];
  }
  __syncthreads();
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= n) return;
  node_rates(m, rhoi + p * m.nspecies, Tn[p], wdot + p * m.nspecies);
}

// EqnSet::SourceTermJacobian (ucs/eqnset.tcc:163) of the reacting set, one
// thread per node: A[j*neqn + i] = (S_j(Q + h e_i) - S_j(Q)) / h, h = 1e-8,
// S = SourceTerm (ucs/compressibleFR.tcc:1276) = vol * wdot / (ref_density /
// ref_time) in the species rows.  SourceTerm reads rhoi and T only, and the
// rate constants depend on T only: the ns species columns reuse the base
// point's constants (the same values the reference recomputes), and only
// the T column forms them again; likewise the concentrations rhoi / MW of
// the species a column does not perturb.  The velocity columns are
// (S - S) / h and the momentum and energy rows (0 - 0) / h in the
// reference: S - S and +0 here, the same values without the division.
__global__ void __launch_bounds__(128) k_chem_source_jac(long long n, const pcfd_chem_model* __restrict__ gm,
                                                         pcfd_chem_ref ref, double ref_time,
                                                         const double* __restrict__ q, const double* __restrict__ vol,
                                                         double* __restrict__ A) {
  __shared__ pcfd_chem_model m;
  {
    const unsigned long long* src = reinterpret_cast<const unsigned long long*>(gm);
    unsigned long long* dst = reinterpret_cast<unsigned long long*>(&m);
    for (int k = threadIdx.x; k < (int)(sizeof(pcfd_chem_model) / 8); k += blockDim.x) dst[k] = src[k];
  }
  __syncthreads();
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int ns = m.nspecies, neqn = ns + 4, nv = 6 + 3 * ns;
  const double h = 1.0e-8;
  const double* Q = q + p * nv;
  const double V = vol[p];
  const double scale = ref.density / ref_time;
  double* Ap = A + p * (long long)neqn * neqn;
  double X[PCFD_CHEM_MAX_SPECIES], w[PCFD_CHEM_MAX_SPECIES], S0[PCFD_CHEM_MAX_SPECIES];
  double Kf[PCFD_CHEM_MAX_REACTIONS], Kb[PCFD_CHEM_MAX_REACTIONS];
  for (int k = 0; k < ns; k++) X[k] = (Q[k] * ref.density) / m.mw[k];
  const double T0 = Q[ns + 3] * ref.temperature;
  {
    const double logT = log(T0);
    for (int j = 0; j < m.nreactions; j++) rate_consts(m, j, T0, logT, Kf[j], Kb[j]);
  }
  auto stored = [&](int j, double& kf, double& kb) {
    kf = Kf[j];
    kb = Kb[j];
  };
  rates_with(m, X, stored, w);
  for (int k = 0; k < ns; k++) S0[k] = V * (w[k] / scale);
  // a column of the difference quotients from the perturbed source in w
  auto column = [&](int i) {
    for (int j = 0; j < ns; j++) Ap[j * neqn + i] = (V * (w[j] / scale) - S0[j]) / h;
  };
  for (int i = 0; i < ns; i++) {
    const double keep = X[i];
    X[i] = ((Q[i] + h) * ref.density) / m.mw[i];
    rates_with(m, X, stored, w);
    X[i] = keep;
    column(i);
  }
  for (int i = ns; i < ns + 3; i++)
    for (int j = 0; j < ns; j++) Ap[j * neqn + i] = S0[j] - S0[j];
  {
    const double T = (Q[ns + 3] + h) * ref.temperature;
    const double logT = log(T);
    rates_with(m, X, [&](int j, double& kf, double& kb) { rate_consts(m, j, T, logT, kf, kb); }, w);
    column(ns + 3);
  }
  for (int j = ns; j < neqn; j++)
    for (int i = 0; i < neqn; i++) Ap[j * neqn + i] = 0.0;
}

// ---- node state of the reacting equation set ------------------------------

// the curve of Species::GetThermoCoeff (ucs/species.tcc:96): the high set
// above 1000 K (and above 6000 K, at the unpinned T), the low set otherwise
__device__ __forceinline__ int curve(double T) { return (T > 1000.0) ? 1 : 0; }

// Species<T>::GetCp and GetH (ucs/species.tcc:43,56; href = 0, :327), J/kg
__device__ __forceinline__ double species_cp(const ChemDerived& d, int s, double T) {
  const double* a = d.cp[curve(T)][s];
  const double cp_R = a[0] + T * (a[1] + T * (a[2] + T * (a[3] + T * a[4])));
  return cp_R * d.R[s];
}
__device__ __forceinline__ double species_h(const ChemDerived& d, int s, double T) {
  const double* c = d.h[curve(T)][s];
  const double h_R = c[0] + T * (c[1] + T * (c[2] + T * (c[3] + T * (c[4] + T * c[5]))));
  return h_R * d.R[s];
}
// ChemModel::GetP (ucs/chem.tcc:989): Dalton's law over IdealGasEOS::GetP
__device__ __forceinline__ double mix_P(const ChemDerived& d, int ns, const double* rhoiDim, double T) {
  double P = 0.0;
  for (int i = 0; i < ns; i++) P += rhoiDim[i] * d.R[i] * T;
  return P;
}
// ChemModel::GetSpecificEnthalpy (ucs/chem.tcc:586)
__device__ __forceinline__ double mix_h(const ChemDerived& d, int ns, const double* X, double T) {
  double h = 0.0;
  for (int i = 0; i < ns; i++) h += species_h(d, i, T) * X[i];
  return h;
}

// NewtonFindTGivenP: the pressure is linear in T, so the finite-difference
// Newton step lands in one or two iterations; counts nodes that used all 28
__global__ void __launch_bounds__(128) k_chem_find_T(long long n, const pcfd_chem_model* __restrict__ gm,
                                                     const ChemDerived* __restrict__ gd,
                                                     pcfd_chem_ref ref, const double* __restrict__ rhoi,
                                                     const double* __restrict__ P, const double* __restrict__ Tinit,
                                                     double* __restrict__ Tout, long long* __restrict__ nonconv) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= n) return;
  const pcfd_chem_model& m = *gm;
  const ChemDerived& d = *gd;
  const int ns = m.nspecies;
  double rhoiDim[PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < ns; i++) rhoiDim[i] = rhoi[p * ns + i] * ref.density;
  double TDim = Tinit[p] * ref.temperature;
  const double PgoalDim = P[p] * ref.pressure;
  int j;
  for (j = 0; j < 28; j++) {
    const double TpDim = TDim + 1.0e-8;
    const double zpoint = PgoalDim - mix_P(d, ns, rhoiDim, TDim);
    const double zpointp = PgoalDim - mix_P(d, ns, rhoiDim, TpDim);
    const double dzdT = (zpointp - zpoint) / (TpDim - TDim);
    const double dT = -zpoint / dzdT;
    if (fabs(dT / ref.temperature) < 1.0e-15) break;
    TDim += dT;
  }
  if (j == 28) atomicAdd((unsigned long long*)nonconv, 1ull);
  Tout[p] = TDim / ref.temperature;
}

// ConservativeToNative: the temperature Newton from total energy in FP64
// (finite-difference slope, |dT| < 1e-12, at most 20 iterations)
__global__ void __launch_bounds__(128) k_chem_c2n(long long n, const pcfd_chem_model* __restrict__ gm,
                                                     const ChemDerived* __restrict__ gd,
                                                  pcfd_chem_ref ref, const double* __restrict__ q,
                                                  const double* __restrict__ Pst, double* __restrict__ native,
                                                  long long* __restrict__ nonconv) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= n) return;
  const pcfd_chem_model& m = *gm;
  const ChemDerived& d = *gd;
  const int ns = m.nspecies;
  const double* qp = q + p * (ns + 4);
  double rho = 0.0, R = 0.0, Y[PCFD_CHEM_MAX_SPECIES], rhoiDim[PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < ns; i++) {
    rho += qp[i];
    rhoiDim[i] = qp[i] * ref.density;
    R += rhoiDim[i] * d.R[i];
  }
  R /= ref.density * rho;
  for (int i = 0; i < ns; i++) Y[i] = qp[i] / rho;
  const double u = qp[ns] / rho, v = qp[ns + 1] / rho, w = qp[ns + 2] / rho;
  const double v2 = u * u + v * v + w * w;
  const double res = qp[ns + 3] - 0.5 * v2 * rho;
  // IdealGasEOS::GetT (ucs/EOS.tcc:22) from the stored pressure
  double T = (Pst[p] * ref.pressure) / ((rho * ref.density) * R) / ref.temperature;
  int j;
  for (j = 0; j < 20; j++) {
    const double Tp = T + 1.0e-8;
    const double H = rho * (mix_h(d, ns, Y, T * ref.temperature) / ref.specific_enthalpy);
    const double Hp = rho * (mix_h(d, ns, Y, Tp * ref.temperature) / ref.specific_enthalpy);
    const double Pn = mix_P(d, ns, rhoiDim, T * ref.temperature) / ref.pressure;
    const double Pp = mix_P(d, ns, rhoiDim, Tp * ref.temperature) / ref.pressure;
    const double zpoint = res - (H - Pn), zpointp = res - (Hp - Pp);
    const double dzdT = (zpointp - zpoint) / (Tp - T);
    const double dT = -zpoint / dzdT;
    T += dT;
    if (fabs(dT) < 1.0e-12) break;
  }
  if (j == 20) atomicAdd((unsigned long long*)nonconv, 1ull);
  double* o = native + p * 4;
  o[0] = u;
  o[1] = v;
  o[2] = w;
  o[3] = T;
}

// NativeToConservative with GetTotalEnergy (ucs/compressibleFR.tcc:1219)
__global__ void __launch_bounds__(128) k_chem_n2c(long long n, const pcfd_chem_model* __restrict__ gm,
                                                     const ChemDerived* __restrict__ gd,
                                                  pcfd_chem_ref ref, const double* __restrict__ rhoi,
                                                  const double* __restrict__ native, const double* __restrict__ P,
                                                  double* __restrict__ q) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= n) return;
  const pcfd_chem_model& m = *gm;
  const ChemDerived& d = *gd;
  const int ns = m.nspecies;
  double rho = 0.0, X[PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < ns; i++) rho += rhoi[p * ns + i];
  for (int i = 0; i < ns; i++) X[i] = rhoi[p * ns + i] / rho;
  const double* nv = native + p * 4;
  const double u = nv[0], v = nv[1], w = nv[2], T = nv[3];
  const double v2 = u * u + v * v + w * w;
  const double h = mix_h(d, ns, X, T * ref.temperature) / ref.specific_enthalpy;
  const double E = h * rho - P[p];
  double* o = q + p * 4;
  o[0] = u * rho;
  o[1] = v * rho;
  o[2] = w * rho;
  o[3] = E + 0.5 * rho * v2;
}

// ComputeAuxiliaryVariables: pressure, species cv (Mayer's relation with the
// species R, IdealGasEOS::GetCv, ucs/EOS.tcc:79) and concentrations
__global__ void __launch_bounds__(128) k_chem_aux(long long n, const pcfd_chem_model* __restrict__ gm,
                                                     const ChemDerived* __restrict__ gd,
                                                  pcfd_chem_ref ref, const double* __restrict__ rhoi,
                                                  const double* __restrict__ T, double* __restrict__ Pout,
                                                  double* __restrict__ cvi, double* __restrict__ mol) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= n) return;
  const pcfd_chem_model& m = *gm;
  const ChemDerived& d = *gd;
  const int ns = m.nspecies;
  double rhoiDim[PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < ns; i++) rhoiDim[i] = rhoi[p * ns + i] * ref.density;
  const double TDim = T[p] * ref.temperature;
  Pout[p] = mix_P(d, ns, rhoiDim, TDim) / ref.pressure;
  const double s_ref = ref.velocity * ref.velocity / ref.temperature;
  for (int i = 0; i < ns; i++) {
    cvi[p * ns + i] = (species_cp(d, i, TDim) - d.R[i]) / s_ref;
    mol[p * ns + i] = rhoi[p * ns + i] / m.mw[i] / 1000.0;
  }
}

// ChemModel::GetFluidProperties (ucs/chem.tcc:545) through the equation
// set's wrapper (ucs/compressibleFR.tcc:1523): the non-dimensional speed of
// sound squared, gamma R T with the mixture's cp / cv
__device__ __forceinline__ double fr_c2(const ChemDerived& d, int ns, const pcfd_chem_ref& ref, const double* rhoi,
                                        double T) {
  double rhoiDim[PCFD_CHEM_MAX_SPECIES];
  const double Tdim = T * ref.temperature;
  double rho = 0.0, R = 0.0, cp = 0.0, cv = 0.0;
  for (int i = 0; i < ns; i++) rhoiDim[i] = rhoi[i] * ref.density;
  for (int i = 0; i < ns; i++) rho += rhoiDim[i];
  for (int i = 0; i < ns; i++) R += rhoiDim[i] * d.R[i];
  R /= rho;
  for (int i = 0; i < ns; i++) {
    const double X = rhoiDim[i] / rho;
    const double cpi = species_cp(d, i, Tdim);
    cp += cpi * X;
    cv += X * (cpi - d.R[i]);
  }
  const double gamma = cp / cv;
  return gamma * R * Tdim / (ref.velocity * ref.velocity);
}

// CompressibleFREqnSet::GetFluidProperties (ucs/compressibleFR.tcc:1523)
// over ChemModel::GetFluidProperties (ucs/chem.tcc:545): the mixture R and
// the frozen speed of sound squared, non-dimensional
__device__ __forceinline__ void fr_fluid_R_c2(const ChemDerived& d, int ns, const pcfd_chem_ref& ref,
                                              const double* rhoi, double T, double& R, double& c2) {
  double rhoiDim[PCFD_CHEM_MAX_SPECIES];
  const double s_ref = ref.velocity * ref.velocity / ref.temperature;
  const double Tdim = T * ref.temperature;
  double rho = 0.0, RDim = 0.0, cp = 0.0, cv = 0.0;
  for (int i = 0; i < ns; i++) rhoiDim[i] = rhoi[i] * ref.density;
  for (int i = 0; i < ns; i++) rho += rhoiDim[i];
  for (int i = 0; i < ns; i++) RDim += rhoiDim[i] * d.R[i];
  RDim /= rho;
  for (int i = 0; i < ns; i++) {
    const double X = rhoiDim[i] / rho;
    const double cpi = species_cp(d, i, Tdim);
    cp += cpi * X;
    cv += X * (cpi - d.R[i]);
  }
  const double gamma = cp / cv;
  R = RDim / s_ref;
  c2 = gamma * RDim * Tdim / (ref.velocity * ref.velocity);
}

// ---- transport ----------------------------------------------------------
// Species::GetViscosity / GetThermalConductivity (ucs/species.tcc:393,430):
// at or below 1000 K White's Sutherland forms with air's constants for every
// species, above it the last NASA RP-1311 fit whose range holds T,
// ln(y) = A ln T + B/T + C/T^2 + D, from micropoise and microwatt/(cm K).
// *bad is set when no fit holds T (the reference aborts).
__device__ double transport_fit(const double (*fit)[6], int nfit, double T, double conv, int& bad) {
  int range = -1;
  for (int i = 0; i < nfit; i++)
    if (T >= fit[i][0] && T <= fit[i][1]) range = i;
  if (range < 0) {
    bad = 1;
    return 0.0;
  }
  const double* c = fit[range];
  return exp(c[2] * log(T) + c[3] / T + c[4] / (T * T) + c[5]) * conv;
}

__device__ __forceinline__ double species_mu(const pcfd_chem_model& m, int s, double T, int& bad) {
  if (T <= 1000.0) return 1.716e-5 * pow(T / 273.0, 1.5) * ((273.0 + 111.0) / (T + 111.0));
  return transport_fit(m.mu_fit[s], m.nmu[s], T, 1.0e-7, bad);
}

__device__ __forceinline__ double species_k(const pcfd_chem_model& m, int s, double T, int& bad) {
  if (T <= 1000.0) return 0.0241 * pow(T / 273.0, 1.5) * ((273.0 + 194.0) / (T + 194.0));
  return transport_fit(m.k_fit[s], m.nk[s], T, 1.0e-4, bad);
}

// ChemModel::WilkesMixtureRule (ucs/chem.tcc:876) for the viscosity and the
// conductivity together: mole fractions from mass fractions (the last one
// 1 - the sum of the others, MassFractionToMoleFraction, :941), weights from
// the species' viscosities for both properties, as the reference forms them.
__device__ void wilke_mu_k(const pcfd_chem_model& m, const double* rhoiDim, double TDim, double& mu, double& k,
                           int& bad) {
  const int ns = m.nspecies;
  double X[PCFD_CHEM_MAX_SPECIES], vi[PCFD_CHEM_MAX_SPECIES], ki[PCFD_CHEM_MAX_SPECIES];
  double rho = 0.0;
  for (int i = 0; i < ns; i++) rho += rhoiDim[i];
  double summ = 0.0;
  for (int i = 0; i < ns; i++) {
    X[i] = (rhoiDim[i] / rho) / m.mw[i];
    summ += X[i];
  }
  for (int i = 0; i < ns; i++) X[i] /= summ;
  summ = 0.0;
  for (int i = 0; i < ns - 1; i++) summ += X[i];
  X[ns - 1] = 1.0 - summ;
  for (int i = 0; i < ns; i++) {
    vi[i] = species_mu(m, i, TDim, bad);
    ki[i] = species_k(m, i, TDim, bad);
  }
  const double sqrt8 = sqrt(8.0);
  mu = 0.0;
  k = 0.0;
  for (int i = 0; i < ns; i++) {
    double wi = 0.0;
    for (int j = 0; j < ns; j++) {
      const double temp = 1.0 + sqrt(vi[i] / vi[j]) * pow(m.mw[j] / m.mw[i], 0.25);
      const double phi = pow(1.0 + m.mw[i] / m.mw[j], -0.5) * temp * temp / sqrt8;
      wi += X[j] * phi;
    }
    mu += (X[i] / wi) * vi[i];
    k += (X[i] / wi) * ki[i];
  }
}

// GetMolecularViscosity / GetThermalConductivity of the reacting set
// (ucs/compressibleFR.tcc:1580,1590), non-dimensional in and out
__device__ __forceinline__ void fr_transport(const pcfd_chem_model& m, const pcfd_chem_ref& ref, const double* rhoi,
                                             double T, double& mu, double& k, int& bad) {
  double rd[PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < m.nspecies; i++) rd[i] = rhoi[i] * ref.density;
  wilke_mu_k(m, rd, T * ref.temperature, mu, k, bad);
  mu /= (ref.viscosity != 0.0 ? ref.viscosity : 1.0);
  k /= (ref.conductivity != 0.0 ? ref.conductivity : 1.0);
}

__global__ void __launch_bounds__(128) k_chem_transport(long long n, const pcfd_chem_model* __restrict__ gm,
                                                        pcfd_chem_ref ref, const double* __restrict__ rhoi,
                                                        const double* __restrict__ T, double* __restrict__ mu,
                                                        double* __restrict__ k, long long* bad_count) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= n) return;
  const pcfd_chem_model& m = *gm;
  int bad = 0;
  double a, b;
  fr_transport(m, ref, &rhoi[p * m.nspecies], T[p], a, b, bad);
  mu[p] = bad ? 0.0 : a;
  k[p] = bad ? 0.0 : b;
  if (bad) atomicAdd((unsigned long long*)bad_count, 1ull);
}

// CompressibleFREqnSet::ContributeTemporalTerms (ucs/compressibleFR.tcc:1319),
// one thread per node: Aout = Ain + vol/dt terms times dq/dQ (conservative
// over native), with ChemModel::dEtdP_dEtdRhoi (ucs/chem.tcc:829, at
// constant T) and Gupta's beta preconditioning on the temperature column.
// The species speeds of sound are the mixture's, as the reference sets them.
__global__ void __launch_bounds__(128) k_chem_temporal(long long n, const pcfd_chem_model* __restrict__ gm,
                                                       const ChemDerived* __restrict__ gd, pcfd_chem_ref ref,
                                                       const double* __restrict__ q, const double* __restrict__ vol,
                                                       const double* __restrict__ dtau,
                                                       const double* __restrict__ betav, double cnp1, double dt,
                                                       int local_ts, const double* Ain, double* Aout) {
  const long long p = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (p >= n) return;
  const ChemDerived& d = *gd;
  const int ns = gm->nspecies, neqn = ns + 4, nv = 6 + 3 * ns;
  const int uloc = ns, vloc = ns + 1, wloc = ns + 2, tloc = ns + 3;
  const double* Q = q + p * nv;
  const double* Ai = Ain + p * (long long)neqn * neqn;
  double* Ao = Aout + p * (long long)neqn * neqn;
  if (Ao != Ai)
    for (int k = 0; k < neqn * neqn; k++) Ao[k] = Ai[k];
  const double V = vol[p], beta = betav[p];
  const double vOverDt = local_ts ? cnp1 * V / dt + V / dtau[p] : cnp1 * V / dtau[p];
  const double rho = Q[ns + 5], T = Q[tloc];
  const double u = Q[uloc], v = Q[vloc], w = Q[wloc];
  const double rvOverDt = rho * vOverDt;
  double v2 = u * u + v * v + w * w;
  double R, c2;
  fr_fluid_R_c2(d, ns, ref, Q, T, R, c2);
  const double s_ref = ref.velocity * ref.velocity / ref.temperature;
  const double rhoDim = rho * ref.density;
  const double TDim = T * ref.temperature;
  v2 *= ref.velocity * ref.velocity;
  double rhoiDim[PCFD_CHEM_MAX_SPECIES], dEtdRhoi[PCFD_CHEM_MAX_SPECIES], theta[PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < ns; i++) rhoiDim[i] = Q[i] * ref.density;
  // dEtdP_dEtdRhoi with dRmixdRhoi (ucs/chem.tcc:862), dimensional
  double dEtdP;
  {
    const double hv2 = 0.5 * v2;
    double rhomix = 0.0, Rmix = 0.0;
    for (int i = 0; i < ns; i++) {
      rhomix += rhoiDim[i];
      Rmix += rhoiDim[i] * d.R[i];
    }
    Rmix /= rhomix;
    const double dPdrhomix = Rmix * TDim, dPdRmix = rhomix * TDim;
    for (int i = 0; i < ns; i++) {
      double dR = d.R[i] * (rhomix - rhoiDim[i]) / (rhomix * rhomix);
      for (int j = 0; j < ns; j++) {
        if (j == i) continue;
        dR -= d.R[j] * rhoiDim[j] / (rhomix * rhomix);
      }
      dEtdRhoi[i] = hv2 + species_h(d, i, TDim) - (dPdrhomix + dPdRmix * dR);
    }
    const double dTdP = 1.0 / (rhomix * Rmix);
    dEtdP = 0.0;
    for (int i = 0; i < ns; i++) dEtdP += rhoiDim[i] * species_cp(d, i, TDim) * dTdP;
    dEtdP -= 1.0;
  }
  const double ref_detdrho = ref.specific_enthalpy * ref.density / ref.density;
  for (int i = 0; i < ns; i++) dEtdRhoi[i] /= ref_detdrho;
  const double ref_detdP = ref.specific_enthalpy * ref.density / ref.pressure;
  dEtdP /= ref_detdP;
  double dPdT = rhoDim * (R * s_ref);
  dPdT /= (ref.pressure / ref.temperature);
  const double oneOBeta = 1.0 / beta, oneMbeta = 1.0 - beta;
  for (int i = 0; i < ns; i++) theta[i] = (Q[i] / rho * oneMbeta / c2) * oneOBeta;
  for (int i = 0; i < ns; i++) {
    Ao[neqn * i + i] += vOverDt;
    Ao[neqn * i + tloc] += theta[i] * vOverDt * dPdT;
  }
  const double vel[3] = {u, v, w};
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const int r = uloc + k;
    double precond = 0.0;
    for (int j = 0; j < ns; j++) {
      Ao[neqn * r + j] += vel[k] * vOverDt;
      precond += theta[j] * vel[k];
    }
    Ao[neqn * r + r] += rvOverDt;
    Ao[neqn * r + tloc] += precond * vOverDt * dPdT;
  }
  double precond = 0.0;
  for (int j = 0; j < ns; j++) {
    Ao[neqn * tloc + j] += dEtdRhoi[j] * vOverDt;
    precond += dEtdRhoi[j] * theta[j];
  }
  Ao[neqn * tloc + uloc] += u * rvOverDt;
  Ao[neqn * tloc + vloc] += v * rvOverDt;
  Ao[neqn * tloc + wloc] += w * rvOverDt;
  precond += dEtdP * oneOBeta;
  Ao[neqn * tloc + tloc] += precond * vOverDt * dPdT;
}

// GetTotalEnthalpy (ucs/compressibleFR.tcc:1249) of a node record
__device__ __forceinline__ double fr_Ht(const ChemDerived& d, int ns, const pcfd_chem_ref& ref, const double* Q) {
  double X[PCFD_CHEM_MAX_SPECIES];
  const double T = Q[ns + 3], rho = Q[ns + 5], u = Q[ns], v = Q[ns + 1], w = Q[ns + 2];
  const double v2 = u * u + v * v + w * w;
  for (int i = 0; i < ns; i++) X[i] = Q[i] / rho;
  const double h = mix_h(d, ns, X, T * ref.temperature) / ref.specific_enthalpy;
  return h * rho + 0.5 * rho * v2;
}

// HLLC flux of one edge on a static grid (vdotn = 0), in FP64; the wave
// speeds are the Roe-averaged and one-sided eigenvalues with Gupta's beta
// modification.  Writes zeros and returns 1 when no branch applies.
__device__ int fr_hllc(const ChemDerived& d, int ns, const pcfd_chem_ref& ref, const pcfd_chem_flux_opts& o,
                       const double* QL, const double* QR, const EdgeArea a, double* flux) {
  const double beta = o.beta, Pref = o.pref;
  const double uL = QL[ns], vL = QL[ns + 1], wL = QL[ns + 2], TL = QL[ns + 3], pL = QL[ns + 4], rhoL = QL[ns + 5];
  const double uR = QR[ns], vR = QR[ns + 1], wR = QR[ns + 2], TR = QR[ns + 3], pR = QR[ns + 4], rhoR = QR[ns + 5];
  const double pgL = pL - Pref, pgR = pR - Pref;
  const double c2L = fr_c2(d, ns, ref, QL, TL), c2R = fr_c2(d, ns, ref, QR, TR);
  const double ETL = fr_Ht(d, ns, ref, QL) - pL, ETR = fr_Ht(d, ns, ref, QR) - pR;
  const double thetaL = uL * a.x + vL * a.y + wL * a.z;
  const double thetaR = uR * a.x + vR * a.y + wR * a.z;
  const double rho = sqrt(rhoL * rhoR);
  const double sigma = rho / (rhoL + rho);
  double roe[PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < ns; i++) roe[i] = QL[i] + sigma * (QR[i] - QL[i]);
  const double u = uL + sigma * (uR - uL), v = vL + sigma * (vR - vL), w = wL + sigma * (wR - wL);
  const double T = TL + sigma * (TR - TL);
  const double theta = u * a.x + v * a.y + w * a.z;
  const double c2 = fr_c2(d, ns, ref, roe, T);
  const double oneMBeta = 1.0 - beta;
  const double thetaPrime = theta * (1.0 + beta) * 0.5;
  const double cPrime = 0.5 * sqrt(theta * theta * (oneMBeta * oneMBeta) + 4.0 * beta * c2);
  const double thetaLPrime = thetaL * (1.0 + beta) * 0.5, thetaRPrime = thetaR * (1.0 + beta) * 0.5;
  const double cLPrime = 0.5 * sqrt(thetaL * thetaL * (oneMBeta * oneMBeta) + 4.0 * beta * c2L);
  const double cRPrime = 0.5 * sqrt(thetaR * thetaR * (oneMBeta * oneMBeta) + 4.0 * beta * c2R);
  const double eig5L = thetaLPrime - cLPrime, eig4R = thetaRPrime + cRPrime;
  const double eig4 = thetaPrime + cPrime, eig5 = thetaPrime - cPrime;
  const double SL = (eig5L < eig5) ? eig5L : eig5;
  const double SR = (eig4R > eig4) ? eig4R : eig4;
  double SM = (pgR - pgL + rhoL * thetaL * (SL - thetaL) - rhoR * thetaR * (SR - thetaR)) /
              (rhoL * (SL - thetaL) - rhoR * (SR - thetaR));
  // the state of the chosen HLLC region: species densities scaled by sf of
  // side s, momentum and energy as below
  const double* Qs;
  double sf, m0, m1, m2, Et, pStar;
  if (SL >= 0.0) {
    Qs = QL; sf = 1.0;
    m0 = rhoL * uL; m1 = rhoL * vL; m2 = rhoL * wL; Et = ETL;
    pStar = pgL;
    SM = thetaL;
  } else if (SR <= 0.0) {
    Qs = QR; sf = 1.0;
    m0 = rhoR * uR; m1 = rhoR * vR; m2 = rhoR * wR; Et = ETR;
    pStar = pgR;
    SM = thetaR;
  } else if (SL <= 0.0 && SM >= 0.0) {
    pStar = pgL + rhoL * (thetaL - SL) * (thetaL - SM);
    const double omega = 1.0 / (SL - SM), const1 = SL - thetaL, const2 = pStar - pgL;
    Qs = QL; sf = omega * const1;
    m0 = omega * (const1 * rhoL * uL + const2 * a.x);
    m1 = omega * (const1 * rhoL * vL + const2 * a.y);
    m2 = omega * (const1 * rhoL * wL + const2 * a.z);
    Et = omega * (const1 * ETL - pgL * thetaL + (pStar * SM)) + Pref * (SM - thetaL) * omega;
  } else if (SM <= 0.0 && SR >= 0.0) {
    pStar = pgR + rhoR * (thetaR - SR) * (thetaR - SM);
    const double omega = 1.0 / (SR - SM), const1 = SR - thetaR, const2 = pStar - pgR;
    Qs = QR; sf = omega * const1;
    m0 = omega * (const1 * rhoR * uR + const2 * a.x);
    m1 = omega * (const1 * rhoR * vR + const2 * a.y);
    m2 = omega * (const1 * rhoR * wR + const2 * a.z);
    Et = omega * (const1 * ETR - pgR * thetaR + (pStar * SM)) + Pref * (SM - thetaR) * omega;
  } else {
    for (int i = 0; i < ns + 4; i++) flux[i] = 0.0;
    return 1;
  }
  const double area = a.w;
  for (int i = 0; i < ns; i++) flux[i] = area * (sf * Qs[i]) * SM;
  flux[ns] = area * (m0 * SM + pStar * a.x);
  flux[ns + 1] = area * (m1 * SM + pStar * a.y);
  flux[ns + 2] = area * (m2 * SM + pStar * a.z);
  flux[ns + 3] = area * (Et * SM + pStar * SM) + Pref * SM * area;
  if (o.symmetry2D >= 1 && o.symmetry2D <= 3) flux[ns + o.symmetry2D - 1] = 0.0;
  return 0;
}

// one thread per edge; the two node records are read as consecutive
// doubles (6 + 3 ns per node)
__global__ void __launch_bounds__(128) k_chem_hllc(long long nedge, long long nnode,
                                                   const pcfd_chem_model* __restrict__ gm,
                                                   const ChemDerived* __restrict__ gd, pcfd_chem_ref ref,
                                                   pcfd_chem_flux_opts o, const double* __restrict__ q,
                                                   const int2* __restrict__ edges, const EdgeArea* __restrict__ avec,
                                                   double* __restrict__ flux, long long* __restrict__ nfail) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= nedge) return;
  const int ns = gm->nspecies;
  const int nv = 6 + 3 * ns;
  const int2 n = edges[e];
  if (n.x < 0 || n.y < 0 || n.x >= nnode || n.y >= nnode) {
    // an edge naming a node outside the record array: no access, counted
    for (int i = 0; i < ns + 4; i++) flux[e * (ns + 4) + i] = 0.0;
    atomicAdd((unsigned long long*)nfail, 1ull);
    return;
  }
  double QL[6 + 2 * PCFD_CHEM_MAX_SPECIES], QR[6 + 2 * PCFD_CHEM_MAX_SPECIES];
  // the flux reads the record up to rho (ns + 6 values)
  for (int i = 0; i < ns + 6; i++) {
    QL[i] = q[(size_t)n.x * nv + i];
    QR[i] = q[(size_t)n.y * nv + i];
  }
  double f[PCFD_CHEM_MAX_SPECIES + 4];
  if (fr_hllc(*gd, ns, ref, o, QL, QR, avec[e], f)) atomicAdd((unsigned long long*)nfail, 1ull);
  for (int i = 0; i < ns + 4; i++) flux[e * (ns + 4) + i] = f[i];
}

// Kernel_Inviscid_Flux (ucs/residual.tcc:192) at second order: both records
// extrapolated to the edge midpoint (ExtrapolateVariables,
// ucs/compressibleFR.tcc:734: q + lim (chi/2 dQ + (1 - chi) grad.dx) on
// rhoi, u, v, w, T, dx = (x_R - x_L)/2), their pressure and density
// recomputed (the part of ComputeAuxiliaryVariables the flux reads), then
// the HLLC flux
__global__ void __launch_bounds__(128) k_chem_hllc2(long long nedge, const pcfd_chem_model* __restrict__ gm,
                                                    const ChemDerived* __restrict__ gd, pcfd_chem_ref ref,
                                                    pcfd_chem_flux_opts o, double chi, const double* __restrict__ q,
                                                    const double* __restrict__ grad, const double* __restrict__ lim,
                                                    const double* __restrict__ xyz, const int2* __restrict__ edges,
                                                    const EdgeArea* __restrict__ avec, double* __restrict__ flux,
                                                    long long* __restrict__ nfail) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= nedge) return;
  const int ns = gm->nspecies, neqn = ns + 4, nv = 6 + 3 * ns, nt = 2 * ns + 4;
  const int2 n = edges[e];
  const double* qa = &q[(size_t)n.x * nv];
  const double* qc = &q[(size_t)n.y * nv];
  double dx[3];
  for (int i = 0; i < 3; i++) dx[i] = 0.5 * (xyz[3 * (size_t)n.y + i] - xyz[3 * (size_t)n.x + i]);
  const double* gL = &grad[(size_t)n.x * nt * 3];
  const double* gR = &grad[(size_t)n.y * nt * 3];
  double QL[6 + 2 * PCFD_CHEM_MAX_SPECIES], QR[6 + 2 * PCFD_CHEM_MAX_SPECIES];
  for (int j = 0; j < neqn; j++) {
    const double dQ = qc[j] - qa[j];
    const double cl = 0.5 * chi * dQ + (1.0 - chi) * (gL[3 * j] * dx[0] + gL[3 * j + 1] * dx[1] + gL[3 * j + 2] * dx[2]);
    const double cr = 0.5 * chi * (-dQ) +
                      (1.0 - chi) * (gR[3 * j] * (-dx[0]) + gR[3 * j + 1] * (-dx[1]) + gR[3 * j + 2] * (-dx[2]));
    QL[j] = qa[j] + cl * lim[(size_t)n.x * neqn + j];
    QR[j] = qc[j] + cr * lim[(size_t)n.y * neqn + j];
  }
  for (int k = 0; k < 2; k++) {
    double* Q = k ? QR : QL;
    double rhoiDim[PCFD_CHEM_MAX_SPECIES], rho = 0.0;
    for (int i = 0; i < ns; i++) {
      rho += Q[i];
      rhoiDim[i] = Q[i] * ref.density;
    }
    Q[ns + 4] = mix_P(*gd, ns, rhoiDim, Q[ns + 3] * ref.temperature) / ref.pressure;
    Q[ns + 5] = rho;
  }
  double f[PCFD_CHEM_MAX_SPECIES + 4];
  if (fr_hllc(*gd, ns, ref, o, QL, QR, avec[e], f)) atomicAdd((unsigned long long*)nfail, 1ull);
  for (int i = 0; i < neqn; i++) flux[e * neqn + i] = f[i];
}

// boundary half-edges: the node's record against its phantom record
__global__ void __launch_bounds__(128) k_chem_bflux(long long nbedge, const pcfd_chem_model* __restrict__ gm,
                                                    const ChemDerived* __restrict__ gd, pcfd_chem_ref ref,
                                                    pcfd_chem_flux_opts o, const double* __restrict__ q,
                                                    const int2* __restrict__ bn, const EdgeArea* __restrict__ ba,
                                                    double* __restrict__ bf, long long* __restrict__ nfail) {
  const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k >= nbedge) return;
  const int ns = gm->nspecies;
  const int nv = 6 + 3 * ns;
  const int2 n = bn[k];
  double QL[6 + 2 * PCFD_CHEM_MAX_SPECIES], QR[6 + 2 * PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < ns + 6; i++) {
    QL[i] = q[(size_t)n.x * nv + i];
    QR[i] = q[(size_t)n.y * nv + i];
  }
  double f[PCFD_CHEM_MAX_SPECIES + 4];
  if (fr_hllc(*gd, ns, ref, o, QL, QR, ba[k], f)) atomicAdd((unsigned long long*)nfail, 1ull);
  for (int i = 0; i < ns + 4; i++) bf[k * (ns + 4) + i] = f[i];
}

// per node: -sum of the fluxes out of it (incident edges in ascending id,
// signed: ~e where the node is the edge's left end), then its boundary
// half-edges, then vol * wdot; per-block partial sums of squares
// Gradient<T>::Compute of the reacting set, one node per thread: the
// weighted least-squares gradient (Kernel_LSQ_Gradient, ucs/gradient.tcc:251,
// with ComputeLSQCoefficients, :141) of the gradient list of
// GetGradientsLocation (ucs/compressibleFR.tcc:693: rhoi, u, v, w, T,
// concentrations) over the node's edges in ascending edge order, each edge's
// term formed as the edge-ordered sum forms it; then Bkernel_Symmetry_Fix
// (:545) on the node's half-edges whose tag is in sym (nsym entries).
constexpr int kChemMaxSym = 8;
struct ChemSym {
  int n;
  int tag[kChemMaxSym];
};

__global__ void __launch_bounds__(128) k_chem_gradient(long long nnode, const pcfd_chem_model* __restrict__ gm,
                                                       const double* __restrict__ q, const int2* __restrict__ en,
                                                       const int* __restrict__ nptr, const int* __restrict__ nedg,
                                                       const double* __restrict__ xyz, const double* __restrict__ sw,
                                                       const int* __restrict__ bptr, const int* __restrict__ bhe,
                                                       const int* __restrict__ btag, const EdgeArea* __restrict__ ba,
                                                       ChemSym sym, double* __restrict__ grad) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= nnode) return;
  const pcfd_chem_model& m = *gm;
  const int ns = m.nspecies, nv = 6 + 3 * ns, nt = 2 * ns + 4;
  double g[3 * (2 * PCFD_CHEM_MAX_SPECIES + 4)];
  for (int t = 0; t < 3 * nt; t++) g[t] = 0.0;
  const double* s = &sw[6 * i];
  const double s11 = s[0], s12 = s[1], s13 = s[2], s22 = s[3], s23 = s[4], s33 = s[5];
  const double r11 = s11, r12 = s12, r13 = s13;
  const double r12_r11 = (r11 == 0.0) ? 0.0 : r12 / r11;
  const double r22 = s22 - r12 * r12_r11;
  const double r23 = s23 - r12_r11 * r13;
  const double r13_r11 = (r11 == 0.0) ? 0.0 : r13 / r11;
  const double r23_r22 = (r22 == 0.0) ? 0.0 : r23 / r22;
  const double r33 = s33 - r13 * r13_r11 - r23 * r23_r22;
  for (int k = nptr[i]; k < nptr[i + 1]; k++) {
    const int se = nedg[k];
    const bool left = se < 0;
    const int2 n = en[left ? ~se : se];
    const double* xL = &xyz[3 * (size_t)n.x];
    const double* xR = &xyz[3 * (size_t)n.y];
    double d0 = xL[0] - xR[0], d1 = xL[1] - xR[1], d2 = xL[2] - xR[2];
    const double weight = 1.0 / sqrt(d0 * d0 + d1 * d1 + d2 * d2);
    d0 *= weight;
    d1 *= weight;
    d2 *= weight;
    if (!left) {
      d0 = -d0;
      d1 = -d1;
      d2 = -d2;
    }
    const double dykdx = (d1 - r12_r11 * d0);
    const double we2 = (r33 == 0.0) ? 0.0 : (d2 - r13_r11 * d0 - r23_r22 * dykdx) / r33;
    const double we1 = (r22 == 0.0) ? 0.0 : (dykdx - r23 * we2) / r22;
    const double we0 = (r11 == 0.0) ? 0.0 : (d0 - r12 * we1 - r13 * we2) / r11;
    const double* qL = &q[(size_t)n.x * nv];
    const double* qR = &q[(size_t)n.y * nv];
    for (int t = 0; t < nt; t++) {
      const int loc = t < ns + 4 ? t : 2 * ns + 6 + (t - ns - 4);
      const double dq = weight * (qR[loc] - qL[loc]);
      if (left) {
        g[3 * t + 0] += -we0 * dq;
        g[3 * t + 1] += -we1 * dq;
        g[3 * t + 2] += -we2 * dq;
      } else {
        g[3 * t + 0] += +we0 * dq;
        g[3 * t + 1] += +we1 * dq;
        g[3 * t + 2] += +we2 * dq;
      }
    }
  }
  for (int p = bptr[i]; p < bptr[i + 1]; p++) {
    const int he = bhe[p];
    bool on = false;
    for (int u = 0; u < sym.n; u++) on |= btag[he] == sym.tag[u];
    if (!on) continue;
    const EdgeArea a = ba[he];
    for (int t = 0; t < nt; t++) {
      const double dot = g[3 * t] * a.x + g[3 * t + 1] * a.y + g[3 * t + 2] * a.z;
      g[3 * t + 0] -= dot * a.x;
      g[3 * t + 1] -= dot * a.y;
      g[3 * t + 2] -= dot * a.z;
    }
  }
  for (int t = 0; t < 3 * nt; t++) grad[(size_t)i * nt * 3 + t] = g[t];
}

// ComputeAuxiliaryVariables (ucs/compressibleFR.tcc:755) of one record in
// place: P, rho, cvi, concentrations from rhoi and T (as k_chem_aux forms them)
__device__ void record_aux(const pcfd_chem_model& m, const ChemDerived& d, const pcfd_chem_ref& ref, double* Q) {
  const int ns = m.nspecies;
  double rhoiDim[PCFD_CHEM_MAX_SPECIES], rho = 0.0;
  for (int i = 0; i < ns; i++) {
    rho += Q[i];
    rhoiDim[i] = Q[i] * ref.density;
  }
  const double TDim = Q[ns + 3] * ref.temperature;
  Q[ns + 4] = mix_P(d, ns, rhoiDim, TDim) / ref.pressure;
  Q[ns + 5] = rho;
  const double s_ref = ref.velocity * ref.velocity / ref.temperature;
  for (int i = 0; i < ns; i++) {
    Q[ns + 6 + i] = (species_cp(d, i, TDim) - d.R[i]) / s_ref;
    Q[2 * ns + 6 + i] = Q[i] / m.mw[i] / 1000.0;
  }
}

// UpdateBCs (ucs/bc.tcc:1400) of the reacting set, one boundary node per
// thread: the node's half-edges in ascending order, each through
// CalculateBoundaryVariables (:1059) and then ComputeAuxiliaryVariables of
// its phantom and of the node.  A half-edge changes only its node and its
// own phantom, so per node this is the reference's sequential order.
// Types: sonic inflow / Dirichlet (the tag's reference record), sonic
// outflow / Neumann (copy), isothermal no-slip with a resting wall
// (GetViscousWallBoundaryVariables, ucs/compressibleFR.tcc:2049), and with
// no_cvbc the impermeable wall / symmetry (mirror, :1042); any other type
// is counted in *bad and leaves the records as they are.
struct ChemBc {
  int ntags, no_cvbc;
  const int* type;
  const double* twall;
  const double* qref;
};

__global__ void __launch_bounds__(128) k_chem_bcs(long long nnode, const pcfd_chem_model* __restrict__ gm,
                                                  const ChemDerived* __restrict__ gd, pcfd_chem_ref ref, ChemBc bc,
                                                  const int2* __restrict__ bn, const EdgeArea* __restrict__ ba,
                                                  const int* __restrict__ btag, const int* __restrict__ bptr,
                                                  const int* __restrict__ bhe, double* __restrict__ q,
                                                  long long* bad_count) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= nnode || bptr[i] == bptr[i + 1]) return;
  const pcfd_chem_model& m = *gm;
  const ChemDerived& d = *gd;
  const int ns = m.nspecies, neqn = ns + 4, nv = 6 + 3 * ns;
  double* QL = &q[(size_t)i * nv];
  for (int p = bptr[i]; p < bptr[i + 1]; p++) {
    const int k = bhe[p];
    const int tag = btag[k];
    const int bt = (tag >= 0 && tag < bc.ntags) ? bc.type[tag] : -1;
    double* QR = &q[(size_t)bn[k].y * nv];
    if (bt == PCFD_BC_SONIC_INFLOW || bt == PCFD_BC_DIRICHLET) {
      for (int j = 0; j < nv; j++) QR[j] = QL[j] = bc.qref[(size_t)tag * nv + j];
    } else if (bt == PCFD_BC_SONIC_OUTFLOW || bt == PCFD_BC_NEUMANN) {
      for (int j = 0; j < neqn; j++) QR[j] = QL[j];
    } else if (bt == PCFD_BC_NOSLIP && bc.twall[tag] > 0.0) {
      for (int j = 0; j < ns; j++) QR[j] = QL[j];
      QR[ns + 3] = QL[ns + 3] = bc.twall[tag] / ref.temperature;
      QR[ns] = QL[ns] = 0.0;
      QR[ns + 1] = QL[ns + 1] = 0.0;
      QR[ns + 2] = QL[ns + 2] = 0.0;
    } else if ((bt == PCFD_BC_IMPERMEABLE_WALL || bt == PCFD_BC_SYMMETRY) && bc.no_cvbc) {
      double Qm[6 + 3 * PCFD_CHEM_MAX_SPECIES];
      for (int j = 0; j < nv; j++) Qm[j] = QL[j];
      record_aux(m, d, ref, Qm);
      for (int j = 0; j < neqn; j++) QR[j] = Qm[j];
      const EdgeArea a = ba[k];
      const double dot = 2.0 * (Qm[ns] * a.x + Qm[ns + 1] * a.y + Qm[ns + 2] * a.z);
      QR[ns] = Qm[ns] - dot * a.x;
      QR[ns + 1] = Qm[ns + 1] - dot * a.y;
      QR[ns + 2] = Qm[ns + 2] - dot * a.z;
    } else {
      atomicAdd((unsigned long long*)bad_count, 1ull);
      continue;
    }
    record_aux(m, d, ref, QR);
    record_aux(m, d, ref, QL);
  }
}

// Limiter<T>::Compute with Kernel_VenkatMod (ucs/limiters.tcc:53,534; K = 1
// as hard-coded there) on the reacting set's native variables, one node per
// thread: neighbour bounds from 0 (Kernel_FindMinMax, :135), each incident
// edge's unlimited extrapolation (ExtrapolateVariables,
// ucs/compressibleFR.tcc:734, dx = (x_j - x_i)/2), the running minimum,
// negatives clamped to 0.  The pressure clip is not applied.
__global__ void __launch_bounds__(128) k_chem_limiter(long long nnode, const pcfd_chem_model* __restrict__ gm,
                                                      double chi, const double* __restrict__ q,
                                                      const double* __restrict__ grad, const double* __restrict__ xyz,
                                                      const double* __restrict__ vol, const int2* __restrict__ en,
                                                      const int* __restrict__ nptr, const int* __restrict__ nedg,
                                                      double* __restrict__ lim) {
  const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (i >= nnode) return;
  const int ns = gm->nspecies, neqn = ns + 4, nv = 6 + 3 * ns, nt = 2 * ns + 4;
  const double* qi = &q[(size_t)i * nv];
  double mn[PCFD_CHEM_MAX_SPECIES + 4], mx[PCFD_CHEM_MAX_SPECIES + 4], l[PCFD_CHEM_MAX_SPECIES + 4];
  for (int j = 0; j < neqn; j++) {
    mn[j] = mx[j] = 0.0;
    l[j] = 1.0;
  }
  auto nbr = [&](int k) {
    const int se = nedg[k];
    const int2 n = en[se < 0 ? ~se : se];
    return se < 0 ? n.y : n.x;
  };
  for (int k = nptr[i]; k < nptr[i + 1]; k++) {
    const double* qj = &q[(size_t)nbr(k) * nv];
    for (int j = 0; j < neqn; j++) {
      mx[j] = mx[j] > qj[j] ? mx[j] : qj[j];
      mn[j] = mn[j] < qj[j] ? mn[j] : qj[j];
    }
  }
  const double ep2 = (6.0 * 3.141592653589793 * vol[i]) * 1.0;
  const double* g = &grad[(size_t)i * nt * 3];
  for (int k = nptr[i]; k < nptr[i + 1]; k++) {
    const int j0 = nbr(k);
    const double* qj = &q[(size_t)j0 * nv];
    double dx[3];
    for (int c = 0; c < 3; c++) dx[c] = 0.5 * (xyz[3 * (size_t)j0 + c] - xyz[3 * (size_t)i + c]);
    double DP = 0.0;
    for (int j = 0; j < neqn; j++) {
      const double dQ = qj[j] - qi[j];
      const double corr = 0.5 * chi * dQ + (1.0 - chi) * (g[3 * j] * dx[0] + g[3 * j + 1] * dx[1] + g[3 * j + 2] * dx[2]);
      const double Q = qi[j] + corr * 1.0;
      const double DM = Q - qi[j];
      if (Q > qi[j]) DP = mx[j] - qi[j];
      else if (Q < qi[j]) DP = mn[j] - qi[j];
      const double t = (DP * DP + ep2 + 2.0 * DM * DP) / (DP * DP + 2.0 * DM * DM + DM * DP + ep2);
      if (t < l[j]) l[j] = t;
    }
  }
  for (int j = 0; j < neqn; j++) lim[(size_t)i * neqn + j] = l[j] < 0.0 ? 0.0 : l[j];
}

// CompressibleFREqnSet::ViscousFlux (ucs/compressibleFR.tcc:551) on the face
// state Q (native record) and face gradient g of the reacting gradient list
// (rhoi, u, v, w, T, concentrations): laminar, no species diffusion
__device__ void fr_viscous_flux(const pcfd_chem_model& m, const pcfd_chem_ref& ref, int sym2d, double Re,
                                const double* Q, const double* g, const EdgeArea& a, double* flux, int& bad) {
  const int ns = m.nspecies, off = 3 * ns;
  const double ux = g[off + 0], uy = g[off + 1], uz = g[off + 2];
  const double vx = g[off + 3], vy = g[off + 4], vz = g[off + 5];
  const double wx = g[off + 6], wy = g[off + 7], wz = g[off + 8];
  const double Tx = g[off + 9], Ty = g[off + 10], Tz = g[off + 11];
  const double u = Q[ns], v = Q[ns + 1], w = Q[ns + 2];
  double mu, kc;
  fr_transport(m, ref, Q, Q[ns + 3], mu, kc, bad);
  const double fact = 2.0 / 3.0;
  const double tauxx = 2.0 * fact * ux - fact * vy - fact * wz;
  const double tauyy = 2.0 * fact * vy - fact * ux - fact * wz;
  const double tauzz = 2.0 * fact * wz - fact * ux - fact * vy;
  const double tauxy = uy + vx, tauxz = uz + wx, tauyz = vz + wy;
  const double RK = a.w / Re, RKT = RK * mu;
  const double Tn = Tx * a.x + Ty * a.y + Tz * a.z;
  const double tauxn = -tauxx * a.x - tauxy * a.y - tauxz * a.z;
  const double tauyn = -tauxy * a.x - tauyy * a.y - tauyz * a.z;
  const double tauzn = -tauxz * a.x - tauyz * a.y - tauzz * a.z;
  for (int i = 0; i < ns; i++) flux[i] = 0.0;
  flux[ns + 0] = RKT * tauxn;
  flux[ns + 1] = RKT * tauyn;
  flux[ns + 2] = RKT * tauzn;
  flux[ns + 3] = RKT * (tauxn * u + tauyn * v + tauzn * w) + RK * (-kc) * Tn;
  if (sym2d >= 1 && sym2d <= 3) flux[ns + sym2d - 1] = 0.0;
}

// Kernel_Viscous_Flux (ucs/residual.tcc:390) of the reacting set, one edge
// per thread: averaged face state and gradients, the directional correction
// along the edge when `directional`, the flux leaving the left node into ef.
// Only the velocity and temperature terms of the gradient reach the flux, so
// only they are corrected.
__global__ void __launch_bounds__(128) k_chem_visc_edge(long long nedge, const pcfd_chem_model* __restrict__ gm,
                                                        pcfd_chem_ref ref, int sym2d, double Re, int directional,
                                                        const double* __restrict__ q, const double* __restrict__ grad,
                                                        const double* __restrict__ xyz, const int2* __restrict__ en,
                                                        const EdgeArea* __restrict__ ea, double* __restrict__ ef,
                                                        long long* bad_count) {
  const long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (e >= nedge) return;
  const pcfd_chem_model& m = *gm;
  const int ns = m.nspecies, neqn = ns + 4, nv = 6 + 3 * ns, nt = 2 * ns + 4;
  const int2 n = en[e];
  const double* qL = &q[(size_t)n.x * nv];
  const double* qR = &q[(size_t)n.y * nv];
  double Q[PCFD_CHEM_MAX_SPECIES + 4], g[3 * (2 * PCFD_CHEM_MAX_SPECIES + 4)];
  for (int i = 0; i < neqn; i++) Q[i] = (qL[i] + qR[i]) / 2.0;
  const double* gL = &grad[(size_t)n.x * nt * 3];
  const double* gR = &grad[(size_t)n.y * nt * 3];
  for (int j = ns; j < ns + 4; j++)
    for (int i = 0; i < 3; i++) g[3 * j + i] = 0.5 * (gL[3 * j + i] + gR[3 * j + i]);
  if (directional) {
    double dx[3], s2 = 0.0;
    for (int i = 0; i < 3; i++) {
      dx[i] = xyz[3 * (size_t)n.y + i] - xyz[3 * (size_t)n.x + i];
      s2 += dx[i] * dx[i];
    }
    for (int j = ns; j < ns + 4; j++) {
      const double qdots = dx[0] * g[3 * j] + dx[1] * g[3 * j + 1] + dx[2] * g[3 * j + 2];
      const double dq = (qR[j] - qL[j] - qdots) / s2;
      for (int i = 0; i < 3; i++) g[3 * j + i] += dq * dx[i];
    }
  }
  int bad = 0;
  double f[PCFD_CHEM_MAX_SPECIES + 4];
  fr_viscous_flux(m, ref, sym2d, Re, Q, g, ea[e], f, bad);
  for (int i = 0; i < neqn; i++) ef[(size_t)e * neqn + i] = f[i];
  if (bad) atomicAdd((unsigned long long*)bad_count, 1ull);
}

// Bkernel_Viscous_Flux (ucs/residual.tcc:473) on one partition: the face
// state averages the node and its phantom record, the gradient is the node's
__global__ void __launch_bounds__(128) k_chem_visc_bedge(long long nbedge, const pcfd_chem_model* __restrict__ gm,
                                                         pcfd_chem_ref ref, int sym2d, double Re,
                                                         const double* __restrict__ q,
                                                         const double* __restrict__ grad, const int2* __restrict__ bn,
                                                         const EdgeArea* __restrict__ ba, double* __restrict__ bf,
                                                         long long* bad_count) {
  const long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  if (k >= nbedge) return;
  const pcfd_chem_model& m = *gm;
  const int ns = m.nspecies, neqn = ns + 4, nv = 6 + 3 * ns, nt = 2 * ns + 4;
  const int2 n = bn[k];
  const double* qL = &q[(size_t)n.x * nv];
  const double* qR = &q[(size_t)n.y * nv];
  double Q[PCFD_CHEM_MAX_SPECIES + 4];
  for (int i = 0; i < neqn; i++) Q[i] = 0.5 * (qL[i] + qR[i]);
  int bad = 0;
  double f[PCFD_CHEM_MAX_SPECIES + 4];
  fr_viscous_flux(m, ref, sym2d, Re, Q, &grad[(size_t)n.x * nt * 3], ba[k], f, bad);
  for (int i = 0; i < neqn; i++) bf[(size_t)k * neqn + i] = f[i];
  if (bad) atomicAdd((unsigned long long*)bad_count, 1ull);
}

__global__ void __launch_bounds__(256) k_chem_gather(long long nnode, const pcfd_chem_model* __restrict__ gm,
                                                     pcfd_chem_ref ref, double ref_time, int reactions,
                                                     const double* __restrict__ q, const int* __restrict__ nptr,
                                                     const int* __restrict__ nedg, const double* __restrict__ ef,
                                                     const int* __restrict__ bptr, const int* __restrict__ bhe,
                                                     const double* __restrict__ bf, const double* __restrict__ vol,
                                                     double* __restrict__ b, double* __restrict__ part) {
  const pcfd_chem_model& m = *gm;
  const int ns = m.nspecies, neqn = ns + 4, nv = 6 + 3 * ns;
  double acc[PCFD_CHEM_MAX_SPECIES + 4];
  for (int j = 0; j < neqn; j++) acc[j] = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < nnode;
       i += (long long)gridDim.x * blockDim.x) {
    double r[PCFD_CHEM_MAX_SPECIES + 4];
    for (int j = 0; j < neqn; j++) r[j] = 0.0;
    for (int k = nptr[i]; k < nptr[i + 1]; k++) {
      const int se = nedg[k];
      if (se < 0) {
        const double* f = &ef[(size_t)(~se) * neqn];
        for (int j = 0; j < neqn; j++) r[j] += -f[j];
      } else {
        const double* f = &ef[(size_t)se * neqn];
        for (int j = 0; j < neqn; j++) r[j] += f[j];
      }
    }
    for (int p = bptr[i]; p < bptr[i + 1]; p++) {
      const double* f = &bf[(size_t)bhe[p] * neqn];
      for (int j = 0; j < neqn; j++) r[j] += -f[j];
    }
    if (reactions) {
      const double* Q = &q[(size_t)i * nv];
      double rhoi[PCFD_CHEM_MAX_SPECIES], w[PCFD_CHEM_MAX_SPECIES];
      for (int s = 0; s < ns; s++) rhoi[s] = Q[s] * ref.density;
      node_rates(m, rhoi, Q[ns + 3] * ref.temperature, w);
      for (int s = 0; s < ns; s++) {
        const double wn = w[s] / (ref.density / ref_time);
        r[s] += vol[i] * wn;
      }
    }
    for (int j = 0; j < neqn; j++) {
      b[(size_t)i * neqn + j] = r[j];
      acc[j] += r[j] * r[j];
    }
  }
  // deterministic block sums: warp shuffles, then a fixed-order sum
  __shared__ double red[8][PCFD_CHEM_MAX_SPECIES + 4];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int j = 0; j < neqn; j++) {
    double v = acc[j];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid][j] = v;
  }
  __syncthreads();
  if (threadIdx.x < neqn) {
    double v = 0.0;
    for (int w = 0; w < 8; w++) v += red[w][threadIdx.x];
    part[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = v;
  }
}

// the norms from the per-block partials, a warp per component, fixed order
__global__ void k_chem_norms(int nblocks, long long nnode, int neqn, const double* __restrict__ part,
                             double* __restrict__ norms) {
  const int lane = threadIdx.x & 31, c = threadIdx.x >> 5;
  if (c >= neqn) return;
  double v = 0.0;
  for (int bl = lane; bl < nblocks; bl += 32) v += part[(size_t)c * nblocks + bl];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) norms[1 + c] = sqrt(v) / (double)nnode;
  // resGlobal from the component sums (all squares), one more pass by warp 0
  if (c == 0) {
    double t = 0.0;
    for (int j = 0; j < neqn; j++) {
      double s = 0.0;
      for (int bl = lane; bl < nblocks; bl += 32) s += part[(size_t)j * nblocks + bl];
      for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      t += s;
    }
    if (lane == 0) norms[0] = sqrt(t) / ((double)nnode * neqn);
  }
}

int validate(const pcfd_chem_model* m) {
  if (m->nspecies < 1 || m->nspecies > PCFD_CHEM_MAX_SPECIES || m->nreactions < 0 ||
      m->nreactions > PCFD_CHEM_MAX_REACTIONS)
    return 0;
  for (int k = 0; k < m->nspecies; k++)
    if (!(m->mw[k] > 0.0) || m->nmu[k] < 0 || m->nmu[k] > PCFD_CHEM_MAX_TRANSPORT_FITS || m->nk[k] < 0 ||
        m->nk[k] > PCFD_CHEM_MAX_TRANSPORT_FITS)
      return 0;
  for (int j = 0; j < m->nreactions; j++) {
    const pcfd_chem_reaction& r = m->rx[j];
    if (r.type < 0 || r.type > 3 || r.nlocal < 0 || r.nlocal > PCFD_CHEM_MAX_LOCAL) return 0;
    for (int l = 0; l < r.nlocal; l++) {
      if (r.global[l] < 0 || r.global[l] >= m->nspecies) return 0;
      for (int q = 0; q < l; q++)
        if (r.global[q] == r.global[l]) return 0;  // one entry per species, as the reference merges them
    }
  }
  return 1;
}

int ensure_buf(ChemHandle* c, size_t ndoubles) {
  if (c->buf_cap >= ndoubles) return PCFD_OK;
  cudaFree(c->d_buf);
  c->d_buf = nullptr;
  c->buf_cap = 0;
  CHEM_TRY(cudaMalloc(&c->d_buf, ndoubles * sizeof(double)), "chem buffers");
  c->buf_cap = ndoubles;
  return PCFD_OK;
}

// Runs one node-state kernel on the handle's stream.  Inputs and outputs are
// (pointer, doubles per node) pairs; with dev = 0 they are staged through
// the handle's buffer (inputs copied in, outputs copied back).  Returns the
// count the kernel left in *d_count.
template <int NIN, int NOUT, class F>
int node_call(ChemHandle* c, long long n, int dev, const double* const (&in)[NIN], const int (&win)[NIN],
              double* const (&out)[NOUT], const int (&wout)[NOUT], long long* count, F&& launch_kernel) {
  const double* din[NIN];
  double* dout[NOUT];
  if (!c->d_count) CHEM_TRY(cudaMalloc(&c->d_count, sizeof(long long)), "chem buffers");
  CHEM_TRY(cudaMemsetAsync(c->d_count, 0, sizeof(long long), c->stream), "chem count");
  if (dev) {
    for (int k = 0; k < NIN; k++) din[k] = in[k];
    for (int k = 0; k < NOUT; k++) dout[k] = out[k];
  } else {
    size_t total = 0;
    for (int k = 0; k < NIN; k++) total += (size_t)n * win[k];
    for (int k = 0; k < NOUT; k++) total += (size_t)n * wout[k];
    int rc = ensure_buf(c, total);
    if (rc) return rc;
    double* b = c->d_buf;
    for (int k = 0; k < NIN; k++) {
      CHEM_TRY(cudaMemcpyAsync(b, in[k], (size_t)n * win[k] * sizeof(double), cudaMemcpyHostToDevice, c->stream),
               "chem copy in");
      din[k] = b;
      b += (size_t)n * win[k];
    }
    for (int k = 0; k < NOUT; k++) {
      dout[k] = b;
      b += (size_t)n * wout[k];
    }
  }
  launch_kernel(din, dout);
  CHEM_TRY(cudaGetLastError(), "chem node-state launch");
  if (!dev)
    for (int k = 0; k < NOUT; k++)
      CHEM_TRY(cudaMemcpyAsync(out[k], dout[k], (size_t)n * wout[k] * sizeof(double), cudaMemcpyDeviceToHost,
                               c->stream),
               "chem copy out");
  long long cnt = 0;
  CHEM_TRY(cudaMemcpyAsync(&cnt, c->d_count, sizeof(long long), cudaMemcpyDeviceToHost, c->stream), "chem count");
  CHEM_TRY(cudaStreamSynchronize(c->stream), "chem node-state");
  if (count) *count = cnt;
  return PCFD_OK;
}

bool ref_ok(const pcfd_chem_ref* r) {
  return r && r->density > 0.0 && r->pressure > 0.0 && r->temperature > 0.0 && r->specific_enthalpy > 0.0 &&
         r->velocity > 0.0;
}

int ensure_io(ChemHandle* c, long long n) {
  if (c->cap >= n) return PCFD_OK;
  cudaFree(c->d_rho);
  cudaFree(c->d_T);
  cudaFree(c->d_w);
  c->d_rho = c->d_T = c->d_w = nullptr;
  c->cap = 0;
  const size_t ns = c->host.nspecies;
  CHEM_TRY(cudaMalloc(&c->d_rho, (size_t)n * ns * sizeof(double)), "chem buffers");
  CHEM_TRY(cudaMalloc(&c->d_T, (size_t)n * sizeof(double)), "chem buffers");
  CHEM_TRY(cudaMalloc(&c->d_w, (size_t)n * ns * sizeof(double)), "chem buffers");
  c->cap = n;
  return PCFD_OK;
}

}  // namespace

extern "C" {

PCFD_API int pcfd_chem_create(const pcfd_chem_model* model, pcfd_chem_t* out) {
  if (!model || !out) {
    pcfd_set_last_error("pcfd_chem_create: null pointer");
    return PCFD_ERR_ARG;
  }
  *out = nullptr;
  if (!validate(model)) {
    pcfd_set_last_error("pcfd_chem_create: model out of range (species, reactions or indices)");
    return PCFD_ERR_ARG;
  }
  ChemHandle* c = new ChemHandle();
  std::memcpy(&c->host, model, sizeof(pcfd_chem_model));
  cudaError_t e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
  if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
  if (e == cudaSuccess) e = cudaMalloc(&c->dev, sizeof(pcfd_chem_model));
  if (e == cudaSuccess) e = cudaMemcpy(c->dev, model, sizeof(pcfd_chem_model), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    ChemDerived d;
    std::memset(&d, 0, sizeof(d));
    for (int s = 0; s < model->nspecies; s++) {
      d.R[s] = kUnivR / model->mw[s];
      for (int k = 0; k < 2; k++) {
        const double* a = k ? model->nasa_hi[s] : model->nasa_lo[s];
        const double hc[6] = {a[5], a[0], a[1] / 2.0, a[2] / 3.0, a[3] / 4.0, a[4] / 5.0};
        for (int t = 0; t < 6; t++) d.h[k][s][t] = hc[t];
        for (int t = 0; t < 5; t++) d.cp[k][s][t] = a[t];
      }
    }
    e = cudaMalloc(&c->dder, sizeof(ChemDerived));
    if (e == cudaSuccess) e = cudaMemcpy(c->dder, &d, sizeof(ChemDerived), cudaMemcpyHostToDevice);
  }
  if (e != cudaSuccess) {
    int rc = cuda_fail(e, "pcfd_chem_create");
    pcfd_chem_destroy((pcfd_chem_t)c);
    return rc;
  }
  *out = (pcfd_chem_t)c;
  return PCFD_OK;
}

PCFD_API int pcfd_chem_destroy(pcfd_chem_t h) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c) return PCFD_OK;
  if (c->stream) cudaStreamSynchronize(c->stream);
  cudaFree(c->dev);
  cudaFree(c->dder);
  cudaFree(c->d_rho);
  cudaFree(c->d_T);
  cudaFree(c->d_w);
  cudaFree(c->d_buf);
  cudaFree(c->d_count);
  void* mesh_ptrs[] = {c->d_en, c->d_bn, c->d_ea, c->d_ba, c->d_vol, c->d_nptr, c->d_nedg, c->d_bptr,
                       c->d_bhe, c->d_q, c->d_ef, c->d_bf, c->d_b, c->d_part, c->d_norms};
  for (void* p : mesh_ptrs) cudaFree(p);
  if (c->ev0) cudaEventDestroy(c->ev0);
  if (c->ev1) cudaEventDestroy(c->ev1);
  if (c->stream) cudaStreamDestroy(c->stream);
  delete c;
  return PCFD_OK;
}

PCFD_API int pcfd_chem_production_rates_dev(pcfd_chem_t h, long long n, const double* rhoi, const double* T,
                                            double* wdot, double* ms_out) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || n < 0 || (n > 0 && (!rhoi || !T || !wdot))) {
    pcfd_set_last_error("pcfd_chem_production_rates_dev: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (n == 0) {
    if (ms_out) *ms_out = 0.0;
    return PCFD_OK;
  }
  CHEM_TRY(cudaEventRecord(c->ev0, c->stream), "chem event");
  k_chem_rates<<<(unsigned)((n + 127) / 128), 128, 0, c->stream>>>(n, c->dev, rhoi, T, wdot);
  CHEM_TRY(cudaGetLastError(), "k_chem_rates launch");
  CHEM_TRY(cudaEventRecord(c->ev1, c->stream), "chem event");
  CHEM_TRY(cudaEventSynchronize(c->ev1), "k_chem_rates");
  if (ms_out) {
    float ms = 0.f;
    CHEM_TRY(cudaEventElapsedTime(&ms, c->ev0, c->ev1), "chem event");
    *ms_out = ms;
  }
  return PCFD_OK;
}

PCFD_API int pcfd_chem_production_rates(pcfd_chem_t h, long long n, const double* rhoi, const double* T,
                                        double* wdot) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || n < 0 || (n > 0 && (!rhoi || !T || !wdot))) {
    pcfd_set_last_error("pcfd_chem_production_rates: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (n == 0) return PCFD_OK;
  int rc = ensure_io(c, n);
  if (rc) return rc;
  const size_t ns = c->host.nspecies;
  CHEM_TRY(cudaMemcpyAsync(c->d_rho, rhoi, (size_t)n * ns * sizeof(double), cudaMemcpyHostToDevice, c->stream),
           "chem copy");
  CHEM_TRY(cudaMemcpyAsync(c->d_T, T, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream), "chem copy");
  rc = pcfd_chem_production_rates_dev(h, n, c->d_rho, c->d_T, c->d_w, nullptr);
  if (rc) return rc;
  CHEM_TRY(cudaMemcpyAsync(wdot, c->d_w, (size_t)n * ns * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
           "chem copy");
  CHEM_TRY(cudaStreamSynchronize(c->stream), "chem sync");
  return PCFD_OK;
}

#define CHEM_GRID(n) (unsigned)(((n) + 127) / 128), 128, 0, c->stream

PCFD_API int pcfd_chem_find_T_given_P(pcfd_chem_t h, const pcfd_chem_ref* ref, long long n, const double* rhoi,
                                      const double* P, const double* T_init, double* T, long long* nonconverged,
                                      int dev) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || !ref_ok(ref) || n < 0 || (n > 0 && (!rhoi || !P || !T_init || !T))) {
    pcfd_set_last_error("pcfd_chem_find_T_given_P: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (nonconverged) *nonconverged = 0;
  if (n == 0) return PCFD_OK;
  const int ns = c->host.nspecies;
  const pcfd_chem_ref r = *ref;
  return node_call<3, 1>(c, n, dev, {rhoi, P, T_init}, {ns, 1, 1}, {T}, {1}, nonconverged,
                         [&](const double* const* in, double* const* out) {
                           k_chem_find_T<<<CHEM_GRID(n)>>>(n, c->dev, c->dder, r, in[0], in[1], in[2], out[0], c->d_count);
                         });
}

PCFD_API int pcfd_chem_conservative_to_native(pcfd_chem_t h, const pcfd_chem_ref* ref, long long n, const double* q,
                                              const double* P, double* native, int dev) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || !ref_ok(ref) || n < 0 || (n > 0 && (!q || !P || !native))) {
    pcfd_set_last_error("pcfd_chem_conservative_to_native: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (n == 0) return PCFD_OK;
  const int ns = c->host.nspecies;
  const pcfd_chem_ref r = *ref;
  long long bad = 0;
  int rc = node_call<2, 1>(c, n, dev, {q, P}, {ns + 4, 1}, {native}, {4}, &bad,
                           [&](const double* const* in, double* const* out) {
                             k_chem_c2n<<<CHEM_GRID(n)>>>(n, c->dev, c->dder, r, in[0], in[1], out[0], c->d_count);
                           });
  if (rc) return rc;
  if (bad) {
    pcfd_set_last_error("pcfd_chem_conservative_to_native: the temperature Newton iteration did not converge on " +
                        std::to_string(bad) + " node(s)");
    return PCFD_ERR_NUMERIC;
  }
  return PCFD_OK;
}

PCFD_API int pcfd_chem_native_to_conservative(pcfd_chem_t h, const pcfd_chem_ref* ref, long long n, const double* rhoi,
                                              const double* native, const double* P, double* q, int dev) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || !ref_ok(ref) || n < 0 || (n > 0 && (!rhoi || !native || !P || !q))) {
    pcfd_set_last_error("pcfd_chem_native_to_conservative: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (n == 0) return PCFD_OK;
  const int ns = c->host.nspecies;
  const pcfd_chem_ref r = *ref;
  return node_call<3, 1>(c, n, dev, {rhoi, native, P}, {ns, 4, 1}, {q}, {4}, nullptr,
                         [&](const double* const* in, double* const* out) {
                           k_chem_n2c<<<CHEM_GRID(n)>>>(n, c->dev, c->dder, r, in[0], in[1], in[2], out[0]);
                         });
}

PCFD_API int pcfd_chem_aux(pcfd_chem_t h, const pcfd_chem_ref* ref, long long n, const double* rhoi, const double* T,
                           double* P, double* cvi, double* mol, int dev) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || !ref_ok(ref) || n < 0 || (n > 0 && (!rhoi || !T || !P || !cvi || !mol))) {
    pcfd_set_last_error("pcfd_chem_aux: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (n == 0) return PCFD_OK;
  const int ns = c->host.nspecies;
  const pcfd_chem_ref r = *ref;
  return node_call<2, 3>(c, n, dev, {rhoi, T}, {ns, 1}, {P, cvi, mol}, {1, ns, ns}, nullptr,
                         [&](const double* const* in, double* const* out) {
                           k_chem_aux<<<CHEM_GRID(n)>>>(n, c->dev, c->dder, r, in[0], in[1], out[0], out[1], out[2]);
                         });
}

PCFD_API int pcfd_chem_transport(pcfd_chem_t h, const pcfd_chem_ref* ref, long long n, const double* rhoi,
                                 const double* T, double* mu, double* k, int dev) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || !ref_ok(ref) || n < 0 || (n > 0 && (!rhoi || !T || !mu || !k))) {
    pcfd_set_last_error("pcfd_chem_transport: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (n == 0) return PCFD_OK;
  const int ns = c->host.nspecies;
  const pcfd_chem_ref r = *ref;
  long long bad = 0;
  int rc = node_call<2, 2>(c, n, dev, {rhoi, T}, {ns, 1}, {mu, k}, {1, 1}, &bad,
                           [&](const double* const* in, double* const* out) {
                             k_chem_transport<<<CHEM_GRID(n)>>>(n, c->dev, r, in[0], in[1], out[0], out[1],
                                                                c->d_count);
                           });
  if (rc) return rc;
  if (bad) {
    pcfd_set_last_error("pcfd_chem_transport: " + std::to_string(bad) +
                        " node(s) above every transport fit's temperature range");
    return PCFD_ERR_ARG;
  }
  return PCFD_OK;
}

PCFD_API int pcfd_chem_source_jacobian(pcfd_chem_t h, const pcfd_chem_ref* ref, double ref_time, long long n,
                                       const double* q, const double* vol, double* A, int dev) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || !ref_ok(ref) || !(ref_time > 0.0) || n < 0 || (n > 0 && (!q || !vol || !A))) {
    pcfd_set_last_error("pcfd_chem_source_jacobian: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (n == 0) return PCFD_OK;
  const int ns = c->host.nspecies, neqn = ns + 4, nv = 6 + 3 * ns;
  const pcfd_chem_ref r = *ref;
  return node_call<2, 1>(c, n, dev, {q, vol}, {nv, 1}, {A}, {neqn * neqn}, nullptr,
                         [&](const double* const* in, double* const* out) {
                           k_chem_source_jac<<<CHEM_GRID(n)>>>(n, c->dev, r, ref_time, in[0], in[1], out[0]);
                         });
}

PCFD_API int pcfd_chem_temporal_terms(pcfd_chem_t h, const pcfd_chem_ref* ref, long long n, const double* q,
                                      const double* vol, const double* dtau, const double* beta, double cnp1,
                                      double dt, int local_ts, double* A, int dev) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || !ref_ok(ref) || n < 0 || (n > 0 && (!q || !vol || !dtau || !beta || !A))) {
    pcfd_set_last_error("pcfd_chem_temporal_terms: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (n == 0) return PCFD_OK;
  const int ns = c->host.nspecies, neqn = ns + 4, nv = 6 + 3 * ns;
  const pcfd_chem_ref r = *ref;
  return node_call<5, 1>(c, n, dev, {q, vol, dtau, beta, A}, {nv, 1, 1, 1, neqn * neqn}, {A}, {neqn * neqn}, nullptr,
                         [&](const double* const* in, double* const* out) {
                           k_chem_temporal<<<CHEM_GRID(n)>>>(n, c->dev, c->dder, r, in[0], in[1], in[2], in[3], cnp1,
                                                             dt, local_ts, in[4], out[0]);
                         });
}

PCFD_API int pcfd_chem_hllc_flux(pcfd_chem_t h, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o, long long nnode,
                                 const double* q, long long nedge, const int* edges, const double* avec, double* flux,
                                 long long* nfail, int dev) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || !ref_ok(ref) || !o || nnode < 0 || nedge < 0 ||
      (nedge > 0 && (nnode <= 0 || !q || !edges || !avec || !flux))) {
    pcfd_set_last_error("pcfd_chem_hllc_flux: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (nfail) *nfail = 0;
  if (nedge == 0) return PCFD_OK;
  const int ns = c->host.nspecies;
  const size_t nv = 6 + 3 * (size_t)ns;
  if (!dev) {
    // the node ids are checked here; device callers own their edge list
    for (long long e = 0; e < 2 * nedge; e++)
      if (edges[e] < 0 || edges[e] >= nnode) {
        pcfd_set_last_error("pcfd_chem_hllc_flux: edge node id out of range");
        return PCFD_ERR_ARG;
      }
  }
  if (!c->d_count) CHEM_TRY(cudaMalloc(&c->d_count, sizeof(long long)), "chem buffers");
  CHEM_TRY(cudaMemsetAsync(c->d_count, 0, sizeof(long long), c->stream), "chem count");
  const double* dq = q;
  const int2* de = (const int2*)edges;
  const EdgeArea* da = (const EdgeArea*)avec;
  double* df = flux;
  if (!dev) {
    // staging: avec first (the EdgeArea loads want 32-byte alignment; the
    // buffer is 256-byte aligned), then q, flux and the edge ids
    const size_t need = (size_t)nedge * 4 + (size_t)nnode * nv + (size_t)nedge * (ns + 4) + (size_t)nedge;
    int rc = ensure_buf(c, need);
    if (rc) return rc;
    double* b = c->d_buf;
    CHEM_TRY(cudaMemcpyAsync(b, avec, (size_t)nedge * 4 * sizeof(double), cudaMemcpyHostToDevice, c->stream), "chem copy");
    da = (const EdgeArea*)b;
    b += (size_t)nedge * 4;
    CHEM_TRY(cudaMemcpyAsync(b, q, (size_t)nnode * nv * sizeof(double), cudaMemcpyHostToDevice, c->stream), "chem copy");
    dq = b;
    b += (size_t)nnode * nv;
    df = b;
    b += (size_t)nedge * (ns + 4);
    CHEM_TRY(cudaMemcpyAsync(b, edges, (size_t)nedge * 2 * sizeof(int), cudaMemcpyHostToDevice, c->stream), "chem copy");
    de = (const int2*)b;
  } else if ((reinterpret_cast<uintptr_t>(avec) & 31) != 0 || (reinterpret_cast<uintptr_t>(edges) & 7) != 0) {
    pcfd_set_last_error("pcfd_chem_hllc_flux: device avec must be 32-byte and edges 8-byte aligned");
    return PCFD_ERR_ARG;
  }
  const pcfd_chem_ref r = *ref;
  const pcfd_chem_flux_opts oo = *o;
  k_chem_hllc<<<CHEM_GRID(nedge)>>>(nedge, nnode, c->dev, c->dder, r, oo, dq, de, da, df, c->d_count);
  CHEM_TRY(cudaGetLastError(), "k_chem_hllc launch");
  if (!dev)
    CHEM_TRY(cudaMemcpyAsync(flux, df, (size_t)nedge * (ns + 4) * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
             "chem copy out");
  long long bad = 0;
  CHEM_TRY(cudaMemcpyAsync(&bad, c->d_count, sizeof(long long), cudaMemcpyDeviceToHost, c->stream), "chem count");
  CHEM_TRY(cudaStreamSynchronize(c->stream), "k_chem_hllc");
  if (nfail) *nfail = bad;
  if (bad) {
    pcfd_set_last_error("pcfd_chem_hllc_flux: " + std::to_string(bad) +
                        " edge(s) with no HLLC branch or a node id out of range");
    return PCFD_ERR_NUMERIC;
  }
  return PCFD_OK;
}

PCFD_API int pcfd_chem_attach_mesh(pcfd_chem_t h, const pcfd_mesh_view* m) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || !m || m->nnode <= 0 || m->nedge < 0 || m->nbedge < 0 || (m->nedge > 0 && (!m->edges || !m->edge_area)) ||
      (m->nbedge > 0 && (!m->bedges || !m->bedge_area)) || !m->vol) {
    pcfd_set_last_error("pcfd_chem_attach_mesh: bad mesh");
    return PCFD_ERR_ARG;
  }
  const long long nn = m->nnode, ne = m->nedge, nb = m->nbedge, ntot = nn + nb;
  for (long long e = 0; e < 2 * ne; e++)
    if (m->edges[e] < 0 || m->edges[e] >= nn) {
      pcfd_set_last_error("pcfd_chem_attach_mesh: edge node id out of range");
      return PCFD_ERR_ARG;
    }
  for (long long k = 0; k < nb; k++)
    if (m->bedges[2 * k] < 0 || m->bedges[2 * k] >= nn || m->bedges[2 * k + 1] < nn || m->bedges[2 * k + 1] >= ntot) {
      pcfd_set_last_error("pcfd_chem_attach_mesh: boundary half-edge ids out of range");
      return PCFD_ERR_ARG;
    }
  // node -> incident edges (ascending id, ~e at the left end), node -> half-edges
  std::vector<int> nptr(nn + 1, 0), bptr(nn + 1, 0);
  for (long long e = 0; e < ne; e++) {
    nptr[m->edges[2 * e] + 1]++;
    nptr[m->edges[2 * e + 1] + 1]++;
  }
  for (long long k = 0; k < nb; k++) bptr[m->bedges[2 * k] + 1]++;
  for (long long i = 0; i < nn; i++) {
    nptr[i + 1] += nptr[i];
    bptr[i + 1] += bptr[i];
  }
  std::vector<int> nedg(2 * ne > 0 ? 2 * ne : 1), bhe(nb > 0 ? nb : 1), fill(nptr.begin(), nptr.end() - 1),
      bfill(bptr.begin(), bptr.end() - 1);
  for (long long e = 0; e < ne; e++) {
    nedg[fill[m->edges[2 * e]]++] = ~(int)e;
    nedg[fill[m->edges[2 * e + 1]]++] = (int)e;
  }
  for (long long k = 0; k < nb; k++) bhe[bfill[m->bedges[2 * k]]++] = (int)k;
  void* mesh_ptrs[] = {c->d_en, c->d_bn, c->d_ea, c->d_ba, c->d_vol, c->d_nptr, c->d_nedg, c->d_bptr,
                       c->d_bhe, c->d_q, c->d_ef, c->d_bf, c->d_b, c->d_part, c->d_norms, c->d_xyz, c->d_grad,
                       c->d_sw, c->d_btag, c->d_bctab, c->d_lim};
  for (void* p : mesh_ptrs) cudaFree(p);
  c->d_en = c->d_bn = nullptr;
  c->d_ea = c->d_ba = nullptr;
  c->d_vol = c->d_q = c->d_ef = c->d_bf = c->d_b = c->d_part = c->d_norms = c->d_xyz = c->d_grad = c->d_sw = nullptr;
  c->d_btag = nullptr;
  c->d_bctab = nullptr;
  c->bc_cap = 0;
  c->d_lim = nullptr;
  c->d_nptr = c->d_nedg = c->d_bptr = c->d_bhe = nullptr;
  c->nnode = c->nedge = c->nbedge = 0;
  const int ns = c->host.nspecies, neqn = ns + 4;
  const size_t nv = 6 + 3 * (size_t)ns;
  auto up = [&](void** dst, const void* src, size_t bytes) -> cudaError_t {
    cudaError_t e = cudaMalloc(dst, bytes > 0 ? bytes : 16);
    if (e == cudaSuccess && bytes > 0) e = cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice);
    return e;
  };
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = up((void**)&c->d_en, m->edges, (size_t)ne * 2 * sizeof(int));
  if (e == cudaSuccess) e = up((void**)&c->d_ea, m->edge_area, (size_t)ne * 4 * sizeof(double));
  if (e == cudaSuccess) e = up((void**)&c->d_bn, m->bedges, (size_t)nb * 2 * sizeof(int));
  if (e == cudaSuccess) e = up((void**)&c->d_ba, m->bedge_area, (size_t)nb * 4 * sizeof(double));
  if (e == cudaSuccess) e = up((void**)&c->d_vol, m->vol, (size_t)nn * sizeof(double));
  if (e == cudaSuccess && m->xyz) e = up((void**)&c->d_xyz, m->xyz, (size_t)nn * 3 * sizeof(double));
  if (e == cudaSuccess && m->sw) e = up((void**)&c->d_sw, m->sw, (size_t)nn * 6 * sizeof(double));
  if (e == cudaSuccess && m->bfactag) e = up((void**)&c->d_btag, m->bfactag, (size_t)nb * sizeof(int));
  if (e == cudaSuccess) e = up((void**)&c->d_nptr, nptr.data(), nptr.size() * sizeof(int));
  if (e == cudaSuccess) e = up((void**)&c->d_nedg, nedg.data(), nedg.size() * sizeof(int));
  if (e == cudaSuccess) e = up((void**)&c->d_bptr, bptr.data(), bptr.size() * sizeof(int));
  if (e == cudaSuccess) e = up((void**)&c->d_bhe, bhe.data(), bhe.size() * sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_q, (size_t)ntot * nv * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_ef, ((size_t)ne > 0 ? ne : 1) * neqn * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_bf, ((size_t)nb > 0 ? nb : 1) * neqn * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_b, (size_t)nn * neqn * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_part, (size_t)kChemNormBlocks * neqn * sizeof(double));
  if (e == cudaSuccess) e = cudaMalloc((void**)&c->d_norms, (size_t)(1 + neqn) * sizeof(double));
  if (e != cudaSuccess) return cuda_fail(e, "pcfd_chem_attach_mesh");
  c->nnode = nn;
  c->nedge = ne;
  c->nbedge = nb;
  return PCFD_OK;
}

PCFD_API int pcfd_chem_update_bcs(pcfd_chem_t h, const pcfd_chem_ref* ref, int ntags, const int* bc_type,
                                  const double* twall, const double* qref, int no_cvbc, double* q, int dev) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || !ref_ok(ref) || ntags <= 0 || !bc_type || !twall || !qref || !q) {
    pcfd_set_last_error("pcfd_chem_update_bcs: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (c->nnode <= 0 || (c->nbedge > 0 && !c->d_btag)) {
    pcfd_set_last_error("pcfd_chem_update_bcs: no mesh with face tags attached");
    return PCFD_ERR_STATE;
  }
  const int ns = c->host.nspecies;
  const size_t nv = 6 + 3 * (size_t)ns;
  const long long nn = c->nnode, nb = c->nbedge;
  // the per-tag tables on the device
  const size_t tb = (size_t)ntags * (sizeof(int) + sizeof(double) + nv * sizeof(double));
  if (c->bc_cap < tb) {
    cudaFree(c->d_bctab);
    c->d_bctab = nullptr;
    c->bc_cap = 0;
    CHEM_TRY(cudaMalloc(&c->d_bctab, tb), "chem buffers");
    c->bc_cap = tb;
  }
  double* d_twall = (double*)c->d_bctab;
  double* d_qref = d_twall + ntags;
  int* d_type = (int*)(d_qref + (size_t)ntags * nv);
  CHEM_TRY(cudaMemcpyAsync(d_twall, twall, (size_t)ntags * sizeof(double), cudaMemcpyHostToDevice, c->stream),
           "chem copy");
  CHEM_TRY(cudaMemcpyAsync(d_qref, qref, (size_t)ntags * nv * sizeof(double), cudaMemcpyHostToDevice, c->stream),
           "chem copy");
  CHEM_TRY(cudaMemcpyAsync(d_type, bc_type, (size_t)ntags * sizeof(int), cudaMemcpyHostToDevice, c->stream),
           "chem copy");
  double* dq = q;
  if (!dev) {
    CHEM_TRY(cudaMemcpyAsync(c->d_q, q, (size_t)(nn + nb) * nv * sizeof(double), cudaMemcpyHostToDevice, c->stream),
             "chem copy");
    dq = c->d_q;
  }
  if (!c->d_count) CHEM_TRY(cudaMalloc(&c->d_count, sizeof(long long)), "chem buffers");
  CHEM_TRY(cudaMemsetAsync(c->d_count, 0, sizeof(long long), c->stream), "chem count");
  const ChemBc bc{ntags, no_cvbc, d_type, d_twall, d_qref};
  k_chem_bcs<<<CHEM_GRID(nn)>>>(nn, c->dev, c->dder, *ref, bc, c->d_bn, c->d_ba, c->d_btag, c->d_bptr, c->d_bhe, dq,
                                c->d_count);
  CHEM_TRY(cudaGetLastError(), "k_chem_bcs launch");
  if (!dev)
    CHEM_TRY(cudaMemcpyAsync(q, dq, (size_t)(nn + nb) * nv * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
             "chem copy out");
  long long bad = 0;
  CHEM_TRY(cudaMemcpyAsync(&bad, c->d_count, sizeof(long long), cudaMemcpyDeviceToHost, c->stream), "chem count");
  CHEM_TRY(cudaStreamSynchronize(c->stream), "chem boundary conditions");
  if (bad) {
    pcfd_set_last_error("pcfd_chem_update_bcs: " + std::to_string(bad) +
                        " half-edge(s) with a condition the reacting path does not build (far field, "
                        "characteristic wall, adiabatic no-slip)");
    return PCFD_ERR_ARG;
  }
  return PCFD_OK;
}

PCFD_API int pcfd_chem_limiter(pcfd_chem_t h, double chi, const double* q, const double* grad, double* lim, int dev) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || !q || !grad || !lim) {
    pcfd_set_last_error("pcfd_chem_limiter: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (c->nnode <= 0 || !c->d_xyz) {
    pcfd_set_last_error("pcfd_chem_limiter: no mesh with coordinates attached");
    return PCFD_ERR_STATE;
  }
  const int ns = c->host.nspecies, neqn = ns + 4, nt = 2 * ns + 4;
  const size_t nv = 6 + 3 * (size_t)ns;
  const long long nn = c->nnode, nb = c->nbedge;
  const double* dq = q;
  const double* dg = grad;
  double* dl = lim;
  if (!dev) {
    if (!c->d_grad) CHEM_TRY(cudaMalloc(&c->d_grad, (size_t)nn * nt * 3 * sizeof(double)), "chem buffers");
    if (!c->d_lim) CHEM_TRY(cudaMalloc(&c->d_lim, (size_t)nn * neqn * sizeof(double)), "chem buffers");
    CHEM_TRY(cudaMemcpyAsync(c->d_q, q, (size_t)(nn + nb) * nv * sizeof(double), cudaMemcpyHostToDevice, c->stream),
             "chem copy");
    CHEM_TRY(cudaMemcpyAsync(c->d_grad, grad, (size_t)nn * nt * 3 * sizeof(double), cudaMemcpyHostToDevice,
                             c->stream),
             "chem copy");
    dq = c->d_q;
    dg = c->d_grad;
    dl = c->d_lim;
  }
  k_chem_limiter<<<CHEM_GRID(nn)>>>(nn, c->dev, chi, dq, dg, c->d_xyz, c->d_vol, c->d_en, c->d_nptr, c->d_nedg, dl);
  CHEM_TRY(cudaGetLastError(), "k_chem_limiter launch");
  if (!dev)
    CHEM_TRY(cudaMemcpyAsync(lim, dl, (size_t)nn * neqn * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
             "chem copy out");
  CHEM_TRY(cudaStreamSynchronize(c->stream), "chem limiter");
  return PCFD_OK;
}

PCFD_API int pcfd_chem_gradient(pcfd_chem_t h, const double* q, const int* sym_tags, int nsym, double* grad,
                                int dev) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || !q || !grad || nsym < 0 || nsym > kChemMaxSym || (nsym > 0 && !sym_tags)) {
    pcfd_set_last_error("pcfd_chem_gradient: bad arguments (at most 8 symmetry tags)");
    return PCFD_ERR_ARG;
  }
  if (c->nnode <= 0 || !c->d_xyz || !c->d_sw || (c->nbedge > 0 && !c->d_btag)) {
    pcfd_set_last_error("pcfd_chem_gradient: no mesh with coordinates and LSQ matrices attached");
    return PCFD_ERR_STATE;
  }
  const int ns = c->host.nspecies, nt = 2 * ns + 4;
  const size_t nv = 6 + 3 * (size_t)ns;
  const long long nn = c->nnode, nb = c->nbedge;
  ChemSym sym{nsym, {0}};
  for (int u = 0; u < nsym; u++) sym.tag[u] = sym_tags[u];
  const double* dq = q;
  double* dg = grad;
  if (!dev) {
    if (!c->d_grad) CHEM_TRY(cudaMalloc(&c->d_grad, (size_t)nn * nt * 3 * sizeof(double)), "chem buffers");
    CHEM_TRY(cudaMemcpyAsync(c->d_q, q, (size_t)(nn + nb) * nv * sizeof(double), cudaMemcpyHostToDevice, c->stream),
             "chem copy");
    dq = c->d_q;
    dg = c->d_grad;
  }
  k_chem_gradient<<<CHEM_GRID(nn)>>>(nn, c->dev, dq, c->d_en, c->d_nptr, c->d_nedg, c->d_xyz, c->d_sw, c->d_bptr,
                                     c->d_bhe, c->d_btag, c->d_ba, sym, dg);
  CHEM_TRY(cudaGetLastError(), "k_chem_gradient launch");
  if (!dev)
    CHEM_TRY(cudaMemcpyAsync(grad, dg, (size_t)nn * nt * 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
             "chem copy out");
  CHEM_TRY(cudaStreamSynchronize(c->stream), "chem gradient");
  return PCFD_OK;
}

PCFD_API int pcfd_chem_viscous_residual(pcfd_chem_t h, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o,
                                        double Re, int directional, const double* q, const double* grad, double* b,
                                        int dev) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || !ref_ok(ref) || !o || !q || !grad || !b || !(Re > 0.0)) {
    pcfd_set_last_error("pcfd_chem_viscous_residual: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (c->nnode <= 0) {
    pcfd_set_last_error("pcfd_chem_viscous_residual: no mesh attached (pcfd_chem_attach_mesh)");
    return PCFD_ERR_STATE;
  }
  if (directional && !c->d_xyz) {
    pcfd_set_last_error("pcfd_chem_viscous_residual: the attached mesh has no coordinates");
    return PCFD_ERR_STATE;
  }
  for (int s = 0; s < c->host.nspecies; s++)
    if (c->host.nmu[s] == 0 || c->host.nk[s] == 0) {
      pcfd_set_last_error("pcfd_chem_viscous_residual: the model has no transport fits");
      return PCFD_ERR_STATE;
    }
  const int ns = c->host.nspecies, neqn = ns + 4, nt = 2 * ns + 4;
  const size_t nv = 6 + 3 * (size_t)ns;
  const long long nn = c->nnode, ne = c->nedge, nb = c->nbedge;
  const double* dq = q;
  const double* dg = grad;
  if (!dev) {
    if (!c->d_grad) CHEM_TRY(cudaMalloc(&c->d_grad, (size_t)nn * nt * 3 * sizeof(double)), "chem buffers");
    CHEM_TRY(cudaMemcpyAsync(c->d_q, q, (size_t)(nn + nb) * nv * sizeof(double), cudaMemcpyHostToDevice, c->stream),
             "chem copy");
    CHEM_TRY(cudaMemcpyAsync(c->d_grad, grad, (size_t)nn * nt * 3 * sizeof(double), cudaMemcpyHostToDevice,
                             c->stream),
             "chem copy");
    dq = c->d_q;
    dg = c->d_grad;
  }
  double* db = dev ? b : c->d_b;
  if (!c->d_count) CHEM_TRY(cudaMalloc(&c->d_count, sizeof(long long)), "chem buffers");
  CHEM_TRY(cudaMemsetAsync(c->d_count, 0, sizeof(long long), c->stream), "chem count");
  const pcfd_chem_ref r = *ref;
  if (ne > 0) {
    k_chem_visc_edge<<<CHEM_GRID(ne)>>>(ne, c->dev, r, o->symmetry2D, Re, directional, dq, dg, c->d_xyz, c->d_en,
                                        c->d_ea, c->d_ef, c->d_count);
    CHEM_TRY(cudaGetLastError(), "k_chem_visc_edge launch");
  }
  if (nb > 0) {
    k_chem_visc_bedge<<<CHEM_GRID(nb)>>>(nb, c->dev, r, o->symmetry2D, Re, dq, dg, c->d_bn, c->d_ba, c->d_bf,
                                         c->d_count);
    CHEM_TRY(cudaGetLastError(), "k_chem_visc_bedge launch");
  }
  // the same deterministic per-node sum as the inviscid residual, without
  // the chemistry source
  k_chem_gather<<<kChemNormBlocks, 256, 0, c->stream>>>(nn, c->dev, r, 1.0, 0, dq, c->d_nptr, c->d_nedg, c->d_ef,
                                                        c->d_bptr, c->d_bhe, c->d_bf, c->d_vol, db, c->d_part);
  CHEM_TRY(cudaGetLastError(), "k_chem_gather launch");
  if (!dev)
    CHEM_TRY(cudaMemcpyAsync(b, db, (size_t)nn * neqn * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
             "chem copy out");
  long long bad = 0;
  CHEM_TRY(cudaMemcpyAsync(&bad, c->d_count, sizeof(long long), cudaMemcpyDeviceToHost, c->stream), "chem count");
  CHEM_TRY(cudaStreamSynchronize(c->stream), "chem viscous residual");
  if (bad) {
    pcfd_set_last_error("pcfd_chem_viscous_residual: " + std::to_string(bad) +
                        " face(s) above every transport fit's temperature range");
    return PCFD_ERR_ARG;
  }
  return PCFD_OK;
}

PCFD_API int pcfd_chem_residual(pcfd_chem_t h, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o,
                                double ref_time, int reactions, const double* q, double* b, double* norms, int dev) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || !ref_ok(ref) || !o || !q || !(ref_time > 0.0)) {
    pcfd_set_last_error("pcfd_chem_residual: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (c->nnode <= 0) {
    pcfd_set_last_error("pcfd_chem_residual: no mesh attached (pcfd_chem_attach_mesh)");
    return PCFD_ERR_STATE;
  }
  const int ns = c->host.nspecies, neqn = ns + 4;
  const size_t nv = 6 + 3 * (size_t)ns;
  const long long nn = c->nnode, ne = c->nedge, nb = c->nbedge;
  const double* dq = q;
  if (!dev) {
    CHEM_TRY(cudaMemcpyAsync(c->d_q, q, (size_t)(nn + nb) * nv * sizeof(double), cudaMemcpyHostToDevice, c->stream),
             "chem copy");
    dq = c->d_q;
  }
  double* db = (dev && b) ? b : c->d_b;
  if (!c->d_count) CHEM_TRY(cudaMalloc(&c->d_count, sizeof(long long)), "chem buffers");
  CHEM_TRY(cudaMemsetAsync(c->d_count, 0, sizeof(long long), c->stream), "chem count");
  const pcfd_chem_ref r = *ref;
  const pcfd_chem_flux_opts oo = *o;
  if (ne > 0) {
    k_chem_hllc<<<CHEM_GRID(ne)>>>(ne, nn + nb, c->dev, c->dder, r, oo, dq, c->d_en, c->d_ea, c->d_ef, c->d_count);
    CHEM_TRY(cudaGetLastError(), "k_chem_hllc launch");
  }
  if (nb > 0) {
    k_chem_bflux<<<CHEM_GRID(nb)>>>(nb, c->dev, c->dder, r, oo, dq, c->d_bn, c->d_ba, c->d_bf, c->d_count);
    CHEM_TRY(cudaGetLastError(), "k_chem_bflux launch");
  }
  k_chem_gather<<<kChemNormBlocks, 256, 0, c->stream>>>(nn, c->dev, r, ref_time, reactions, dq, c->d_nptr, c->d_nedg,
                                                        c->d_ef, c->d_bptr, c->d_bhe, c->d_bf, c->d_vol, db,
                                                        c->d_part);
  CHEM_TRY(cudaGetLastError(), "k_chem_gather launch");
  k_chem_norms<<<1, 32 * neqn, 0, c->stream>>>(kChemNormBlocks, nn, neqn, c->d_part, c->d_norms);
  CHEM_TRY(cudaGetLastError(), "k_chem_norms launch");
  if (b && !dev)
    CHEM_TRY(cudaMemcpyAsync(b, db, (size_t)nn * neqn * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
             "chem copy out");
  if (norms)
    CHEM_TRY(cudaMemcpyAsync(norms, c->d_norms, (size_t)(1 + neqn) * sizeof(double), cudaMemcpyDeviceToHost,
                             c->stream),
             "chem copy out");
  long long bad = 0;
  CHEM_TRY(cudaMemcpyAsync(&bad, c->d_count, sizeof(long long), cudaMemcpyDeviceToHost, c->stream), "chem count");
  CHEM_TRY(cudaStreamSynchronize(c->stream), "chem residual");
  if (bad) {
    pcfd_set_last_error("pcfd_chem_residual: " + std::to_string(bad) + " face(s) with no HLLC branch");
    return PCFD_ERR_NUMERIC;
  }
  return PCFD_OK;
}

PCFD_API int pcfd_chem_residual_ho(pcfd_chem_t h, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o, double chi,
                                   double ref_time, int reactions, const double* q, const double* grad,
                                   const double* lim, double* b, double* norms, int dev) {
  ChemHandle* c = (ChemHandle*)h;
  if (!c || !ref_ok(ref) || !o || !q || !grad || !lim || !(ref_time > 0.0)) {
    pcfd_set_last_error("pcfd_chem_residual_ho: bad arguments");
    return PCFD_ERR_ARG;
  }
  if (c->nnode <= 0) {
    pcfd_set_last_error("pcfd_chem_residual_ho: no mesh attached (pcfd_chem_attach_mesh)");
    return PCFD_ERR_STATE;
  }
  if (!c->d_xyz) {
    pcfd_set_last_error("pcfd_chem_residual_ho: the attached mesh has no coordinates");
    return PCFD_ERR_STATE;
  }
  const int ns = c->host.nspecies, neqn = ns + 4;
  const size_t nv = 6 + 3 * (size_t)ns;
  const long long nn = c->nnode, ne = c->nedge, nb = c->nbedge;
  const double* dq = q;
  if (!dev) {
    CHEM_TRY(cudaMemcpyAsync(c->d_q, q, (size_t)(nn + nb) * nv * sizeof(double), cudaMemcpyHostToDevice, c->stream),
             "chem copy");
    dq = c->d_q;
  }
  const int nt = 2 * ns + 4;
  const double* dg = grad;
  const double* dl = lim;
  if (!dev) {
    if (!c->d_grad) CHEM_TRY(cudaMalloc(&c->d_grad, (size_t)nn * nt * 3 * sizeof(double)), "chem buffers");
    if (!c->d_lim) CHEM_TRY(cudaMalloc(&c->d_lim, (size_t)nn * neqn * sizeof(double)), "chem buffers");
    CHEM_TRY(cudaMemcpyAsync(c->d_grad, grad, (size_t)nn * nt * 3 * sizeof(double), cudaMemcpyHostToDevice,
                             c->stream),
             "chem copy");
    CHEM_TRY(cudaMemcpyAsync(c->d_lim, lim, (size_t)nn * neqn * sizeof(double), cudaMemcpyHostToDevice, c->stream),
             "chem copy");
    dg = c->d_grad;
    dl = c->d_lim;
  }
  double* db = (dev && b) ? b : c->d_b;
  if (!c->d_count) CHEM_TRY(cudaMalloc(&c->d_count, sizeof(long long)), "chem buffers");
  CHEM_TRY(cudaMemsetAsync(c->d_count, 0, sizeof(long long), c->stream), "chem count");
  const pcfd_chem_ref r = *ref;
  const pcfd_chem_flux_opts oo = *o;
  if (ne > 0) {
    k_chem_hllc2<<<CHEM_GRID(ne)>>>(ne, c->dev, c->dder, r, oo, chi, dq, dg, dl, c->d_xyz, c->d_en, c->d_ea, c->d_ef,
                                    c->d_count);
    CHEM_TRY(cudaGetLastError(), "k_chem_hllc2 launch");
  }
  if (nb > 0) {
    k_chem_bflux<<<CHEM_GRID(nb)>>>(nb, c->dev, c->dder, r, oo, dq, c->d_bn, c->d_ba, c->d_bf, c->d_count);
    CHEM_TRY(cudaGetLastError(), "k_chem_bflux launch");
  }
  k_chem_gather<<<kChemNormBlocks, 256, 0, c->stream>>>(nn, c->dev, r, ref_time, reactions, dq, c->d_nptr, c->d_nedg,
                                                        c->d_ef, c->d_bptr, c->d_bhe, c->d_bf, c->d_vol, db,
                                                        c->d_part);
  CHEM_TRY(cudaGetLastError(), "k_chem_gather launch");
  k_chem_norms<<<1, 32 * neqn, 0, c->stream>>>(kChemNormBlocks, nn, neqn, c->d_part, c->d_norms);
  CHEM_TRY(cudaGetLastError(), "k_chem_norms launch");
  if (b && !dev)
    CHEM_TRY(cudaMemcpyAsync(b, db, (size_t)nn * neqn * sizeof(double), cudaMemcpyDeviceToHost, c->stream),
             "chem copy out");
  if (norms)
    CHEM_TRY(cudaMemcpyAsync(norms, c->d_norms, (size_t)(1 + neqn) * sizeof(double), cudaMemcpyDeviceToHost,
                             c->stream),
             "chem copy out");
  long long bad = 0;
  CHEM_TRY(cudaMemcpyAsync(&bad, c->d_count, sizeof(long long), cudaMemcpyDeviceToHost, c->stream), "chem count");
  CHEM_TRY(cudaStreamSynchronize(c->stream), "chem residual");
  if (bad) {
    pcfd_set_last_error("pcfd_chem_residual_ho: " + std::to_string(bad) + " face(s) with no HLLC branch");
    return PCFD_ERR_NUMERIC;
  }
  return PCFD_OK;
}

}  // extern "C"
