/*
 * CPU ORACLE - test infrastructure only.  Plain-C restatement of the
 * finite-rate chemistry production rates (pcfd_chem_* in include/pcfd.h):
 *   ChemModel<T>::GetMassProductionRates            ucs/chem.tcc:575
 *   Reaction<T>::GetForwardReactionRate             ucs/reaction.tcc:608
 *   Reaction<T>::GetEquilibriumReactionRate         ucs/reaction.tcc:629
 *   Reaction<T>::GetBackwardReactionRate            ucs/reaction.tcc:683
 *   Reaction<T>::Arrhenius/ModArrhenius/GuptaModArrhenius/PowerRxn
 *                                                   ucs/reaction.tcc:712-750
 *   Reaction<T>::GetMassProductionRate              ucs/reaction.tcc:763
 *   Species<T>::GetThermoCoeff                      ucs/species.tcc:96
 * Constants: UNIV_R (ucs/chem_constants.h:5), Pref = 101325 Pa
 * (ucs/reaction.tcc:665).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "oracle.h"

#define UNIV_R_ 8.31447215

/* NASA-7 coefficients for T: low set up to 1000 K, high set above; outside
 * 200..6000 K the end set is used with the unpinned T (the reference pins
 * only its local copy of T) */
static const double* thermo_coeff(const pcfd_chem_model* m, int s, double T) {
  if (T < 200.0) return m->nasa_lo[s];
  if (T > 6000.0) return m->nasa_hi[s];
  return T > 1000.0 ? m->nasa_hi[s] : m->nasa_lo[s];
}

double oracle_chem_kf(const pcfd_chem_reaction* r, double T) {
  switch (r->type) {
    case 0: return r->A * exp(-r->EA / (UNIV_R_ * T));
    case 1: return r->A * pow(T, r->n) * exp(-r->EA / (UNIV_R_ * T));
    case 2: return r->A * pow(T, r->n) * exp(-r->EA / T);
    case 3: return r->A * pow(T, r->n);
  }
  return -999.0;
}

static int whole(double v) { return v == floor(v); }

double oracle_chem_kc(const pcfd_chem_model* m, const pcfd_chem_reaction* r, double T) {
  double nu = 0.0, d[7] = {0, 0, 0, 0, 0, 0, 0};
  for (int i = 0; i < r->nlocal; i++) {
    const double* a = thermo_coeff(m, r->global[i], T);
    double dnu = r->nupp[i] - r->nup[i];
    nu += dnu;
    for (int k = 0; k < 7; k++) d[k] += dnu * a[k];
  }
  double Kp = exp(d[0] * (log(T) - 1.0) + T * (d[1] / 2.0 + T * (d[2] / 6.0 + T * (d[3] / 12.0 + d[4] / 20.0 * T))) -
                  d[5] / T + d[6]);
  double Kc = Kp;
  if (!(fabs(nu) < 1.0e-15)) {
    const double Pref = 101325.0;
    Kc *= pow(Pref / (UNIV_R_ * T), whole(nu) ? (double)(int)nu : nu);
  }
  return Kc;
}

/* wdot [nspecies] for one node */
void oracle_chem_rates(const pcfd_chem_model* m, const double* rhoi, double T, double* wdot) {
  double X[PCFD_CHEM_MAX_SPECIES];
  for (int k = 0; k < m->nspecies; k++) X[k] = rhoi[k] / m->mw[k];
  for (int i = 0; i < m->nspecies; i++) wdot[i] = 0.0;
  for (int i = 0; i < m->nspecies; i++) {
    for (int j = 0; j < m->nreactions; j++) {
      const pcfd_chem_reaction* r = &m->rx[j];
      int kk = -1;
      for (int l = 0; l < r->nlocal; l++)
        if (r->global[l] == i) { kk = l; break; }
      double nu_ir = kk >= 0 ? r->nupp[kk] - r->nup[kk] : 0.0;
      if (nu_ir == 0.0) continue;
      double Kf = oracle_chem_kf(r, T);
      double Kb = Kf / oracle_chem_kc(m, r, T);
      double form = 1.0, dest = 1.0;
      for (int l = 0; l < r->nlocal; l++) {
        double x = X[r->global[l]];
        double a = r->nup[l], b = r->nupp[l];
        form *= pow(x, whole(a) ? (double)(int)a : a);
        dest *= pow(x, whole(b) ? (double)(int)b : b);
      }
      double Mc = 1.0;
      if (r->third_bodies) {
        Mc = 0.0;
        for (int k = 0; k < m->nspecies; k++) Mc += X[k];
        for (int l = 0; l < r->nlocal; l++) Mc += (r->tbeff[l] - 1.0) * X[r->global[l]];
      }
      double net = Kf * form - Kb * dest;
      double w = nu_ir * Mc * net;
      w *= m->mw[i];
      wdot[i] += w;
    }
  }
}

void oracle_chem_rates_n(const pcfd_chem_model* m, long long n, const double* rhoi, const double* T, double* wdot) {
  for (long long p = 0; p < n; p++)
    oracle_chem_rates(m, rhoi + p * m->nspecies, T[p], wdot + p * m->nspecies);
}

/* ---- node state of the reacting equation set (ideal-gas mixture) ------- */

/* Species<T>::GetCp and GetH (ucs/species.tcc:43,56; href = 0, :327), J/kg */
static double species_cp(const pcfd_chem_model* m, int s, double T) {
  const double* a = thermo_coeff(m, s, T);
  double cp_R = a[0] + T * (a[1] + T * (a[2] + T * (a[3] + T * a[4])));
  return cp_R * (UNIV_R_ / m->mw[s]);
}
static double species_h(const pcfd_chem_model* m, int s, double T) {
  const double* a = thermo_coeff(m, s, T);
  double h_R = a[5] + T * (a[0] + T * (a[1] / 2.0 + T * (a[2] / 3.0 + T * (a[3] / 4.0 + T * a[4] / 5.0))));
  return h_R * (UNIV_R_ / m->mw[s]);
}
/* ChemModel::GetP (ucs/chem.tcc:989), Dalton's law over IdealGasEOS::GetP */
static double mix_P(const pcfd_chem_model* m, const double* rhoiDim, double T) {
  double P = 0.0;
  for (int i = 0; i < m->nspecies; i++) P += rhoiDim[i] * (UNIV_R_ / m->mw[i]) * T;
  return P;
}
/* ChemModel::GetSpecificEnthalpy (ucs/chem.tcc:586) */
static double mix_h(const pcfd_chem_model* m, const double* X, double T) {
  double h = 0.0;
  for (int i = 0; i < m->nspecies; i++) h += species_h(m, i, T) * X[i];
  return h;
}

/* CompressibleFREqnSet::NewtonFindTGivenP (ucs/compressibleFR.tcc:2343);
 * returns the iterations used (28 = not converged) */
int oracle_chem_find_T(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* rhoi, double P, double Tinit,
                       double* T) {
  const int maxit = 28;
  const double tol = 1.0e-15;
  double TDim = Tinit * ref->temperature;
  double PgoalDim = P * ref->pressure;
  double rhoiDim[PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < m->nspecies; i++) rhoiDim[i] = rhoi[i] * ref->density;
  int j;
  for (j = 0; j < maxit; j++) {
    double TpDim = TDim + 1.0e-8;
    double PDim = mix_P(m, rhoiDim, TDim);
    double PpDim = mix_P(m, rhoiDim, TpDim);
    double zpoint = PgoalDim - PDim;
    double zpointp = PgoalDim - PpDim;
    double dzdT = (zpointp - zpoint) / (TpDim - TDim);
    double dT = -zpoint / dzdT;
    if (fabs(dT / ref->temperature) < tol) break;
    TDim += dT;
  }
  *T = TDim / ref->temperature;
  return j;
}

/* ConservativeToNative (ucs/compressibleFR.tcc:2133); returns the
 * iterations used (20 = not converged, where the reference aborts) */
int oracle_chem_c2n(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* q, double P, double* native) {
  const int ns = m->nspecies, maxit = 20;
  const double tol = 1.0e-12;
  double rho = 0.0, R = 0.0;
  double Y[PCFD_CHEM_MAX_SPECIES], rhoiDim[PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < ns; i++) {
    rho += q[i];
    rhoiDim[i] = q[i] * ref->density;
    R += rhoiDim[i] * (UNIV_R_ / m->mw[i]);
  }
  R /= ref->density * rho;
  for (int i = 0; i < ns; i++) Y[i] = q[i] / rho;
  double u = q[ns] / rho, v = q[ns + 1] / rho, w = q[ns + 2] / rho;
  double v2 = u * u + v * v + w * w;
  double res = q[ns + 3] - 0.5 * v2 * rho;
  /* IdealGasEOS::GetT (ucs/EOS.tcc:22) from the stored pressure */
  double T = (P * ref->pressure) / ((rho * ref->density) * R) / ref->temperature;
  int j;
  for (j = 0; j < maxit; j++) {
    double Tp = T + 1.0e-8;
    double H = rho * (mix_h(m, Y, T * ref->temperature) / ref->specific_enthalpy);
    double Hp = rho * (mix_h(m, Y, Tp * ref->temperature) / ref->specific_enthalpy);
    double Pn = mix_P(m, rhoiDim, T * ref->temperature) / ref->pressure;
    double Pp = mix_P(m, rhoiDim, Tp * ref->temperature) / ref->pressure;
    double E = H - Pn, Ep = Hp - Pp;
    double zpoint = res - E, zpointp = res - Ep;
    double dzdT = (zpointp - zpoint) / (Tp - T);
    double dT = -zpoint / dzdT;
    T += dT;
    if (fabs(dT) < tol) break;
  }
  native[0] = u;
  native[1] = v;
  native[2] = w;
  native[3] = T;
  return j;
}

/* NativeToConservative (ucs/compressibleFR.tcc:2117) with GetTotalEnergy
 * (:1219): q = (rho u, rho v, rho w, rho Et) */
void oracle_chem_n2c(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* rhoi, const double* native,
                     double P, double* q) {
  const int ns = m->nspecies;
  double rho = 0.0, X[PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < ns; i++) rho += rhoi[i];
  for (int i = 0; i < ns; i++) X[i] = rhoi[i] / rho;
  double u = native[0], v = native[1], w = native[2], T = native[3];
  double v2 = u * u + v * v + w * w;
  double h = mix_h(m, X, T * ref->temperature) / ref->specific_enthalpy;
  double E = h * rho - P;
  q[0] = u * rho;
  q[1] = v * rho;
  q[2] = w * rho;
  q[3] = E + 0.5 * rho * v2;
}

/* ComputeAuxiliaryVariables (ucs/compressibleFR.tcc:755) */
void oracle_chem_aux(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* rhoi, double T, double* P,
                     double* cvi, double* mol) {
  const int ns = m->nspecies;
  double rho = 0.0, rhoiDim[PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < ns; i++) {
    rho += rhoi[i];
    rhoiDim[i] = rhoi[i] * ref->density;
  }
  double TDim = T * ref->temperature;
  double pDim = mix_P(m, rhoiDim, TDim);
  *P = pDim / ref->pressure;
  double s_ref = ref->velocity * ref->velocity / ref->temperature;
  for (int i = 0; i < ns; i++) {
    /* IdealGasEOS::GetCv (ucs/EOS.tcc:79): Mayer's relation with the species R */
    cvi[i] = (species_cp(m, i, TDim) - UNIV_R_ / m->mw[i]) / s_ref;
    mol[i] = rhoi[i] / m->mw[i] / 1000.0;
  }
}

/* the same over n nodes (q [n][ns+4], P [n], native [n][4]); returns the
 * number of nodes that used all 20 iterations */
long long oracle_chem_c2n_n(const pcfd_chem_model* m, const pcfd_chem_ref* ref, long long n, const double* q,
                            const double* P, double* native) {
  long long bad = 0;
  for (long long p = 0; p < n; p++)
    if (oracle_chem_c2n(m, ref, q + p * (m->nspecies + 4), P[p], native + p * 4) == 20) bad++;
  return bad;
}

/* ChemModel::GetFluidProperties (ucs/chem.tcc:545) through
 * CompressibleFREqnSet::GetFluidProperties (ucs/compressibleFR.tcc:1523):
 * the non-dimensional speed of sound squared of a node record */
static double fr_c2(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* rhoi, double T) {
  const int ns = m->nspecies;
  double rhoiDim[PCFD_CHEM_MAX_SPECIES], X[PCFD_CHEM_MAX_SPECIES];
  double Tdim = T * ref->temperature;
  double rho = 0.0, R = 0.0;
  for (int i = 0; i < ns; i++) rhoiDim[i] = rhoi[i] * ref->density;
  for (int i = 0; i < ns; i++) rho += rhoiDim[i];
  for (int i = 0; i < ns; i++) R += rhoiDim[i] * (UNIV_R_ / m->mw[i]);
  R /= rho;
  for (int i = 0; i < ns; i++) X[i] = rhoiDim[i] / rho;
  double cp = 0.0, cv = 0.0;
  for (int i = 0; i < ns; i++) cp += species_cp(m, i, Tdim) * X[i];
  for (int i = 0; i < ns; i++) cv += X[i] * (species_cp(m, i, Tdim) - UNIV_R_ / m->mw[i]);
  double gamma = cp / cv;
  double c2Dim = gamma * R * Tdim;
  return c2Dim / (ref->velocity * ref->velocity);
}

/* GetTotalEnthalpy (ucs/compressibleFR.tcc:1249) */
static double fr_Ht(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* Q) {
  const int ns = m->nspecies;
  double X[PCFD_CHEM_MAX_SPECIES];
  double T = Q[ns + 3], rho = Q[ns + 5], u = Q[ns], v = Q[ns + 1], w = Q[ns + 2];
  double v2 = u * u + v * v + w * w;
  for (int i = 0; i < ns; i++) X[i] = Q[i] / rho;
  double h = mix_h(m, X, T * ref->temperature) / ref->specific_enthalpy;
  return h * rho + 0.5 * rho * v2;
}

/* CompressibleFREqnSet::HLLCFlux (ucs/compressibleFR.tcc:301), vdotn = 0;
 * returns 1 when no branch applies (the reference's soft abort; flux = 0) */
int oracle_chem_hllc(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o,
                     const double* QL, const double* QR, const double* avec, double* flux) {
  const int ns = m->nspecies;
  const double beta = o->beta, Pref = o->pref;
  const double *rhoiL = QL, *rhoiR = QR;
  double uL = QL[ns], vL = QL[ns + 1], wL = QL[ns + 2], TL = QL[ns + 3], pL = QL[ns + 4], rhoL = QL[ns + 5];
  double uR = QR[ns], vR = QR[ns + 1], wR = QR[ns + 2], TR = QR[ns + 3], pR = QR[ns + 4], rhoR = QR[ns + 5];
  double pgL = pL - Pref, pgR = pR - Pref;
  double c2L = fr_c2(m, ref, rhoiL, TL), c2R = fr_c2(m, ref, rhoiR, TR);
  double ETL = fr_Ht(m, ref, QL) - pL, ETR = fr_Ht(m, ref, QR) - pR;
  double thetaL = uL * avec[0] + vL * avec[1] + wL * avec[2];
  double thetaR = uR * avec[0] + vR * avec[1] + wR * avec[2];
  /* Roe-averaged record (ComputeAuxiliaryVariables on it, :755) */
  double rho = sqrt(rhoL * rhoR);
  double sigma = rho / (rhoL + rho);
  double roe[6 + 3 * PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < ns; i++) roe[i] = rhoiL[i] + sigma * (rhoiR[i] - rhoiL[i]);
  double u = uL + sigma * (uR - uL), v = vL + sigma * (vR - vL), w = wL + sigma * (wR - wL);
  double T = TL + sigma * (TR - TL);
  double theta = u * avec[0] + v * avec[1] + w * avec[2];
  double c2 = fr_c2(m, ref, roe, T);
  double oneMBeta = 1.0 - beta;
  double thetaPrime = theta * (1.0 + beta) * 0.5;
  double cPrime = 0.5 * sqrt(theta * theta * (oneMBeta * oneMBeta) + 4.0 * beta * c2);
  double thetaLPrime = thetaL * (1.0 + beta) * 0.5, thetaRPrime = thetaR * (1.0 + beta) * 0.5;
  double cLPrime = 0.5 * sqrt(thetaL * thetaL * (oneMBeta * oneMBeta) + 4.0 * beta * c2L);
  double cRPrime = 0.5 * sqrt(thetaR * thetaR * (oneMBeta * oneMBeta) + 4.0 * beta * c2R);
  double eig5L = thetaLPrime - cLPrime, eig4R = thetaRPrime + cRPrime;
  double eig4 = thetaPrime + cPrime, eig5 = thetaPrime - cPrime;
  double SL = (eig5L < eig5) ? eig5L : eig5;
  double SR = (eig4R > eig4) ? eig4R : eig4;
  double SM = (pgR - pgL + rhoL * thetaL * (SL - thetaL) - rhoR * thetaR * (SR - thetaR)) /
              (rhoL * (SL - thetaL) - rhoR * (SR - thetaR));
  double Qf[PCFD_CHEM_MAX_SPECIES + 4], pStar = 0.0;
  int fail = 0;
  if (SL >= 0.0) {
    for (int i = 0; i < ns; i++) Qf[i] = rhoiL[i];
    Qf[ns] = rhoL * uL; Qf[ns + 1] = rhoL * vL; Qf[ns + 2] = rhoL * wL; Qf[ns + 3] = ETL;
    pStar = pgL;
    SM = thetaL;
  } else if (SR <= 0.0) {
    for (int i = 0; i < ns; i++) Qf[i] = rhoiR[i];
    Qf[ns] = rhoR * uR; Qf[ns + 1] = rhoR * vR; Qf[ns + 2] = rhoR * wR; Qf[ns + 3] = ETR;
    pStar = pgR;
    SM = thetaR;
  } else if (SL <= 0.0 && SM >= 0.0) {
    pStar = pgL + rhoL * (thetaL - SL) * (thetaL - SM);
    double omega = 1.0 / (SL - SM), const1 = SL - thetaL, const2 = pStar - pgL;
    for (int i = 0; i < ns; i++) Qf[i] = omega * const1 * rhoiL[i];
    Qf[ns] = omega * (const1 * rhoL * uL + const2 * avec[0]);
    Qf[ns + 1] = omega * (const1 * rhoL * vL + const2 * avec[1]);
    Qf[ns + 2] = omega * (const1 * rhoL * wL + const2 * avec[2]);
    Qf[ns + 3] = omega * (const1 * ETL - pgL * thetaL + (pStar * SM)) + Pref * (SM - thetaL) * omega;
  } else if (SM <= 0.0 && SR >= 0.0) {
    pStar = pgR + rhoR * (thetaR - SR) * (thetaR - SM);
    double omega = 1.0 / (SR - SM), const1 = SR - thetaR, const2 = pStar - pgR;
    for (int i = 0; i < ns; i++) Qf[i] = omega * const1 * rhoiR[i];
    Qf[ns] = omega * (const1 * rhoR * uR + const2 * avec[0]);
    Qf[ns + 1] = omega * (const1 * rhoR * vR + const2 * avec[1]);
    Qf[ns + 2] = omega * (const1 * rhoR * wR + const2 * avec[2]);
    Qf[ns + 3] = omega * (const1 * ETR - pgR * thetaR + (pStar * SM)) + Pref * (SM - thetaR) * omega;
  } else {
    fail = 1;
  }
  if (fail) {
    for (int i = 0; i < ns + 4; i++) flux[i] = 0.0;
    return 1;
  }
  double area = avec[3];
  double thetabar = SM;  /* theta - vdotn on a static grid */
  for (int i = 0; i < ns; i++) flux[i] = area * Qf[i] * SM;
  flux[ns] = area * (Qf[ns] * SM + pStar * avec[0]);
  flux[ns + 1] = area * (Qf[ns + 1] * SM + pStar * avec[1]);
  flux[ns + 2] = area * (Qf[ns + 2] * SM + pStar * avec[2]);
  flux[ns + 3] = area * (Qf[ns + 3] * SM + pStar * thetabar) + Pref * thetabar * area;
  if (o->symmetry2D >= 1 && o->symmetry2D <= 3) flux[ns + o->symmetry2D - 1] = 0.0;
  return 0;
}

/* the same over an edge list (q [nnode][6 + 3 ns], edges [E][2], avec
 * [E][4], flux [E][ns + 4]); returns the number of failed edges */
long long oracle_chem_hllc_n(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o,
                             const double* q, long long nedge, const int* edges, const double* avec, double* flux) {
  const int nv = 6 + 3 * m->nspecies;
  long long bad = 0;
  for (long long e = 0; e < nedge; e++)
    bad += oracle_chem_hllc(m, ref, o, q + (size_t)edges[2 * e] * nv, q + (size_t)edges[2 * e + 1] * nv,
                            avec + 4 * e, flux + e * (m->nspecies + 4));
  return bad;
}

/* SpatialResidual (ucs/residual.tcc:66) of the reacting equation set,
 * first order and inviscid: edge fluxes scattered as the Driver does (left
 * node -flux, right node +flux), boundary half-edges against their phantom
 * records (the Bdriver), then SourceTerm (ucs/compressibleFR.tcc:1276) with
 * the production rates made non-dimensional by ref_density / ref_time; the
 * norms of ComputeResiduals (ucs/residual.tcc:13, ParallelL2Norm). */
static void fr_aux_rec(const pcfd_chem_model* m, const pcfd_chem_ref* ref, double* Q);

/* With grad and lim (the second-order form, Kernel_Inviscid_Flux,
 * ucs/residual.tcc:192): each edge's two records are extrapolated to the
 * edge midpoint by CompressibleFREqnSet::ExtrapolateVariables
 * (ucs/compressibleFR.tcc:734), q + lim (chi/2 dQ + (1 - chi) grad.dx) on
 * rhoi, u, v, w, T with dx = (x_R - x_L)/2, and their auxiliary variables
 * recomputed; boundary half-edges keep their records (one partition). */
static void chem_residual(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o,
                          const pcfd_mesh_view* mv, const double* q, const double* grad, const double* lim,
                          double chi, double ref_time, int reactions, double* b, double* norms) {
  const int ns = m->nspecies, neqn = ns + 4, nv = 6 + 3 * ns, nt = 2 * ns + 4;
  const int nn = mv->nnode;
  double flux[PCFD_CHEM_MAX_SPECIES + 4];
  double QL[6 + 3 * PCFD_CHEM_MAX_SPECIES], QR[6 + 3 * PCFD_CHEM_MAX_SPECIES];
  for (size_t i = 0; i < (size_t)nn * neqn; i++) b[i] = 0.0;
  for (int e = 0; e < mv->nedge; e++) {
    int a = mv->edges[2 * e], c = mv->edges[2 * e + 1];
    const double* qa = q + (size_t)a * nv;
    const double* qc = q + (size_t)c * nv;
    if (grad) {
      double dx[3];
      for (int i = 0; i < 3; i++) dx[i] = 0.5 * (mv->xyz[3 * (size_t)c + i] - mv->xyz[3 * (size_t)a + i]);
      for (int i = 0; i < nv; i++) {
        QL[i] = qa[i];
        QR[i] = qc[i];
      }
      const double* gL = grad + (size_t)a * nt * 3;
      const double* gR = grad + (size_t)c * nt * 3;
      for (int j = 0; j < neqn; j++) {
        const double dQ = qc[j] - qa[j];
        const double cl = 0.5 * chi * dQ + (1.0 - chi) * (gL[3 * j] * dx[0] + gL[3 * j + 1] * dx[1] + gL[3 * j + 2] * dx[2]);
        const double cr = 0.5 * chi * (-dQ) +
                          (1.0 - chi) * (gR[3 * j] * (-dx[0]) + gR[3 * j + 1] * (-dx[1]) + gR[3 * j + 2] * (-dx[2]));
        QL[j] = qa[j] + cl * lim[(size_t)a * neqn + j];
        QR[j] = qc[j] + cr * lim[(size_t)c * neqn + j];
      }
      fr_aux_rec(m, ref, QL);
      fr_aux_rec(m, ref, QR);
      oracle_chem_hllc(m, ref, o, QL, QR, mv->edge_area + 4 * (size_t)e, flux);
    } else {
      oracle_chem_hllc(m, ref, o, qa, qc, mv->edge_area + 4 * (size_t)e, flux);
    }
    for (int i = 0; i < neqn; i++) b[(size_t)c * neqn + i] += flux[i];
    for (int i = 0; i < neqn; i++) b[(size_t)a * neqn + i] += -flux[i];
  }
  for (int k = 0; k < mv->nbedge; k++) {
    int a = mv->bedges[2 * k], c = mv->bedges[2 * k + 1];
    oracle_chem_hllc(m, ref, o, q + (size_t)a * nv, q + (size_t)c * nv, mv->bedge_area + 4 * (size_t)k, flux);
    for (int i = 0; i < neqn; i++) b[(size_t)a * neqn + i] += -flux[i];
  }
  if (reactions) {
    double rhoi[PCFD_CHEM_MAX_SPECIES], wdot[PCFD_CHEM_MAX_SPECIES];
    for (int n = 0; n < nn; n++) {
      const double* Q = q + (size_t)n * nv;
      double T = Q[ns + 3] * ref->temperature;
      for (int i = 0; i < ns; i++) rhoi[i] = Q[i] * ref->density;
      oracle_chem_rates(m, rhoi, T, wdot);
      for (int i = 0; i < ns; i++) {
        wdot[i] /= (ref->density / ref_time);
        b[(size_t)n * neqn + i] += mv->vol[n] * wdot[i];
      }
    }
  }
  if (norms) {
    double s = 0.0;
    for (size_t i = 0; i < (size_t)nn * neqn; i++) s += b[i] * b[i];
    norms[0] = sqrt(s) / (double)((size_t)nn * neqn);
    for (int j = 0; j < neqn; j++) {
      double t = 0.0;
      for (int i = 0; i < nn; i++) t += b[(size_t)i * neqn + j] * b[(size_t)i * neqn + j];
      norms[1 + j] = sqrt(t) / (double)nn;
    }
  }
}

void oracle_chem_residual(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o,
                          const pcfd_mesh_view* mv, const double* q, double ref_time, int reactions, double* b,
                          double* norms) {
  chem_residual(m, ref, o, mv, q, NULL, NULL, 0.0, ref_time, reactions, b, norms);
}

void oracle_chem_residual_ho(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o,
                             const pcfd_mesh_view* mv, const double* q, const double* grad, const double* lim,
                             double chi, double ref_time, int reactions, double* b, double* norms) {
  chem_residual(m, ref, o, mv, q, grad, lim, chi, ref_time, reactions, b, norms);
}

/* CompressibleFREqnSet::SourceTerm (ucs/compressibleFR.tcc:1276), reactions
 * on, no gravity: vol * wdot made non-dimensional by ref_density / ref_time
 * in the species rows, zero in the momentum and energy rows.  Reads rhoi and
 * T of the native record only. */
static void fr_source(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* Q, double vol,
                      double ref_time, double* source) {
  const int ns = m->nspecies;
  double rhoi[PCFD_CHEM_MAX_SPECIES], wdot[PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < ns + 4; i++) source[i] = 0.0;
  const double T = Q[ns + 3] * ref->temperature;
  for (int i = 0; i < ns; i++) rhoi[i] = Q[i] * ref->density;
  oracle_chem_rates(m, rhoi, T, wdot);
  for (int i = 0; i < ns; i++) {
    wdot[i] /= (ref->density / ref_time);
    source[i] = vol * wdot[i];
  }
}

/* EqnSet::SourceTermJacobian (ucs/eqnset.tcc:163) on one node record Q:
 * A[j*neqn + i] = (S_j(Q + h e_i) - S_j(Q)) / h, h = 1e-8, one column per
 * native value.  The reference recomputes the auxiliary values of the
 * perturbed record before each SourceTerm call; SourceTerm reads none of
 * them, so they are not formed here. */
void oracle_chem_source_jacobian(const pcfd_chem_model* m, const pcfd_chem_ref* ref, double ref_time,
                                 const double* Q, double vol, double* A) {
  const int ns = m->nspecies, neqn = ns + 4;
  const double h = 1.0e-8;
  double source[PCFD_CHEM_MAX_SPECIES + 4], sourceP[PCFD_CHEM_MAX_SPECIES + 4];
  double QP[PCFD_CHEM_MAX_SPECIES + 4];
  for (int k = 0; k < neqn * neqn; k++) A[k] = 0.0;
  fr_source(m, ref, Q, vol, ref_time, source);
  for (int i = 0; i < neqn; i++) {
    for (int k = 0; k < neqn; k++) QP[k] = Q[k];
    QP[i] += h;
    fr_source(m, ref, QP, vol, ref_time, sourceP);
    for (int j = 0; j < neqn; j++) A[j * neqn + i] = (sourceP[j] - source[j]) / h;
  }
}

void oracle_chem_source_jacobian_n(const pcfd_chem_model* m, const pcfd_chem_ref* ref, double ref_time, long long n,
                                   const double* q, const double* vol, double* A) {
  const int ns = m->nspecies, neqn = ns + 4, nv = 6 + 3 * ns;
  for (long long p = 0; p < n; p++)
    oracle_chem_source_jacobian(m, ref, ref_time, q + p * nv, vol[p], A + p * neqn * neqn);
}

/* CompressibleFREqnSet::GetFluidProperties (ucs/compressibleFR.tcc:1523)
 * over ChemModel::GetFluidProperties (ucs/chem.tcc:545): the mixture R and
 * the frozen speed of sound squared, non-dimensional */
static void fr_fluid_R_c2(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* rhoi, double T,
                          double* R, double* c2) {
  const int ns = m->nspecies;
  double rhoiDim[PCFD_CHEM_MAX_SPECIES], X[PCFD_CHEM_MAX_SPECIES];
  const double s_ref = ref->velocity * ref->velocity / ref->temperature;
  const double Tdim = T * ref->temperature;
  double rho = 0.0, RDim = 0.0, cp = 0.0, cv = 0.0;
  for (int i = 0; i < ns; i++) rhoiDim[i] = rhoi[i] * ref->density;
  for (int i = 0; i < ns; i++) rho += rhoiDim[i];
  for (int i = 0; i < ns; i++) RDim += rhoiDim[i] * (UNIV_R_ / m->mw[i]);
  RDim /= rho;
  for (int i = 0; i < ns; i++) X[i] = rhoiDim[i] / rho;
  for (int i = 0; i < ns; i++) cp += species_cp(m, i, Tdim) * X[i];
  for (int i = 0; i < ns; i++) cv += X[i] * (species_cp(m, i, Tdim) - UNIV_R_ / m->mw[i]);
  const double gamma = cp / cv;
  *R = RDim / s_ref;
  *c2 = (gamma * RDim * Tdim) / (ref->velocity * ref->velocity);
}

/* ChemModel::dEtdP_dEtdRhoi (ucs/chem.tcc:829) with dRmixdRhoi (:862), at
 * constant T (dimensional arguments); returns dEt/dP */
static double fr_dEt(const pcfd_chem_model* m, const double* rhoi, double T, double v2, double* dEtdRhoi) {
  const int ns = m->nspecies;
  const double hv2 = 0.5 * v2;
  double rhomix = 0.0, Rmix = 0.0;
  for (int i = 0; i < ns; i++) {
    rhomix += rhoi[i];
    Rmix += rhoi[i] * (UNIV_R_ / m->mw[i]);
  }
  Rmix /= rhomix;
  const double dPdrhomix = Rmix * T; /* IdealGasEOS::GetdP_dRho (ucs/EOS.tcc:60) */
  const double dPdRmix = rhomix * T; /* GetdP_dR (:54) */
  for (int i = 0; i < ns; i++) {
    double dR = (UNIV_R_ / m->mw[i]) * (rhomix - rhoi[i]) / (rhomix * rhomix);
    for (int j = 0; j < ns; j++) {
      if (j == i) continue;
      dR -= (UNIV_R_ / m->mw[j]) * rhoi[j] / (rhomix * rhomix);
    }
    dEtdRhoi[i] = hv2 + species_h(m, i, T) - (dPdrhomix + dPdRmix * dR);
  }
  double dEtdP = 0.0;
  const double dTdP = 1.0 / (rhomix * Rmix); /* GetdT_dP (:42) */
  for (int i = 0; i < ns; i++) dEtdP += rhoi[i] * species_cp(m, i, T) * dTdP;
  dEtdP -= 1.0;
  return dEtdP;
}

/* CompressibleFREqnSet::ContributeTemporalTerms (ucs/compressibleFR.tcc:1319)
 * on one node record Q (rhoi, u, v, w, T, P, rho, ...): adds vol/dt terms
 * times dq/dQ (conservative over native) with Gupta's beta preconditioning
 * on the temperature column into the block A [(ns+4)^2]. */
void oracle_chem_temporal(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* Q, double vol,
                          double cnp1, double dt, double dtau, double beta, int local_ts, double* A) {
  const int ns = m->nspecies, neqn = ns + 4;
  const int uloc = ns, vloc = ns + 1, wloc = ns + 2, tloc = ns + 3;
  double dEtdRhoi[PCFD_CHEM_MAX_SPECIES], rhoiDim[PCFD_CHEM_MAX_SPECIES], Yi[PCFD_CHEM_MAX_SPECIES];
  double thetaOBetai[PCFD_CHEM_MAX_SPECIES];
  const double vOverDt = local_ts ? cnp1 * vol / dt + vol / dtau : cnp1 * vol / dtau;
  const double rho = Q[ns + 5], T = Q[tloc], P = Q[ns + 4];
  const double u = Q[uloc], v = Q[vloc], w = Q[wloc];
  const double rvOverDt = rho * vOverDt;
  double v2 = u * u + v * v + w * w;
  double R, c2;
  fr_fluid_R_c2(m, ref, Q, T, &R, &c2);
  const double s_ref = ref->velocity * ref->velocity / ref->temperature;
  const double rhoDim = rho * ref->density;
  const double TDim = T * ref->temperature;
  v2 *= ref->velocity * ref->velocity;
  (void)P;
  for (int i = 0; i < ns; i++) {
    rhoiDim[i] = Q[i] * ref->density;
    Yi[i] = Q[i] / rho;
  }
  double dEtdP = fr_dEt(m, rhoiDim, TDim, v2, dEtdRhoi);
  const double ref_detdrho = ref->specific_enthalpy * ref->density / ref->density;
  for (int i = 0; i < ns; i++) dEtdRhoi[i] /= ref_detdrho;
  const double ref_detdP = ref->specific_enthalpy * ref->density / ref->pressure;
  dEtdP /= ref_detdP;
  double dPdT = rhoDim * (R * s_ref); /* IdealGasEOS::GetdP_dT (ucs/EOS.tcc:66) */
  dPdT /= (ref->pressure / ref->temperature);
  const double oneOBeta = 1.0 / beta, oneMbeta = 1.0 - beta;
  for (int i = 0; i < ns; i++) thetaOBetai[i] = (Yi[i] * oneMbeta / c2) * oneOBeta;
  for (int i = 0; i < ns; i++) {
    A[neqn * i + i] += vOverDt;
    A[neqn * i + tloc] += thetaOBetai[i] * vOverDt * dPdT;
  }
  const int mloc[3] = {uloc, vloc, wloc};
  const double vel[3] = {u, v, w};
  for (int d = 0; d < 3; d++) {
    double precond = 0.0;
    for (int j = 0; j < ns; j++) {
      A[neqn * mloc[d] + j] += vel[d] * vOverDt;
      precond += thetaOBetai[j] * vel[d];
    }
    A[neqn * mloc[d] + mloc[d]] += rvOverDt;
    A[neqn * mloc[d] + tloc] += precond * vOverDt * dPdT;
  }
  double precond = 0.0;
  for (int j = 0; j < ns; j++) {
    A[neqn * tloc + j] += dEtdRhoi[j] * vOverDt;
    precond += dEtdRhoi[j] * thetaOBetai[j];
  }
  A[neqn * tloc + uloc] += u * rvOverDt;
  A[neqn * tloc + vloc] += v * rvOverDt;
  A[neqn * tloc + wloc] += w * rvOverDt;
  precond += dEtdP * oneOBeta;
  A[neqn * tloc + tloc] += precond * vOverDt * dPdT;
}

void oracle_chem_temporal_n(const pcfd_chem_model* m, const pcfd_chem_ref* ref, long long n, const double* q,
                            const double* vol, const double* dtau, const double* beta, double cnp1, double dt,
                            int local_ts, double* A) {
  const int ns = m->nspecies, neqn = ns + 4, nv = 6 + 3 * ns;
  for (long long p = 0; p < n; p++)
    oracle_chem_temporal(m, ref, q + p * nv, vol[p], cnp1, dt, dtau[p], beta[p], local_ts, A + p * neqn * neqn);
}

/* ---- transport ------------------------------------------------------------
 * Species<T>::GetViscosity / GetThermalConductivity (ucs/species.tcc:393,430):
 * at or below 1000 K White's Sutherland forms with air's constants for every
 * species (ucs/species.tcc:13-22), above it the last NASA RP-1311 fit whose
 * range holds T, ln(y) = A ln T + B/T + C/T^2 + D, converted from micropoise
 * and microwatt/(cm K).  *err is set when no fit holds T (the reference
 * aborts). */
static double transport_fit(const double (*fit)[6], int nfit, double T, double conv, int* err) {
  int range = -1;
  for (int i = 0; i < nfit; i++)
    if (T >= fit[i][0] && T <= fit[i][1]) range = i;
  if (range < 0) {
    *err = 1;
    return 0.0;
  }
  const double* c = fit[range];
  const double ly = c[2] * log(T) + c[3] / T + c[4] / (T * T) + c[5];
  return exp(ly) * conv;
}

static double species_mu(const pcfd_chem_model* m, int s, double T, int* err) {
  if (T <= 1000.0) {
    const double mu0 = 1.716e-5, T0 = 273.0, S = 111.0;
    return mu0 * pow(T / T0, 1.5) * ((T0 + S) / (T + S));
  }
  return transport_fit((const double(*)[6])m->mu_fit[s], m->nmu[s], T, 1.0e-7, err);
}

static double species_k(const pcfd_chem_model* m, int s, double T, int* err) {
  if (T <= 1000.0) {
    const double k0 = 0.0241, T0 = 273.0, S = 194.0;
    return k0 * pow(T / T0, 1.5) * ((T0 + S) / (T + S));
  }
  return transport_fit((const double(*)[6])m->k_fit[s], m->nk[s], T, 1.0e-4, err);
}

/* ChemModel<T>::WilkesMixtureRule (ucs/chem.tcc:876) with
 * MassFractionToMoleFraction (:941): mole fractions from mass fractions, the
 * last one 1 - the sum of the others; the weights always use the species'
 * viscosities, whatever property is mixed. */
static double wilke(const pcfd_chem_model* m, const double* rhoi, const double* prop, double T, int* err) {
  const int ns = m->nspecies;
  double rho = 0.0, X[PCFD_CHEM_MAX_SPECIES], visc[PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < ns; i++) rho += rhoi[i];
  double summ = 0.0;
  for (int i = 0; i < ns; i++) {
    X[i] = (rhoi[i] / rho) / m->mw[i];
    summ += X[i];
  }
  for (int i = 0; i < ns; i++) X[i] /= summ;
  summ = 0.0;
  for (int i = 0; i < ns - 1; i++) summ += X[i];
  X[ns - 1] = 1.0 - summ;
  for (int i = 0; i < ns; i++) visc[i] = species_mu(m, i, T, err);
  const double sqrt8 = sqrt(8.0);
  double mix = 0.0;
  for (int i = 0; i < ns; i++) {
    double wi = 0.0;
    for (int j = 0; j < ns; j++) {
      const double temp = 1.0 + sqrt(visc[i] / visc[j]) * pow(m->mw[j] / m->mw[i], 0.25);
      const double phi = pow(1.0 + m->mw[i] / m->mw[j], -0.5) * temp * temp / sqrt8;
      wi += X[j] * phi;
    }
    mix += (X[i] / wi) * prop[i];
  }
  return mix;
}

/* CompressibleFREqnSet<T>::GetMolecularViscosity / GetThermalConductivity
 * (ucs/compressibleFR.tcc:1580,1590): non-dimensional rhoi and T in, the
 * mixture values over ref_viscosity and ref_k out.  Returns 1 when T is
 * above every fit's range. */
int oracle_chem_transport(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* rhoi, double T,
                          double* mu, double* k) {
  const int ns = m->nspecies;
  double rd[PCFD_CHEM_MAX_SPECIES], pm[PCFD_CHEM_MAX_SPECIES], pk[PCFD_CHEM_MAX_SPECIES];
  int err = 0;
  for (int i = 0; i < ns; i++) rd[i] = rhoi[i] * ref->density;
  const double Td = T * ref->temperature;
  for (int i = 0; i < ns; i++) {
    pm[i] = species_mu(m, i, Td, &err);
    pk[i] = species_k(m, i, Td, &err);
  }
  const double rv = ref->viscosity != 0.0 ? ref->viscosity : 1.0;
  const double rk = ref->conductivity != 0.0 ? ref->conductivity : 1.0;
  *mu = wilke(m, rd, pm, Td, &err) / rv;
  *k = wilke(m, rd, pk, Td, &err) / rk;
  return err;
}

long long oracle_chem_transport_n(const pcfd_chem_model* m, const pcfd_chem_ref* ref, long long n, const double* rhoi,
                                  const double* T, double* mu, double* k) {
  long long bad = 0;
  for (long long i = 0; i < n; i++)
    bad += oracle_chem_transport(m, ref, rhoi + (size_t)i * m->nspecies, T[i], mu + i, k + i);
  return bad;
}

/* ---- viscous flux ---------------------------------------------------------
 * CompressibleFREqnSet<T>::ViscousFlux (ucs/compressibleFR.tcc:551) on the
 * face state Q (native record: rhoi, u, v, w, T) with the face gradient g of
 * the reacting set's gradient list (rhoi, u, v, w, T, concentrations; three
 * entries each), laminar (no turbulent viscosity, so the turbulent
 * conductivity term vanishes), no species diffusion. */
static void fr_viscous_flux(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o,
                            double Re, const double* Q, const double* g, const double* avec, double* flux, int* err) {
  const int ns = m->nspecies, off = 3 * ns;
  const double ux = g[off + 0], uy = g[off + 1], uz = g[off + 2];
  const double vx = g[off + 3], vy = g[off + 4], vz = g[off + 5];
  const double wx = g[off + 6], wy = g[off + 7], wz = g[off + 8];
  const double Tx = g[off + 9], Ty = g[off + 10], Tz = g[off + 11];
  const double u = Q[ns], v = Q[ns + 1], w = Q[ns + 2];
  double mu, kc;
  *err |= oracle_chem_transport(m, ref, Q, Q[ns + 3], &mu, &kc);
  const double fact = 2.0 / 3.0;
  const double tauxx = 2.0 * fact * ux - fact * vy - fact * wz;
  const double tauyy = 2.0 * fact * vy - fact * ux - fact * wz;
  const double tauzz = 2.0 * fact * wz - fact * ux - fact * vy;
  const double tauxy = uy + vx, tauxz = uz + wx, tauyz = vz + wy;
  const double RK = avec[3] / Re, RKT = RK * mu;
  const double k = -kc;
  const double Tn = Tx * avec[0] + Ty * avec[1] + Tz * avec[2];
  const double tauxn = -tauxx * avec[0] - tauxy * avec[1] - tauxz * avec[2];
  const double tauyn = -tauxy * avec[0] - tauyy * avec[1] - tauyz * avec[2];
  const double tauzn = -tauxz * avec[0] - tauyz * avec[1] - tauzz * avec[2];
  for (int i = 0; i < ns; i++) flux[i] = 0.0;
  flux[ns + 0] = RKT * tauxn;
  flux[ns + 1] = RKT * tauyn;
  flux[ns + 2] = RKT * tauzn;
  flux[ns + 3] = RKT * (tauxn * u + tauyn * v + tauzn * w) + RK * k * Tn;
  if (o->symmetry2D >= 1 && o->symmetry2D <= 3) flux[ns + o->symmetry2D - 1] = 0.0;
}

/* Kernel_Viscous_Flux / Bkernel_Viscous_Flux (ucs/residual.tcc:390,473) of
 * the reacting set on one partition: the face state is the average of the
 * two native records; an interior face takes the average of the two nodes'
 * gradients, with the directional correction along the edge when
 * `directional` (second order past the first-order steps); a boundary face
 * takes its node's gradient.  b [nnode][ns + 4] receives the viscous part of
 * the residual alone (-F on the left node, +F on the right).  Returns the
 * number of faces whose temperature was above every transport fit. */
int oracle_chem_viscous_residual(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o,
                                 const pcfd_mesh_view* mv, double Re, int directional, const double* q,
                                 const double* grad, double* b) {
  const int ns = m->nspecies, neqn = ns + 4, nv = 6 + 3 * ns, nt = 2 * ns + 4;
  const int nn = mv->nnode;
  double Qa[PCFD_CHEM_MAX_SPECIES + 4], flux[PCFD_CHEM_MAX_SPECIES + 4], g[3 * (2 * PCFD_CHEM_MAX_SPECIES + 4)];
  int bad = 0;
  for (size_t i = 0; i < (size_t)nn * neqn; i++) b[i] = 0.0;
  for (int e = 0; e < mv->nedge; e++) {
    const int a = mv->edges[2 * e], c = mv->edges[2 * e + 1];
    const double* qL = q + (size_t)a * nv;
    const double* qR = q + (size_t)c * nv;
    for (int i = 0; i < neqn; i++) Qa[i] = (qL[i] + qR[i]) / 2.0;
    const double* gL = grad + (size_t)a * nt * 3;
    const double* gR = grad + (size_t)c * nt * 3;
    for (int i = 0; i < nt * 3; i++) g[i] = 0.5 * (gL[i] + gR[i]);
    if (directional) {
      const double* xL = mv->xyz + 3 * (size_t)a;
      const double* xR = mv->xyz + 3 * (size_t)c;
      double dx[3], s2 = 0.0;
      for (int i = 0; i < 3; i++) {
        dx[i] = xR[i] - xL[i];
        s2 += dx[i] * dx[i];
      }
      for (int j = 0; j < nt; j++) {
        const int loc = j < ns + 4 ? j : 2 * ns + 6 + (j - ns - 4);
        const double qdots = dx[0] * g[3 * j] + dx[1] * g[3 * j + 1] + dx[2] * g[3 * j + 2];
        const double dq = (qR[loc] - qL[loc] - qdots) / s2;
        for (int i = 0; i < 3; i++) g[3 * j + i] += dq * dx[i];
      }
    }
    int err = 0;
    fr_viscous_flux(m, ref, o, Re, Qa, g, mv->edge_area + 4 * (size_t)e, flux, &err);
    bad += err;
    for (int i = 0; i < neqn; i++) b[(size_t)c * neqn + i] += flux[i];
    for (int i = 0; i < neqn; i++) b[(size_t)a * neqn + i] += -flux[i];
  }
  for (int k = 0; k < mv->nbedge; k++) {
    const int a = mv->bedges[2 * k], c = mv->bedges[2 * k + 1];
    const double* qL = q + (size_t)a * nv;
    const double* qR = q + (size_t)c * nv;
    for (int i = 0; i < neqn; i++) Qa[i] = 0.5 * (qL[i] + qR[i]);
    int err = 0;
    fr_viscous_flux(m, ref, o, Re, Qa, grad + (size_t)a * nt * 3, mv->bedge_area + 4 * (size_t)k, flux, &err);
    bad += err;
    for (int i = 0; i < neqn; i++) b[(size_t)a * neqn + i] += -flux[i];
  }
  return bad;
}

/* Gradient<T>::Compute for the reacting set: Kernel_LSQ_Gradient (weighted
 * least squares, ucs/gradient.tcc:251) over the interior edges of the
 * gradient list of CompressibleFREqnSet::GetGradientsLocation
 * (ucs/compressibleFR.tcc:693: rhoi, u, v, w, T, concentrations), then
 * Bkernel_Symmetry_Fix (:545) on the half-edges whose tag is one of
 * sym_tags.  grad [nnode][2 ns + 4][3]. */
int oracle_chem_gradient(const pcfd_chem_model* m, const pcfd_mesh_view* mv, const double* q, const int* sym_tags,
                         int nsym, double* grad) {
  const int ns = m->nspecies, nv = 6 + 3 * ns, nt = 2 * ns + 4;
  const int nn = mv->nnode;
  memset(grad, 0, sizeof(double) * (size_t)nn * nt * 3);
  for (int e = 0; e < mv->nedge; e++) {
    const int l = mv->edges[2 * e], r = mv->edges[2 * e + 1];
    const double* xL = &mv->xyz[3 * (size_t)l];
    const double* xR = &mv->xyz[3 * (size_t)r];
    double dx[3] = {xL[0] - xR[0], xL[1] - xR[1], xL[2] - xR[2]};
    const double* qL = &q[(size_t)l * nv];
    const double* qR = &q[(size_t)r * nv];
    const double dx2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
    const double weight = 1.0 / sqrt(dx2);
    dx[0] *= weight;
    dx[1] *= weight;
    dx[2] *= weight;
    double weL[3], weR[3];
    oracle_lsq_coeff(&mv->sw[6 * (size_t)l], dx, weL);
    dx[0] = -dx[0];
    dx[1] = -dx[1];
    dx[2] = -dx[2];
    oracle_lsq_coeff(&mv->sw[6 * (size_t)r], dx, weR);
    for (int i = 0; i < nt; i++) {
      const int k = i < ns + 4 ? i : 2 * ns + 6 + (i - ns - 4);
      const double dq = weight * (qR[k] - qL[k]);
      for (int j = 0; j < 3; j++) {
        grad[(size_t)r * nt * 3 + 3 * i + j] += +weR[j] * dq;
        grad[(size_t)l * nt * 3 + 3 * i + j] += -weL[j] * dq;
      }
    }
  }
  for (int k = 0; k < mv->nbedge; k++) {
    int sym = 0;
    for (int t = 0; t < nsym; t++) sym |= mv->bfactag[k] == sym_tags[t];
    if (!sym) continue;
    const int l = mv->bedges[2 * k];
    const double* a = &mv->bedge_area[4 * (size_t)k];
    double* g = &grad[(size_t)l * nt * 3];
    for (int i = 0; i < nt; i++) {
      const double dot = g[3 * i] * a[0] + g[3 * i + 1] * a[1] + g[3 * i + 2] * a[2];
      for (int j = 0; j < 3; j++) g[3 * i + j] -= dot * a[j];
    }
  }
  return 0;
}

/* ---- boundary conditions ----------------------------------------------------
 * UpdateBCs (ucs/bc.tcc:1400) of the reacting set on one partition, half-edge
 * by half-edge in order, each through CalculateBoundaryVariables (:1059) and
 * then ComputeAuxiliaryVariables of the phantom and the node:
 *   sonic inflow, Dirichlet: node and phantom take the tag's reference record;
 *   sonic outflow, Neumann: the phantom copies the node's rhoi, u, v, w, T;
 *   no-slip, isothermal (twall > 0, K): GetViscousWallBoundaryVariables
 *     (ucs/compressibleFR.tcc:2049) with a resting wall: node and phantom
 *     take u = v = w = 0 and T = twall / ref_temperature, the phantom the
 *     node's rhoi;
 *   impermeable wall, symmetry with no characteristic condition (no_cvbc):
 *     GetInviscidWallBoundaryVariables (:1042), a static grid: the phantom is
 *     the node's record with the velocity mirrored in the face.
 * Other types (far field, the characteristic wall, the adiabatic no-slip
 * wall) are not restated: returns the first such half-edge + 1, else 0. */
static void fr_aux(const pcfd_chem_model* m, const pcfd_chem_ref* ref, double* Q) {
  const int ns = m->nspecies;
  double rho = 0.0;
  for (int i = 0; i < ns; i++) rho += Q[i];
  oracle_chem_aux(m, ref, Q, Q[ns + 3], &Q[ns + 4], &Q[ns + 6], &Q[2 * ns + 6]);
  Q[ns + 5] = rho;
}

int oracle_chem_update_bcs(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_mesh_view* mv, int ntags,
                           const int* bc_type, const double* twall, const double* qref, int no_cvbc, double* q) {
  const int ns = m->nspecies, neqn = ns + 4, nv = 6 + 3 * ns;
  for (int k = 0; k < mv->nbedge; k++) {
    const int tag = mv->bfactag[k];
    const int bt = (tag >= 0 && tag < ntags) ? bc_type[tag] : -1;
    double* QL = q + (size_t)mv->bedges[2 * k] * nv;
    double* QR = q + (size_t)mv->bedges[2 * k + 1] * nv;
    const double* a = &mv->bedge_area[4 * (size_t)k];
    if (bt == PCFD_BC_SONIC_INFLOW || bt == PCFD_BC_DIRICHLET) {
      for (int i = 0; i < nv; i++) QR[i] = QL[i] = qref[(size_t)tag * nv + i];
    } else if (bt == PCFD_BC_SONIC_OUTFLOW || bt == PCFD_BC_NEUMANN) {
      for (int i = 0; i < neqn; i++) QR[i] = QL[i];
    } else if (bt == PCFD_BC_NOSLIP && twall[tag] > 0.0) {
      for (int i = 0; i < ns; i++) QR[i] = QL[i];
      QR[ns + 3] = QL[ns + 3] = twall[tag] / ref->temperature;
      QR[ns] = QL[ns] = 0.0;
      QR[ns + 1] = QL[ns + 1] = 0.0;
      QR[ns + 2] = QL[ns + 2] = 0.0;
    } else if ((bt == PCFD_BC_IMPERMEABLE_WALL || bt == PCFD_BC_SYMMETRY) && no_cvbc) {
      double Qm[6 + 3 * PCFD_CHEM_MAX_SPECIES];
      for (int i = 0; i < nv; i++) Qm[i] = QL[i];
      fr_aux(m, ref, Qm);
      for (int i = 0; i < neqn; i++) QR[i] = Qm[i];
      const double dot = 2.0 * (Qm[ns] * a[0] + Qm[ns + 1] * a[1] + Qm[ns + 2] * a[2]);
      QR[ns] = Qm[ns] - dot * a[0];
      QR[ns + 1] = Qm[ns + 1] - dot * a[1];
      QR[ns + 2] = Qm[ns + 2] - dot * a[2];
    } else {
      return k + 1;
    }
    fr_aux(m, ref, QR);
    fr_aux(m, ref, QL);
  }
  return 0;
}

/* ComputeAuxiliaryVariables of one record in place */
static void fr_aux_rec(const pcfd_chem_model* m, const pcfd_chem_ref* ref, double* Q) { fr_aux(m, ref, Q); }

/* Limiter<T>::Compute (ucs/limiters.tcc:53) with the modified
 * Venkatakrishnan kernel (limiter = 3, Kernel_VenkatMod, :534, K = 1 as
 * hard-coded there) on the reacting set's native variables (rhoi, u, v, w,
 * T): neighbour bounds from 0 (Kernel_FindMinMax, :135), each edge end's
 * unlimited extrapolation (ExtrapolateVariables, ucs/compressibleFR.tcc:734),
 * the running minimum, negatives clamped to 0 (:118-124).  The pressure clip
 * (Kernel_PressureClip, :737) is not restated.  lim [nnode][ns + 4]. */
static void chem_limiter_raw(const pcfd_chem_model* m, const pcfd_mesh_view* mv, const double* q, const double* grad,
                             double chi, double* lim) {
  const int ns = m->nspecies, neqn = ns + 4, nv = 6 + 3 * ns, nt = 2 * ns + 4;
  const int nn = mv->nnode;
  double* qmin = (double*)calloc((size_t)nn * neqn, sizeof(double));
  double* qmax = (double*)calloc((size_t)nn * neqn, sizeof(double));
  for (size_t i = 0; i < (size_t)nn * neqn; i++) lim[i] = 1.0;
  for (int e = 0; e < mv->nedge; e++) {
    const int l = mv->edges[2 * e], r = mv->edges[2 * e + 1];
    for (int j = 0; j < neqn; j++) {
      const double vl = q[(size_t)l * nv + j], vr = q[(size_t)r * nv + j];
      double* xl = &qmax[(size_t)l * neqn + j];
      double* nl = &qmin[(size_t)l * neqn + j];
      double* xr = &qmax[(size_t)r * neqn + j];
      double* nr = &qmin[(size_t)r * neqn + j];
      *xl = *xl > vr ? *xl : vr;
      *nl = *nl < vr ? *nl : vr;
      *xr = *xr > vl ? *xr : vl;
      *nr = *nr < vl ? *nr : vl;
    }
  }
  const double Pi = 3.141592653589793, K3 = 1.0;
  for (int e = 0; e < mv->nedge; e++) {
    const int l = mv->edges[2 * e], r = mv->edges[2 * e + 1];
    const double* qL = &q[(size_t)l * nv];
    const double* qR = &q[(size_t)r * nv];
    double dx[3];
    for (int i = 0; i < 3; i++) dx[i] = 0.5 * (mv->xyz[3 * (size_t)r + i] - mv->xyz[3 * (size_t)l + i]);
    for (int side = 0; side < 2; side++) {
      const int a = side ? r : l;
      const double* qa = side ? qR : qL;
      const double* qb = side ? qL : qR;
      const double s = side ? -1.0 : 1.0;
      const double* g = &grad[(size_t)a * nt * 3];
      const double ep2 = (6.0 * Pi * mv->vol[a]) * K3;
      double DP = 0.0;
      for (int j = 0; j < neqn; j++) {
        const double dQ = qb[j] - qa[j];
        const double corr = 0.5 * chi * dQ + (1.0 - chi) * (g[3 * j] * (s * dx[0]) + g[3 * j + 1] * (s * dx[1]) +
                                                             g[3 * j + 2] * (s * dx[2]));
        const double Q = qa[j] + corr * 1.0;
        const double DM = Q - qa[j];
        if (Q > qa[j]) DP = qmax[(size_t)a * neqn + j] - qa[j];
        else if (Q < qa[j]) DP = qmin[(size_t)a * neqn + j] - qa[j];
        const double temp = (DP * DP + ep2 + 2.0 * DM * DP) / (DP * DP + 2.0 * DM * DM + DM * DP + ep2);
        double* lj = &lim[(size_t)a * neqn + j];
        if (temp < *lj) *lj = temp;
      }
    }
  }
  free(qmin);
  free(qmax);
}

/* the negative-limiter clamp at the end of Limiter<T>::Compute (:118-124) */
static void chem_limiter_clamp(const pcfd_chem_model* m, const pcfd_mesh_view* mv, double* lim) {
  const size_t n = (size_t)mv->nnode * (m->nspecies + 4);
  for (size_t i = 0; i < n; i++)
    if (lim[i] < 0.0) lim[i] = 0.0;
}

void oracle_chem_limiter(const pcfd_chem_model* m, const pcfd_mesh_view* mv, const double* q, const double* grad,
                         double chi, double* lim) {
  chem_limiter_raw(m, mv, q, grad, chi, lim);
  chem_limiter_clamp(m, mv, lim);
}

/* CompressibleFREqnSet::MaxEigenvalue (ucs/compressibleFR.tcc:1603) of a
 * record with current auxiliary variables: the mixture's frozen speed of
 * sound from GetFluidProperties (:1523; ChemModel::GetFluidProperties,
 * ucs/chem.tcc:545: c^2 = (cp / cv) R T with Dalton's R and the mass-fraction
 * weighted cp and cv = cp_i - R_i), and the acoustic eigenvalues modified by
 * Gupta's preconditioning parameter beta. */
static double fr_max_eigenvalue(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* Q,
                                const double* avec, double vdotn, double beta) {
  const int ns = m->nspecies;
  const double T = Q[ns + 3];
  double rhoiDim[PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < ns; i++) rhoiDim[i] = Q[i] * ref->density;
  const double Tdim = T * ref->temperature;
  double rho = 0.0, R = 0.0;
  for (int i = 0; i < ns; i++) rho += rhoiDim[i];
  for (int i = 0; i < ns; i++) R += rhoiDim[i] * (UNIV_R_ / m->mw[i]);
  R /= rho;
  double rhoX = 0.0, X[PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < ns; i++) rhoX += rhoiDim[i];
  for (int i = 0; i < ns; i++) X[i] = rhoiDim[i] / rhoX;
  double cp = 0.0, cv = 0.0;
  for (int i = 0; i < ns; i++) cp += species_cp(m, i, Tdim) * X[i];
  for (int i = 0; i < ns; i++) cv += X[i] * (species_cp(m, i, Tdim) - UNIV_R_ / m->mw[i]);
  const double gamma = cp / cv;
  const double c2 = (gamma * R * Tdim) / (ref->velocity * ref->velocity);
  const double theta = Q[ns] * avec[0] + Q[ns + 1] * avec[1] + Q[ns + 2] * avec[2] + vdotn;
  const double oneMBeta = 1.0 - beta;
  const double thetaPrime = theta * (1.0 + beta) * 0.5;
  const double cPrime = 0.5 * sqrt(theta * theta * (oneMBeta * oneMBeta) + 4.0 * beta * c2);
  const double e4 = fabs(thetaPrime + cPrime), e5 = fabs(thetaPrime - cPrime);
  return e4 > e5 ? e4 : e5;
}

/* ComputeTimesteps (ucs/timestep.tcc:7) of the reacting set with local time
 * stepping on a static mesh: each edge's averaged record (its auxiliary
 * variables recomputed) gives MaxEigenvalue x area to both ends
 * (Kernel_Timestep, :80), each boundary half-edge its own to its node
 * (Bkernel_Timestep, :115), summed in edge order, then half-edge order; dt =
 * cfl vol / sum.  beta is the preconditioning parameter of every node (the
 * reference fills its beta field with one value, ucs/solutionSpace.tcc:236-
 * 248).  q [nnode + nbedge][6 + 3 ns] -> dt [nnode]; returns the smallest. */
double oracle_chem_timestep(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_mesh_view* mv,
                            const double* q, double beta, double cfl, double* dt) {
  const int ns = m->nspecies, neqn = ns + 4, nv = 6 + 3 * ns;
  double Qa[6 + 3 * PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < mv->nnode; i++) dt[i] = 0.0;
  for (int e = 0; e < mv->nedge; e++) {
    const int l = mv->edges[2 * e], r = mv->edges[2 * e + 1];
    for (int j = 0; j < neqn; j++) Qa[j] = 0.5 * (q[(size_t)l * nv + j] + q[(size_t)r * nv + j]);
    fr_aux(m, ref, Qa);
    const double* a = &mv->edge_area[4 * (size_t)e];
    const double v = fr_max_eigenvalue(m, ref, Qa, a, 0.0, 0.5 * (beta + beta)) * a[3];
    dt[l] += v;
    dt[r] += v;
  }
  for (int k = 0; k < mv->nbedge; k++) {
    const int l = mv->bedges[2 * k], r = mv->bedges[2 * k + 1];
    for (int j = 0; j < neqn; j++) Qa[j] = 0.5 * (q[(size_t)l * nv + j] + q[(size_t)r * nv + j]);
    fr_aux(m, ref, Qa);
    const double* a = &mv->bedge_area[4 * (size_t)k];
    dt[l] += fr_max_eigenvalue(m, ref, Qa, a, 0.0, beta) * a[3];
  }
  double dtmin = 0.0;
  for (int i = 0; i < mv->nnode; i++) {
    dt[i] = cfl * (mv->vol[i] / dt[i]);
    if (i == 0 || dt[i] < dtmin) dtmin = dt[i];
  }
  return dtmin;
}

/* CompressibleFREqnSet::BadExtrapolation (ucs/compressibleFR.tcc:714) of a
 * record whose auxiliary variables are current: a negative species density,
 * a total energy (GetTotalEnergy, :1219) not above zero, a pressure or a
 * temperature below 1e-10. */
static int fr_bad_extrapolation(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* Q) {
  const int ns = m->nspecies;
  for (int i = 0; i < ns; i++)
    if (Q[i] < 0.0) return 1;
  const double T = Q[ns + 3], P = Q[ns + 4], rho = Q[ns + 5];
  double X[PCFD_CHEM_MAX_SPECIES];
  for (int i = 0; i < ns; i++) X[i] = Q[i] / rho;
  const double u = Q[ns], v = Q[ns + 1], w = Q[ns + 2];
  const double v2 = u * u + v * v + w * w;
  const double h = mix_h(m, X, T * ref->temperature) / ref->specific_enthalpy;
  const double Et = (h * rho - P) + 0.5 * rho * v2;
  if (Et <= 0.0) return 1;
  if (P < 1.0e-10) return 1;
  if (T < 1.0e-10) return 1;
  return 0;
}

/* Limiter<T>::Compute (ucs/limiters.tcc:53) of the reacting set with its
 * pressure clip: the raw modified Venkatakrishnan limiter as above, then
 * Kernel_PressureClip (:737) edge by edge in edge order - each end's record
 * extrapolated to the edge midpoint with its current limiter
 * (ExtrapolateVariables, ucs/compressibleFR.tcc:734), its auxiliary
 * variables recomputed, and the end's whole limiter zeroed when the state
 * fails BadExtrapolation - then negatives clamped to 0.  lim [nnode][ns + 4]. */
void oracle_chem_limiter_clip(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_mesh_view* mv,
                              const double* q, const double* grad, double chi, double* lim) {
  const int ns = m->nspecies, neqn = ns + 4, nv = 6 + 3 * ns, nt = 2 * ns + 4;
  chem_limiter_raw(m, mv, q, grad, chi, lim);
  double Qe[6 + 3 * PCFD_CHEM_MAX_SPECIES], dQ[PCFD_CHEM_MAX_SPECIES + 4];
  for (int e = 0; e < mv->nedge; e++) {
    const int l = mv->edges[2 * e], r = mv->edges[2 * e + 1];
    const double* xL = &mv->xyz[3 * (size_t)l];
    const double* xR = &mv->xyz[3 * (size_t)r];
    double dx[3] = {0.5 * (xR[0] - xL[0]), 0.5 * (xR[1] - xL[1]), 0.5 * (xR[2] - xL[2])};
    for (int j = 0; j < neqn; j++) dQ[j] = q[(size_t)r * nv + j] - q[(size_t)l * nv + j];
    for (int side = 0; side < 2; side++) {
      const int a = side ? r : l;
      if (side) {
        for (int i = 0; i < 3; i++) dx[i] = -dx[i];
        for (int j = 0; j < neqn; j++) dQ[j] = -dQ[j];
      }
      const double* qa = &q[(size_t)a * nv];
      const double* g = &grad[(size_t)a * nt * 3];
      double* la = &lim[(size_t)a * neqn];
      for (int j = 0; j < neqn; j++) {
        const double corr = 0.5 * chi * dQ[j] + (1.0 - chi) * (g[3 * j] * dx[0] + g[3 * j + 1] * dx[1] +
                                                                 g[3 * j + 2] * dx[2]);
        Qe[j] = qa[j] + corr * la[j];
      }
      fr_aux(m, ref, Qe);
      if (fr_bad_extrapolation(m, ref, Qe))
        for (int j = 0; j < neqn; j++) la[j] = 0.0;
    }
  }
  chem_limiter_clamp(m, mv, lim);
}
