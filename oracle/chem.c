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
