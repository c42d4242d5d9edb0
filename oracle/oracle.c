/*
 * CPU ORACLE - test infrastructure only.
 *
 * A plain-C restatement of ProteusCFD's edge-based residual path, used by
 * tests/, __graft_entry__.smoke() and the cpu_baseline leg of bench.py to
 * check the CUDA implementation against.  It is never linked into, called
 * by or shipped with the product library.
 *
 * Pinning: the reference solver itself is built from its own sources by
 * oracle/refbuild (with stand-ins for MPI, HDF5 and METIS) and run on small
 * cases; tests/golden/ref_*.npz hold what it computed stage by stage (state
 * after the boundary update, gradient, limiter, residual and norms, Jacobian,
 * SGS update, Newton iterates).  tests/test_ref_oracle.py requires this file
 * to reproduce them.  The block LU, LuSolve and MatVecMult are also pinned
 * bit-for-bit against the reference's own ucs/matrix.h, and the dual metric
 * primitives against ucs/geometry.h (oracle/ref_pin.cpp).
 *
 * Layouts are the reference's: q [nnode+nbnode][10], qgrad [nnode][9][3],
 * limiter [nnode][5], b [nnode][5].
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#define NEQN 5
#define NVARS 10
#define NTERMS 9

static double dmax(double a, double b) { return (a > b) ? a : b; } /* MAX, ucs/macros.h:33 */
static double dmin(double a, double b) { return (a < b) ? a : b; } /* MIN, ucs/macros.h:39 */

/* ---------------------------------------------------------------------- */
/* ideal-gas equation set, ucs/compressible.tcc                            */
/* ---------------------------------------------------------------------- */

/* ComputeAuxiliaryVariables, ucs/compressible.tcc:1230 (T = gamma P / rho, :1104) */
void oracle_aux(double gamma, double* Q) {
  double gm1 = gamma - 1.0;
  double u = Q[1] / Q[0];
  double v = Q[2] / Q[0];
  double w = Q[3] / Q[0];
  double V2 = u * u + v * v + w * w;
  double P = gm1 * (Q[4] - 0.5 * Q[0] * V2);
  Q[6] = P;
  {
    /* ComputeTemperature -> ComputePressure recomputes P with v2h */
    double r = Q[0];
    double uu = Q[1] / r, vv = Q[2] / r, ww = Q[3] / r;
    double v2h = 0.5 * (uu * uu + vv * vv + ww * ww);
    double p = gm1 * (Q[4] - r * v2h);
    Q[5] = gamma * p / r;
  }
  Q[7] = u;
  Q[8] = v;
  Q[9] = w;
}

/* ComputePressure, ucs/compressible.tcc:1089 */
static double compute_pressure(const double* Q, double gamma) {
  double r = Q[0];
  double u = Q[1] / r, v = Q[2] / r, w = Q[3] / r;
  double E = Q[4];
  double v2h = 0.5 * (u * u + v * v + w * w);
  double gm1 = gamma - 1.0;
  return gm1 * (E - r * v2h);
}

/* UpdateQinf, ucs/compressible.tcc:827: rho = p gamma / T with p = T = 1. */
void oracle_qinf(const pcfd_params* prm, double* Qinf) {
  double gamma = prm->gamma, gm1 = gamma - 1.0;
  double T = prm->tinf == 0.0 ? 1.0 : prm->tinf;  /* ucs/compressible.tcc:835-837 */
  double p = prm->pinf == 0.0 ? 1.0 : prm->pinf;
  double rho = p * gamma / T;
  double V = prm->mach;
  double u = prm->flowdir[0] * V, v = prm->flowdir[1] * V, w = prm->flowdir[2] * V;
  double E = p / gm1 + 0.5 * rho * (u * u + v * v + w * w);
  Qinf[0] = rho;
  Qinf[1] = rho * u;
  Qinf[2] = rho * v;
  Qinf[3] = rho * w;
  Qinf[4] = E;
  oracle_aux(gamma, Qinf);
}

/* MatVecMult, ucs/matrix.h:63 */
void oracle_matvec(const double* a, const double* x, double* y, int n) {
  for (int i = 0; i < n; i++) {
    y[i] = a[i * n + 0] * x[0];
    for (int j = 1; j < n; j++) y[i] += a[i * n + j] * x[j];
  }
}

/* RoeVariables, ucs/compressible.tcc:533 */
static void roe_variables(const double* QL, const double* QR, double gamma, double* Qroe) {
  double gm1 = gamma - 1.0;
  double rhoL = QL[0], rhoR = QR[0];
  double uL = QL[1] / QL[0], uR = QR[1] / QR[0];
  double vL = QL[2] / QL[0], vR = QR[2] / QR[0];
  double wL = QL[3] / QL[0], wR = QR[3] / QR[0];
  double EL = QL[4], ER = QR[4];
  double v2L = uL * uL + vL * vL + wL * wL;
  double v2R = uR * uR + vR * vR + wR * wR;
  double PL = gm1 * (EL - 0.5 * rhoL * v2L);
  double PR = gm1 * (ER - 0.5 * rhoR * v2R);
  double hL = (EL + PL) / rhoL;
  double hR = (ER + PR) / rhoR;
  double rho = sqrt(rhoL * rhoR);
  double sigma = rho / (rhoL + rho);
  double u = uL + sigma * (uR - uL);
  double v = vL + sigma * (vR - vL);
  double w = wL + sigma * (wR - wL);
  double h = hL + sigma * (hR - hL);
  double v2h = 0.5 * (u * u + v * v + w * w);
  Qroe[0] = rho;
  Qroe[1] = rho * u;
  Qroe[2] = rho * v;
  Qroe[3] = rho * w;
  Qroe[4] = rho / gamma * (h + gm1 * v2h);
}

/* Eigensystem, ucs/compressible.tcc:580 (right/left eigenvectors, row-major 5x5) */
static void eigensystem(const double* Q, const double* avec, double vdotn, double gamma, double* eig,
                        double* T, double* Tinv) {
  double nx = avec[0], ny = avec[1], nz = avec[2];
  double rho = Q[0];
  double u = Q[1] / rho, v = Q[2] / rho, w = Q[3] / rho;
  double rE = Q[4];
  double gm1 = gamma - 1.0;
  double thetaf = u * nx + v * ny + w * nz;
  double theta = thetaf + vdotn;
  double v2h = 0.5 * (u * u + v * v + w * w);
  double P = gm1 * (rE - rho * v2h);
  double c2 = gamma * P / rho;
  double c = sqrt(c2);

  T[0] = nx; T[5] = u * nx; T[10] = v * nx + rho * nz; T[15] = w * nx - rho * ny;
  T[20] = v2h * nx + rho * (v * nz - w * ny);
  T[1] = ny; T[6] = u * ny - rho * nz; T[11] = v * ny; T[16] = w * ny + rho * nx;
  T[21] = v2h * ny + rho * (w * nx - u * nz);
  T[2] = nz; T[7] = u * nz + rho * ny; T[12] = v * nz - rho * nx; T[17] = w * nz;
  T[22] = v2h * nz + rho * (u * ny - v * nx);
  T[3] = rho / c; T[8] = rho * (u / c + nx); T[13] = rho * (v / c + ny); T[18] = rho * (w / c + nz);
  T[23] = rho * (v2h / c + thetaf + c / gm1);
  T[4] = rho / c; T[9] = rho * (u / c - nx); T[14] = rho * (v / c - ny); T[19] = rho * (w / c - nz);
  T[24] = rho * (v2h / c - thetaf + c / gm1);

  Tinv[0] = nx - nz * v / rho + ny * w / rho - nx / c2 * v2h * gm1;
  Tinv[1] = nx / c2 * u * gm1;
  Tinv[2] = nz / rho + nx / c2 * v * gm1;
  Tinv[3] = -ny / rho + nx / c2 * w * gm1;
  Tinv[4] = -nx / c2 * gm1;
  Tinv[5] = ny + nz * u / rho - nx * w / rho - ny / c2 * v2h * gm1;
  Tinv[6] = -nz / rho + ny / c2 * u * gm1;
  Tinv[7] = ny / c2 * v * gm1;
  Tinv[8] = nx / rho + ny / c2 * w * gm1;
  Tinv[9] = -ny / c2 * gm1;
  Tinv[10] = nz - ny * u / rho + nx * v / rho - nz / c2 * v2h * gm1;
  Tinv[11] = ny / rho + nz / c2 * u * gm1;
  Tinv[12] = -nx / rho + nz / c2 * v * gm1;
  Tinv[13] = nz / c2 * w * gm1;
  Tinv[14] = -nz / c2 * gm1;
  Tinv[15] = -0.5 / rho * (thetaf - gm1 * v2h / c);
  Tinv[16] = 0.5 / rho * (nx - gm1 * u / c);
  Tinv[17] = 0.5 / rho * (ny - gm1 * v / c);
  Tinv[18] = 0.5 / rho * (nz - gm1 * w / c);
  Tinv[19] = 0.5 / rho * (gm1 / c);
  Tinv[20] = 0.5 / rho * (thetaf + gm1 * v2h / c);
  Tinv[21] = -0.5 / rho * (nx + gm1 * u / c);
  Tinv[22] = -0.5 / rho * (ny + gm1 * v / c);
  Tinv[23] = -0.5 / rho * (nz + gm1 * w / c);
  Tinv[24] = +0.5 / rho * (gm1 / c);

  eig[0] = theta; eig[1] = theta; eig[2] = theta;
  eig[3] = theta + c;
  eig[4] = theta - c;
}

/* Flux, ucs/compressible.tcc:686 */
static void phys_flux(const double* Q, const double* avec, double vdotn, double gamma, double* f) {
  double rho = Q[0];
  double u = Q[1] / rho, v = Q[2] / rho, w = Q[3] / rho;
  double rEt = Q[4];
  double v2h = 0.5 * (u * u + v * v + w * w);
  double gm1 = gamma - 1.0;
  double P = gm1 * (rEt - rho * v2h);
  double ht = (rEt + P) / rho;
  double rhotheta = rho * (avec[0] * u + avec[1] * v + avec[2] * w + vdotn);
  f[0] = rhotheta;
  f[1] = (u * rhotheta + P * avec[0]);
  f[2] = (v * rhotheta + P * avec[1]);
  f[3] = (w * rhotheta + P * avec[2]);
  f[4] = (ht * rhotheta - vdotn * P);
}

/* Harten-Hyman entropy fix on one eigenvalue, ucs/compressible.tcc:148-185 */
static double entropy_fix(double eig, double eigL, double eigR) {
  double eps = dmax((eig - eigL), (eigR - eig));
  eps = dmax(0.0, eps);
  if (fabs(eig) < eps) return 0.5 * (eig * eig / eps + eps);
  return fabs(eig);
}

/* RoeFlux, ucs/compressible.tcc:93-230 */
void oracle_roe_flux(const double* QL, const double* QR, const double* avec, double vdotn, double gamma,
                     double* flux) {
  double Qroe[5], T[25], Tinv[25], ev[5], fL[5], fR[5], dQ[5], dv[5], dr[5];
  double area = avec[3];
  roe_variables(QL, QR, gamma, Qroe);
  eigensystem(Qroe, avec, vdotn, gamma, ev, T, Tinv);
  double gm1 = gamma - 1.0;
  double rhoL = QL[0], uL = QL[1] / rhoL, vL = QL[2] / rhoL, wL = QL[3] / rhoL, EL = QL[4];
  double PL = gm1 * (EL - 0.5 * rhoL * (uL * uL + vL * vL + wL * wL));
  double rhoR = QR[0], uR = QR[1] / rhoR, vR = QR[2] / rhoR, wR = QR[3] / rhoR, ER = QR[4];
  double PR = gm1 * (ER - 0.5 * rhoR * (uR * uR + vR * vR + wR * wR));
  double thetaL = uL * avec[0] + vL * avec[1] + wL * avec[2] + vdotn;
  double thetaR = uR * avec[0] + vR * avec[1] + wR * avec[2] + vdotn;
  double cR = sqrt(gamma * PR / rhoR);
  double cL = sqrt(gamma * PL / rhoL);
  double e0 = entropy_fix(ev[0], thetaL, thetaR);
  ev[0] = ev[1] = ev[2] = e0;
  ev[3] = entropy_fix(ev[3], thetaL + cL, thetaR + cR);
  ev[4] = entropy_fix(ev[4], thetaL - cL, thetaR - cR);
  for (int i = 0; i < 5; i++) dQ[i] = QR[i] - QL[i];
  oracle_matvec(Tinv, dQ, dv, 5);
  for (int i = 0; i < 5; i++) dv[i] *= fabs(ev[i]);
  oracle_matvec(T, dv, dr, 5);
  phys_flux(QL, avec, vdotn, gamma, fL);
  phys_flux(QR, avec, vdotn, gamma, fR);
  for (int i = 0; i < 5; i++) flux[i] = 0.5 * area * (fL[i] + fR[i] - dr[i]);
}

/* NumericalFlux NaN "kneecap", ucs/eqnset.tcc:73-88 */
static int kneecap(double* flux) {
  int bad = 0;
  for (int i = 0; i < NEQN; i++)
    if (isnan(flux[i])) { flux[i] = 0.0; bad = 1; }
  return bad;
}

/* ExtrapolateVariables + ExtrapolateCorrection, ucs/compressible.tcc:1039,
 * ucs/eqnset.h:231 */
static void extrapolate(double chi, double* Qho, const double* q, const double* dQedge, const double* gradQ,
                        const double* dx, const double* limiter) {
  for (int i = 0; i < NEQN; i++) {
    double corr = (0.5 * chi * dQedge[i] +
                   (1.0 - chi) * (gradQ[i * 3 + 0] * dx[0] + gradQ[i * 3 + 1] * dx[1] + gradQ[i * 3 + 2] * dx[2]));
    Qho[i] = q[i] + corr * limiter[i];
  }
}

/* Sutherland viscosity, EqnSet::ComputeViscosity (ucs/eqnset.h:251) */
static double viscosity(const pcfd_params* prm, const double* Q) {
  double T = Q[5];
  double S = 110.4 / prm->ref_temperature;
  return (1.0 + S) * pow(T, 1.5) / (T + S);
}

/* ViscousFlux, ucs/compressible.tcc:713 */
void oracle_viscous_flux(const pcfd_params* prm, const double* Q, const double* grad, const double* avec, double mut,
                         double* flux) {
  double Tx = grad[15], Ty = grad[16], Tz = grad[17];
  double ux = grad[18], uy = grad[19], uz = grad[20];
  double vx = grad[21], vy = grad[22], vz = grad[23];
  double wx = grad[24], wy = grad[25], wz = grad[26];
  double rho = Q[0];
  double u = Q[1] / rho, v = Q[2] / rho, w = Q[3] / rho;
  double mu = viscosity(prm, Q);
  double tmut = (mu + mut);
  double fact = -2.0 / 3.0 * (ux + vy + wz);
  double tauxx = 2.0 * ux + fact, tauyy = 2.0 * vy + fact, tauzz = 2.0 * wz + fact;
  double tauxy = uy + vx, tauxz = uz + wx, tauyz = vz + wy;
  double Mach = prm->mach;
  double ReTilde = prm->Re / Mach;
  double RK = avec[3] / ReTilde;
  double RKT = RK * tmut;
  double cp = 1.0 / (prm->gamma - 1.0);
  double k = mu / prm->Pr * cp;
  double kT = mut / prm->PrT * cp;
  double c1 = -(k + kT);
  double Tn = Tx * avec[0] + Ty * avec[1] + Tz * avec[2];
  double tauxn = tauxx * avec[0] + tauxy * avec[1] + tauxz * avec[2];
  double tauyn = tauxy * avec[0] + tauyy * avec[1] + tauyz * avec[2];
  double tauzn = tauxz * avec[0] + tauyz * avec[1] + tauzz * avec[2];
  flux[0] = 0.0;
  flux[1] = -RKT * (tauxn);
  flux[2] = -RKT * (tauyn);
  flux[3] = -RKT * (tauzn);
  flux[4] = -RKT * (tauxn * u + tauyn * v + tauzn * w) + RK * c1 * Tn;
}

/* ---------------------------------------------------------------------- */
/* boundary conditions, ucs/bc.tcc:1059 and ucs/compressible.tcc:1246-1575 */
/* ---------------------------------------------------------------------- */

/* GetFarfieldBoundaryVariables, ucs/compressible.tcc:1246 (static grid) */
static void bc_farfield(double gamma, double* QL, double* QR, const double* Qinf, const double* avec, double vdotn) {
  double tmp[NEQN];
  for (int subit = 0; subit < 10; subit++) {
    double u = vdotn * avec[0], v = vdotn * avec[1], w = vdotn * avec[2];
    for (int i = 0; i < NEQN; i++) tmp[i] = (QL[i] + QR[i]) / 2.0;
    double theta = tmp[1] / tmp[0] * avec[0] + tmp[2] / tmp[0] * avec[1] + tmp[3] / tmp[0] * avec[2] + vdotn;
    double rhob, ub, vb, wb, pb;
    double rhoi = QL[0];
    double ui = QL[1] / QL[0] + u, vi = QL[2] / QL[0] + v, wi = QL[3] / QL[0] + w;
    double pi = QL[6];
    double rhoinf = Qinf[0];
    double uinf = Qinf[1] / Qinf[0] + u, vinf = Qinf[2] / Qinf[0] + v, winf = Qinf[3] / Qinf[0] + w;
    double pinf = Qinf[6];
    double pavg = compute_pressure(tmp, gamma);
    double rhoavg = tmp[0];
    double c2avg = gamma * (pavg / rhoavg);
    double cavg = sqrt(c2avg);
    double nx = avec[0], ny = avec[1], nz = avec[2];
    if (theta == 0.0) {
      return;
    } else if (theta > 0.0 && fabs(theta / cavg) >= 1.0) {
      for (int i = 0; i < NEQN; i++) QR[i] = QL[i];
    } else if (theta < 0.0 && fabs(theta / cavg) >= 1.0) {
      for (int i = 0; i < NEQN; i++) QR[i] = Qinf[i];
    } else if (theta > 0.0 && fabs(theta / cavg) < 1.0) {
      pb = pinf;
      rhob = rhoi + (pb - pi) / c2avg;
      double t = (pb - pi) / (rhoavg * cavg);
      ub = ui - nx * t; vb = vi - ny * t; wb = wi - nz * t;
      QR[0] = rhob; QR[1] = rhob * ub; QR[2] = rhob * vb; QR[3] = rhob * wb;
      QR[4] = pb / (gamma - 1.0) + 0.5 * rhob * (ub * ub + vb * vb + wb * wb);
    } else if (theta < 0.0 && fabs(theta / cavg) < 1.0) {
      pb = 0.5 * (pinf + pi + rhoavg * cavg * (nx * (uinf - ui) + ny * (vinf - vi) + nz * (winf - wi)));
      rhob = rhoinf + (pb - pinf) / c2avg;
      double t = (pb - pinf) / (rhoavg * cavg);
      ub = uinf + nx * t; vb = vinf + ny * t; wb = winf + nz * t;
      QR[0] = rhob; QR[1] = rhob * ub; QR[2] = rhob * vb; QR[3] = rhob * wb;
      QR[4] = pb / (gamma - 1.0) + 0.5 * rhob * (ub * ub + vb * vb + wb * wb);
    } else {
      return;
    }
  }
}

/* GetInviscidWallBoundaryVariables, ucs/compressible.tcc:1375 (CVBC branch,
 * static grid: vdotn = 0 so the grid-speed terms vanish) */
static void bc_inviscid_wall(double gamma, int no_cvbc, double* QL, double* QR, const double* avec, double vdotn) {
  double tmp[NEQN], QLmod[NEQN];
  for (int subit = 0; subit < 10; subit++) {
    memcpy(QLmod, QL, sizeof(double) * NEQN);
    double u = vdotn * avec[0], v = vdotn * avec[1], w = vdotn * avec[2];
    double rhoi = QLmod[0];
    double ru = u * rhoi, rv = v * rhoi, rw = w * rhoi;
    QLmod[1] += ru; QLmod[2] += rv; QLmod[3] += rw;
    for (int i = 0; i < NEQN; i++) tmp[i] = (QL[i] + QR[i]) / 2.0;
    rhoi = QL[0];
    double ui = QL[1] / QL[0] + ru, vi = QL[2] / QL[0] + rv, wi = QL[3] / QL[0] + rw;
    double pi = QL[6];
    double rhoavg = tmp[0];
    tmp[1] += rhoavg * u; tmp[2] += rhoavg * v; tmp[3] += rhoavg * w;
    double pavg = compute_pressure(tmp, gamma);
    double c2avg = gamma * (pavg / rhoavg);
    double cavg = sqrt(c2avg);
    if (!no_cvbc) {
      double nx = avec[0], ny = avec[1], nz = avec[2];
      double thetaL = QL[1] / QL[0] * nx + QL[2] / QL[0] * ny + QL[3] / QL[0] * nz + vdotn;
      double pb = pi + rhoavg * cavg * thetaL;
      double rhob = rhoi + (pb - pi) / c2avg;
      double t = (pb - pi) / (rhoavg * cavg);
      double ub = ui - nx * t, vb = vi - ny * t, wb = wi - nz * t;
      QR[0] = rhob; QR[1] = rhob * ub; QR[2] = rhob * vb; QR[3] = rhob * wb;
      QR[4] = pb / (gamma - 1.0) + 0.5 * rhob * (ub * ub + vb * vb + wb * wb);
    } else {
      /* MirrorVector (ucs/geometry.h): v - 2 (v.n) n */
      for (int i = 0; i < NEQN; i++) QR[i] = QLmod[i];
      double dot = QLmod[1] * avec[0] + QLmod[2] * avec[1] + QLmod[3] * avec[2];
      QR[1] = QLmod[1] - 2.0 * dot * avec[0];
      QR[2] = QLmod[2] - 2.0 * dot * avec[1];
      QR[3] = QLmod[3] - 2.0 * dot * avec[2];
    }
  }
}

/* GetViscousWallBoundaryVariables, ucs/compressible.tcc:1545 (static wall) */
static void bc_viscous_wall(double gamma, double* QL, double* QR, const double* normalQ, double Twall) {
  double vel[3] = {0.0, 0.0, 0.0};
  if (Twall < 0.0) {
    QR[0] = QL[0] = normalQ[0];
    QR[4] = QL[4] = normalQ[4];
  } else {
    double v2 = vel[0] * vel[0] + vel[1] * vel[1] + vel[2] * vel[2];
    double gm1 = gamma - 1.0;
    double rhoEt = (Twall * QL[0] / (gamma * gm1) + 0.5 * QR[0] * v2);
    QR[0] = QL[0];
    QR[4] = QL[4] = rhoEt;
  }
  QR[1] = QL[1] = QL[0] * vel[0];
  QR[2] = QL[2] = QL[0] * vel[1];
  QR[3] = QL[3] = QL[0] * vel[2];
}

/* Most-normal neighbour of a wall node, ucs/bc.tcc:1184-1207 */
int oracle_normal_node(const pcfd_mesh_view* m, int node, const double* avec) {
  int normalNode = -1;
  double dotmax = 0.0;
  const double* wallx = &m->xyz[3 * node];
  for (int indx = m->ipsp[node]; indx < m->ipsp[node + 1]; indx++) {
    int pt = m->psp[indx];
    const double* ptx = &m->xyz[3 * pt];
    double dx[3] = {ptx[0] - wallx[0], ptx[1] - wallx[1], ptx[2] - wallx[2]};
    double mg = sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
    dx[0] = dx[0] / mg; dx[1] = dx[1] / mg; dx[2] = dx[2] / mg;
    double dot = 0.0;
    for (int i = 0; i < 3; i++) dot -= dx[i] * avec[i];
    if (dot >= dotmax) { normalNode = pt; dotmax = dot; }
  }
  return normalNode;
}

static int bc_of(const pcfd_params* prm, int factag) {
  if (factag < 0 || factag >= prm->ntags) return -1;
  return prm->bc_type[factag];
}

/* UpdateBCs -> BdriverNoScatter(BC_Kernel) -> CalculateBoundaryVariables,
 * ucs/bc.tcc:1400,724,1059: half-edges in order, each writes its phantom
 * state and may overwrite the boundary node's own q. */
int oracle_update_bcs(const pcfd_mesh_view* m, const pcfd_params* prm, double* q) {
  double Qinf[NVARS];
  oracle_qinf(prm, Qinf);
  const double gamma = prm->gamma;
  for (int eid = 0; eid < m->nbedge; eid++) {
    int l = m->bedges[2 * eid], r = m->bedges[2 * eid + 1];
    const double* avec = &m->bedge_area[4 * eid];
    double* QL = &q[(size_t)l * NVARS];
    double* QR = &q[(size_t)r * NVARS];
    int bct = bc_of(prm, m->bfactag[eid]);
    double vdotn = -(avec[0] * 0.0 + avec[1] * 0.0 + avec[2] * 0.0); /* static grid */
    switch (bct) {
      case PCFD_BC_SONIC_INFLOW:
      case PCFD_BC_DIRICHLET:
        for (int i = 0; i < NVARS; i++) QR[i] = QL[i] = Qinf[i];
        break;
      case PCFD_BC_SONIC_OUTFLOW:
      case PCFD_BC_NEUMANN:
        for (int i = 0; i < NEQN; i++) QR[i] = QL[i];
        break;
      case PCFD_BC_FARFIELD:
        bc_farfield(gamma, QL, QR, Qinf, avec, vdotn);
        break;
      case PCFD_BC_IMPERMEABLE_WALL:
      case PCFD_BC_SYMMETRY:
        bc_inviscid_wall(gamma, prm->no_cvbc, QL, QR, avec, vdotn);
        break;
      case PCFD_BC_NOSLIP: {
        int nn = oracle_normal_node(m, l, avec);
        double nQ[NVARS];
        memcpy(nQ, &q[(size_t)nn * NVARS], sizeof(nQ));
        double Tw = prm->bc_twall[m->bfactag[eid]] / prm->ref_temperature;
        bc_viscous_wall(gamma, QL, QR, nQ, Tw);
        break;
      }
      default:
        return -1;
    }
    oracle_aux(gamma, QR);
    oracle_aux(gamma, QL);
  }
  return 0;
}

/* ---------------------------------------------------------------------- */
/* gradient, ucs/gradient.tcc                                             */
/* ---------------------------------------------------------------------- */

/* ComputeLSQCoefficients, ucs/gradient.tcc:141 */
static void lsq_coeff(const double* s, const double* dxbar, double* we) {
  double s11 = s[0], s12 = s[1], s13 = s[2], s22 = s[3], s23 = s[4], s33 = s[5];
  double r11 = s11, r12 = s12, r13 = s13;
  double r12_r11 = (r11 == 0.0) ? 0.0 : r12 / r11;
  double r22 = s22 - r12 * r12_r11;
  double r23 = s23 - r12_r11 * r13;
  double r13_r11 = (r11 == 0.0) ? 0.0 : r13 / r11;
  double r23_r22 = (r22 == 0.0) ? 0.0 : r23 / r22;
  double r33 = s33 - r13 * r13_r11 - r23 * r23_r22;
  double dykdx = (dxbar[1] - (r12_r11)*dxbar[0]);
  we[2] = (r33 == 0.0) ? 0.0 : (dxbar[2] - r13_r11 * dxbar[0] - r23_r22 * dykdx) / r33;
  we[1] = (r22 == 0.0) ? 0.0 : (dykdx - r23 * we[2]) / r22;
  we[0] = (r11 == 0.0) ? 0.0 : (dxbar[0] - r12 * we[1] - r13 * we[2]) / r11;
}

void oracle_lsq_coeff(const double* s, const double* dxbar, double* we) { lsq_coeff(s, dxbar, we); }

static const int kGradList[NTERMS] = {0, 1, 2, 3, 4, 5, 7, 8, 9}; /* GetGradientsLocation, :1014 */

/* Gradient::Compute with Kernel_LSQ_Gradient (weighted), then
 * Bkernel_Symmetry_Fix; ucs/gradient.tcc:57,251,545 */
int oracle_gradient(const pcfd_mesh_view* m, const pcfd_params* prm, const double* q, double* grad) {
  const int nn = m->nnode;
  memset(grad, 0, sizeof(double) * (size_t)nn * NTERMS * 3);
  for (int e = 0; e < m->nedge; e++) {
    int l = m->edges[2 * e], r = m->edges[2 * e + 1];
    const double* xL = &m->xyz[3 * l];
    const double* xR = &m->xyz[3 * r];
    double dx[3] = {xL[0] - xR[0], xL[1] - xR[1], xL[2] - xR[2]};
    const double* qL = &q[(size_t)l * NVARS];
    const double* qR = &q[(size_t)r * NVARS];
    double dx2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
    double weight = 1.0 / sqrt(dx2);
    dx[0] *= weight; dx[1] *= weight; dx[2] *= weight;
    double weL[3], weR[3];
    lsq_coeff(&m->sw[6 * l], dx, weL);
    dx[0] = -dx[0]; dx[1] = -dx[1]; dx[2] = -dx[2];
    lsq_coeff(&m->sw[6 * r], dx, weR);
    double tL[NTERMS * 3], tR[NTERMS * 3];
    for (int i = 0; i < NTERMS; i++) {
      int k = kGradList[i];
      double dq = weight * (qR[k] - qL[k]);
      for (int j = 0; j < 3; j++) {
        tL[3 * i + j] = -weL[j] * dq;
        tR[3 * i + j] = +weR[j] * dq;
      }
    }
    for (int i = 0; i < NTERMS * 3; i++) grad[(size_t)r * NTERMS * 3 + i] += tR[i];
    for (int i = 0; i < NTERMS * 3; i++) grad[(size_t)l * NTERMS * 3 + i] += tL[i];
  }
  /* symmetry planes: remove the normal component, half-edge by half-edge */
  for (int eid = 0; eid < m->nbedge; eid++) {
    if (bc_of(prm, m->bfactag[eid]) != PCFD_BC_SYMMETRY) continue;
    int l = m->bedges[2 * eid];
    const double* avec = &m->bedge_area[4 * eid];
    double* g = &grad[(size_t)l * NTERMS * 3];
    for (int i = 0; i < NTERMS; i++) {
      double dot = g[i * 3 + 0] * avec[0] + g[i * 3 + 1] * avec[1] + g[i * 3 + 2] * avec[2];
      for (int j = 0; j < 3; j++) g[i * 3 + j] -= dot * avec[j];
    }
  }
  return 0;
}

/* ---------------------------------------------------------------------- */
/* limiter, ucs/limiters.tcc (limiter = 3, modified Venkatakrishnan)       */
/* ---------------------------------------------------------------------- */

static int bad_extrapolation(double gamma, const double* Q) { /* ucs/compressible.tcc:1056 */
  double r = Q[0];
  double u = Q[1] / r, v = Q[2] / r, w = Q[3] / r;
  double E = Q[4];
  double v2h = 0.5 * (u * u + v * v + w * w);
  double p = (gamma - 1.0) * (E - r * v2h);
  if (p < 1.0e-10) return 1;
  if (r < 0.0) return 1;
  if (E < 1.0e-10) return 1;
  return 0;
}

int oracle_limiter(const pcfd_mesh_view* m, const pcfd_params* prm, const double* q, const double* grad,
                   double* l, long long* nclip) {
  const int nn = m->nnode;
  const double chi = prm->chi;
  const double gamma = prm->gamma;
  for (size_t i = 0; i < (size_t)nn * NEQN; i++) l[i] = 1.0;
  if (nclip) *nclip = 0;
  if (prm->limiter == 0) return 0;
  if (prm->limiter < 1 || prm->limiter > 3) return -1;
  double* qmin = (double*)calloc((size_t)nn * NEQN, sizeof(double));
  double* qmax = (double*)calloc((size_t)nn * NEQN, sizeof(double));
  /* Kernel_FindMinMax, :135 (initialised to zero, quirk kept) */
  for (int e = 0; e < m->nedge; e++) {
    int a = m->edges[2 * e], b = m->edges[2 * e + 1];
    const double* qa = &q[(size_t)a * NVARS];
    const double* qb = &q[(size_t)b * NVARS];
    for (int i = 0; i < NEQN; i++) {
      qmax[a * NEQN + i] = dmax(qmax[a * NEQN + i], qb[i]);
      qmin[a * NEQN + i] = dmin(qmin[a * NEQN + i], qb[i]);
    }
    for (int i = 0; i < NEQN; i++) {
      qmax[b * NEQN + i] = dmax(qmax[b * NEQN + i], qa[i]);
      qmin[b * NEQN + i] = dmin(qmin[b * NEQN + i], qa[i]);
    }
  }
  if (prm->limiter == 1 || prm->limiter == 2) {
    /* Kernel_Barth, :194, and Kernel_Venkat, :372: the ratio of the allowed
     * to the extrapolated change, clamped to [0, 1] (Barth) or passed
     * through (t^2 + 2t)/(t^2 + t + 2) (Venkatakrishnan) */
    const double ones1[NEQN] = {1, 1, 1, 1, 1};
    for (int e = 0; e < m->nedge; e++) {
      int a = m->edges[2 * e], b = m->edges[2 * e + 1];
      const double* qL = &q[(size_t)a * NVARS];
      const double* qR = &q[(size_t)b * NVARS];
      const double* xL = &m->xyz[3 * a];
      const double* xR = &m->xyz[3 * b];
      double QL[NEQN], QR[NEQN], dx[3], dQ[NEQN];
      for (int i = 0; i < NEQN; i++) dQ[i] = qR[i] - qL[i];
      dx[0] = 0.5 * (xR[0] - xL[0]); dx[1] = 0.5 * (xR[1] - xL[1]); dx[2] = 0.5 * (xR[2] - xL[2]);
      extrapolate(chi, QL, qL, dQ, &grad[(size_t)a * NTERMS * 3], dx, ones1);
      dx[0] = -dx[0]; dx[1] = -dx[1]; dx[2] = -dx[2];
      for (int i = 0; i < NEQN; i++) dQ[i] = -dQ[i];
      extrapolate(chi, QR, qR, dQ, &grad[(size_t)b * NTERMS * 3], dx, ones1);
      for (int side = 0; side < 2; side++) {
        const int nd = side ? b : a;
        const double* qs = side ? qR : qL;
        const double* Qs = side ? QR : QL;
        for (int j = 0; j < NEQN; j++) {
          double temp = 1.0;
          if (Qs[j] > qs[j]) temp = (qmax[nd * NEQN + j] - qs[j]) / (Qs[j] - qs[j]);
          else if (Qs[j] < qs[j]) temp = (qmin[nd * NEQN + j] - qs[j]) / (Qs[j] - qs[j]);
          if (prm->limiter == 1) {
            temp = dmax(0.0, temp);
            temp = dmin(1.0, temp);
          } else {
            temp = (temp * temp + 2.0 * temp) / (temp * temp + temp + 2.0);
          }
          l[nd * NEQN + j] = dmin(l[nd * NEQN + j], temp);
        }
      }
    }
    goto clip;
  }
  {
  /* Kernel_VenkatMod, :534 */
  const double Pi = 3.141592653589793;
  const double K = prm->venkat_K;
  const double K3 = K * K * K;
  const double ones[NEQN] = {1, 1, 1, 1, 1};
  for (int e = 0; e < m->nedge; e++) {
    int a = m->edges[2 * e], b = m->edges[2 * e + 1];
    const double* qL = &q[(size_t)a * NVARS];
    const double* qR = &q[(size_t)b * NVARS];
    const double* xL = &m->xyz[3 * a];
    const double* xR = &m->xyz[3 * b];
    double QL[NEQN], QR[NEQN], dx[3], dQ[NEQN];
    double Ll3 = 6.0 * Pi * m->vol[a];
    double Lr3 = 6.0 * Pi * m->vol[b];
    dx[0] = 0.5 * (xR[0] - xL[0]); dx[1] = 0.5 * (xR[1] - xL[1]); dx[2] = 0.5 * (xR[2] - xL[2]);
    for (int i = 0; i < NEQN; i++) dQ[i] = qR[i] - qL[i];
    extrapolate(chi, QL, qL, dQ, &grad[(size_t)a * NTERMS * 3], dx, ones);
    dx[0] = -dx[0]; dx[1] = -dx[1]; dx[2] = -dx[2];
    for (int i = 0; i < NEQN; i++) dQ[i] = -dQ[i];
    extrapolate(chi, QR, qR, dQ, &grad[(size_t)b * NTERMS * 3], dx, ones);
    double DP = 0.0, DM;
    for (int j = 0; j < NEQN; j++) {
      DM = QL[j] - qL[j];
      if (QL[j] > qL[j]) DP = qmax[a * NEQN + j] - qL[j];
      else if (QL[j] < qL[j]) DP = qmin[a * NEQN + j] - qL[j];
      double ep2 = Ll3 * K3;
      double t = (DP * DP + ep2 + 2.0 * DM * DP) / (DP * DP + 2.0 * DM * DM + DM * DP + ep2);
      l[a * NEQN + j] = dmin(l[a * NEQN + j], t);
    }
    for (int j = 0; j < NEQN; j++) {
      DM = QR[j] - qR[j];
      if (QR[j] > qR[j]) DP = qmax[b * NEQN + j] - qR[j];
      if (QR[j] <= qR[j]) DP = qmin[b * NEQN + j] - qR[j];
      double ep2 = Lr3 * K3;
      double t = (DP * DP + ep2 + 2.0 * DM * DP) / (DP * DP + 2.0 * DM * DM + DM * DP + ep2);
      l[b * NEQN + j] = dmin(l[b * NEQN + j], t);
    }
  }
  }
clip:;
  /* Kernel_PressureClip, :737: sequential over edges as in the reference */
  long long clips = 0;
  for (int e = 0; e < m->nedge; e++) {
    int a = m->edges[2 * e], b = m->edges[2 * e + 1];
    const double* qL = &q[(size_t)a * NVARS];
    const double* qR = &q[(size_t)b * NVARS];
    const double* xL = &m->xyz[3 * a];
    const double* xR = &m->xyz[3 * b];
    double QL[NVARS], QR[NVARS], Qroe[NVARS], dx[3], dQ[NEQN];
    dx[0] = 0.5 * (xR[0] - xL[0]); dx[1] = 0.5 * (xR[1] - xL[1]); dx[2] = 0.5 * (xR[2] - xL[2]);
    for (int j = 0; j < NEQN; j++) dQ[j] = qR[j] - qL[j];
    extrapolate(chi, QL, qL, dQ, &grad[(size_t)a * NTERMS * 3], dx, &l[a * NEQN]);
    if (bad_extrapolation(gamma, QL)) { for (int i = 0; i < NEQN; i++) l[a * NEQN + i] = 0.0; clips++; }
    dx[0] = -dx[0]; dx[1] = -dx[1]; dx[2] = -dx[2];
    for (int j = 0; j < NEQN; j++) dQ[j] = -dQ[j];
    extrapolate(chi, QR, qR, dQ, &grad[(size_t)b * NTERMS * 3], dx, &l[b * NEQN]);
    if (bad_extrapolation(gamma, QR)) { for (int i = 0; i < NEQN; i++) l[b * NEQN + i] = 0.0; clips++; }
    roe_variables(QL, QR, gamma, Qroe);
    if (bad_extrapolation(gamma, Qroe)) {
      for (int i = 0; i < NEQN; i++) l[a * NEQN + i] = l[b * NEQN + i] = 0.0;
      clips++;
    }
  }
  for (size_t i = 0; i < (size_t)nn * NEQN; i++)
    if (l[i] < 0.0) l[i] = 0.0;
  if (nclip) *nclip = clips;
  free(qmin);
  free(qmax);
  return 0;
}

/* ---------------------------------------------------------------------- */
/* residual, ucs/residual.tcc                                              */
/* ---------------------------------------------------------------------- */

/* SpatialResidual + ComputeResiduals (ucs/residual.tcc:66,13): interior
 * inviscid edges, boundary inviscid half-edges, then (if viscous) interior
 * and boundary viscous, each Driver loop in order; then the no-slip residual
 * hook and the norms. */
int oracle_residual(const pcfd_mesh_view* m, const pcfd_params* prm, const double* q, const double* grad,
                    const double* lim, double* b, double* norms, long long* nkneecap) {
  return oracle_residual_scaled(m, prm, q, grad, lim, b, NULL, norms, nkneecap);
}

/* As oracle_residual; babs (optional) receives, per node and equation, the
 * sum of the absolute values of the terms added into b - the scale against
 * which the rounding of b is judged. */
int oracle_residual_scaled(const pcfd_mesh_view* m, const pcfd_params* prm, const double* q, const double* grad,
                           const double* lim, double* b, double* babs, double* norms, long long* nkneecap) {
  return oracle_residual_full(m, prm, q, NULL, grad, lim, b, babs, norms, nkneecap);
}

/* Param::dt as the temporal residual reads it: <= 0 is steady (0 stands for
 * the reference's default, -1.0). */
static double param_time_step(const pcfd_params* prm) {
  return prm->time_step == 0.0 ? -1.0 : prm->time_step;
}

/* ComputeResiduals (ucs/residual.tcc:13): SpatialResidual, then, when qold
 * ([nnode][5], the conservative state at the start of the step) is given and
 * Param::torder is set, TemporalResidual (:125) with Param::dt - for a steady
 * run (dt = -1) b += vol (q - qold), non-zero where the boundary update
 * overwrote a node's state - then the boundary hook and the norms. */
int oracle_residual_full(const pcfd_mesh_view* m, const pcfd_params* prm, const double* q, const double* qold,
                         const double* grad, const double* lim, double* b, double* babs, double* norms,
                         long long* nkneecap) {
  const int nn = m->nnode;
  const double gamma = prm->gamma, chi = prm->chi;
  const int ho = prm->sorder > 1;
  long long kc = 0;
  memset(b, 0, sizeof(double) * (size_t)nn * NEQN);
  if (babs) memset(babs, 0, sizeof(double) * (size_t)nn * NEQN);
#define ACCUM_ABS(node, f)                                                            \
  do {                                                                                \
    if (babs)                                                                         \
      for (int i_ = 0; i_ < NEQN; i_++) babs[(size_t)(node) * NEQN + i_] += fabs((f)[i_]); \
  } while (0)
  /* Kernel_Inviscid_Flux, :192 */
  for (int e = 0; e < m->nedge; e++) {
    int a = m->edges[2 * e], c = m->edges[2 * e + 1];
    const double* avec = &m->edge_area[4 * e];
    const double* qL = &q[(size_t)a * NVARS];
    const double* qR = &q[(size_t)c * NVARS];
    double QL[NVARS], QR[NVARS], dQ[NEQN], dx[3], flux[NEQN];
    memcpy(QL, qL, sizeof(QL));
    memcpy(QR, qR, sizeof(QR));
    double vdotn = -(avec[0] * 0.0 + avec[1] * 0.0 + avec[2] * 0.0);
    if (ho) {
      const double* xL = &m->xyz[3 * a];
      const double* xR = &m->xyz[3 * c];
      dx[0] = 0.5 * (xR[0] - xL[0]); dx[1] = 0.5 * (xR[1] - xL[1]); dx[2] = 0.5 * (xR[2] - xL[2]);
      for (int j = 0; j < NEQN; j++) dQ[j] = qR[j] - qL[j];
      extrapolate(chi, QL, qL, dQ, &grad[(size_t)a * NTERMS * 3], dx, &lim[a * NEQN]);
      for (int j = 0; j < NEQN; j++) dQ[j] = -dQ[j];
      dx[0] = -dx[0]; dx[1] = -dx[1]; dx[2] = -dx[2];
      extrapolate(chi, QR, qR, dQ, &grad[(size_t)c * NTERMS * 3], dx, &lim[c * NEQN]);
      oracle_aux(gamma, QL);
      oracle_aux(gamma, QR);
    }
    oracle_roe_flux(QL, QR, avec, vdotn, gamma, flux);
    kc += kneecap(flux);
    for (int i = 0; i < NEQN; i++) b[(size_t)c * NEQN + i] += flux[i];
    for (int i = 0; i < NEQN; i++) b[(size_t)a * NEQN + i] += -flux[i];
    ACCUM_ABS(c, flux);
    ACCUM_ABS(a, flux);
  }
  /* Bkernel_Inviscid_Flux, :299 (no extrapolation toward phantom nodes) */
  for (int eid = 0; eid < m->nbedge; eid++) {
    int a = m->bedges[2 * eid], c = m->bedges[2 * eid + 1];
    const double* avec = &m->bedge_area[4 * eid];
    double QL[NVARS], QR[NVARS], flux[NEQN];
    memcpy(QL, &q[(size_t)a * NVARS], sizeof(QL));
    memcpy(QR, &q[(size_t)c * NVARS], sizeof(QR));
    double vdotn = -(avec[0] * 0.0 + avec[1] * 0.0 + avec[2] * 0.0);
    if (ho) {
      oracle_aux(gamma, QL);
      oracle_aux(gamma, QR);
    }
    oracle_roe_flux(QL, QR, avec, vdotn, gamma, flux);
    kc += kneecap(flux); /* BoundaryFlux -> NumericalFlux kneecap */
    for (int i = 0; i < NEQN; i++) b[(size_t)a * NEQN + i] += -flux[i];
    ACCUM_ABS(a, flux);
  }
  if (prm->viscous) {
    /* Kernel_Viscous_Flux, :390 (laminar: mut = 0) */
    for (int e = 0; e < m->nedge; e++) {
      int a = m->edges[2 * e], c = m->edges[2 * e + 1];
      const double* avec = &m->edge_area[4 * e];
      const double* qL = &q[(size_t)a * NVARS];
      const double* qR = &q[(size_t)c * NVARS];
      const double* gL = &grad[(size_t)a * NTERMS * 3];
      const double* gR = &grad[(size_t)c * NTERMS * 3];
      double Qavg[NVARS], g[NTERMS * 3], flux[NEQN];
      for (int i = 0; i < NEQN; i++) Qavg[i] = (qL[i] + qR[i]) / 2.0;
      oracle_aux(gamma, Qavg);
      double tmut = 0.5 * (0.0 + 0.0);
      for (int i = 0; i < NTERMS * 3; i++) g[i] = 0.5 * (gL[i] + gR[i]);
      if (ho) {
        const double* xL = &m->xyz[3 * a];
        const double* xR = &m->xyz[3 * c];
        double dx[3], s2 = 0.0;
        for (int i = 0; i < 3; i++) { dx[i] = (xR[i] - xL[i]); s2 += dx[i] * dx[i]; }
        for (int j = 0; j < NTERMS; j++) {
          double qdots = dx[0] * g[j * 3 + 0] + dx[1] * g[j * 3 + 1] + dx[2] * g[j * 3 + 2];
          int loc = kGradList[j];
          double dq = (qR[loc] - qL[loc] - qdots) / s2;
          for (int i = 0; i < 3; i++) g[j * 3 + i] += dq * dx[i];
        }
      }
      oracle_viscous_flux(prm, Qavg, g, avec, tmut, flux);
      for (int i = 0; i < NEQN; i++) b[(size_t)c * NEQN + i] += flux[i];
      for (int i = 0; i < NEQN; i++) b[(size_t)a * NEQN + i] += -flux[i];
      ACCUM_ABS(c, flux);
      ACCUM_ABS(a, flux);
    }
    /* Bkernel_Viscous_Flux, :472: boundary node's own gradient */
    for (int eid = 0; eid < m->nbedge; eid++) {
      int a = m->bedges[2 * eid], c = m->bedges[2 * eid + 1];
      const double* avec = &m->bedge_area[4 * eid];
      const double* qL = &q[(size_t)a * NVARS];
      const double* qR = &q[(size_t)c * NVARS];
      double Qavg[NVARS], flux[NEQN];
      for (int i = 0; i < NEQN; i++) Qavg[i] = 0.5 * (qL[i] + qR[i]);
      oracle_aux(gamma, Qavg);
      oracle_viscous_flux(prm, Qavg, &grad[(size_t)a * NTERMS * 3], avec, 0.0, flux);
      for (int i = 0; i < NEQN; i++) b[(size_t)a * NEQN + i] += -flux[i];
      ACCUM_ABS(a, flux);
    }
  }
  /* TemporalResidual, ucs/residual.tcc:125-179 (first order: cnp1 = 1, cnm1 = 0) */
  if (qold && prm->torder) {
    const double timestep = param_time_step(prm);
    for (int i = 0; i < nn; i++) {
      double dt = 1.0 * m->vol[i] / timestep; /* the cnm1 = 0 term adds nothing */
      for (int j = 0; j < NEQN; j++) {
        double dq = q[(size_t)i * NVARS + j] - qold[(size_t)i * NEQN + j];
        b[(size_t)i * NEQN + j] -= dt * dq;
      }
    }
  }
  /* Bkernel_BC_Res_Modify, ucs/bc.tcc:903 -> ModifyViscousWallResidual (:1612) */
  for (int eid = 0; eid < m->nbedge; eid++) {
    if (bc_of(prm, m->bfactag[eid]) != PCFD_BC_NOSLIP) continue;
    int a = m->bedges[2 * eid];
    double Tw = prm->bc_twall[m->bfactag[eid]] / prm->ref_temperature;
    double* r = &b[(size_t)a * NEQN];
    r[1] = 0.0; r[2] = 0.0; r[3] = 0.0; r[4] = 0.0;
    if (Tw < 0.0) r[0] = 0.0;
  }
#undef ACCUM_ABS
  /* ParallelL2Norm / StridedParallelL2Norm, ucs/parallel.h:162,121 */
  if (norms) {
    double s = 0.0;
    for (size_t i = 0; i < (size_t)nn * NEQN; i++) s += b[i] * b[i];
    norms[0] = sqrt(s) / (double)((size_t)nn * NEQN);
    for (int j = 0; j < NEQN; j++) {
      double t = 0.0;
      for (int i = 0; i < nn; i++) t += b[(size_t)i * NEQN + j] * b[(size_t)i * NEQN + j];
      norms[1 + j] = sqrt(t) / (double)nn;
    }
  }
  if (nkneecap) *nkneecap = kc;
  return 0;
}

/* Freestream initial condition of every node, interior and phantom
 * (SetInitialConditions, ucs/compressible.tcc:884), optionally perturbed. */
void oracle_init_state(const pcfd_params* prm, int nrows, double* q) {
  double Qinf[NVARS];
  oracle_qinf(prm, Qinf);
  for (int i = 0; i < nrows; i++) {
    for (int j = 0; j < NEQN; j++) q[(size_t)i * NVARS + j] = Qinf[j];
    oracle_aux(prm->gamma, &q[(size_t)i * NVARS]);
  }
}

/* ---------------------------------------------------------------------- */
/* block LU, ucs/matrix.h:111,238                                         */
/* ---------------------------------------------------------------------- */

int oracle_lu(double* a, int* p, int n) {
  int condBad = 0, row = 0;
  double smallnum = 1.0e-15;
  for (int i = 0; i < n; i++) p[i] = i;
  for (int i = 0; i < n; i++) {
    double large = 0.0;
    for (int j = i; j < n; j++)
      if (fabs(a[p[j] * n + i]) > fabs(large)) { large = a[p[j] * n + i]; row = j; }
    if (large == 0.0) condBad++;
    else if (fabs(large) < smallnum) condBad++;
    int t = p[i]; p[i] = p[row]; p[row] = t;
    large = 1.0 / large;
    for (int j = i + 1; j < n; j++) a[p[j] * n + i] *= large;
    for (int j = i + 1; j < n; j++)
      for (int k = i + 1; k < n; k++) a[p[j] * n + k] -= a[p[j] * n + i] * a[p[i] * n + k];
  }
  return condBad > 0 ? 1 : 0;
}

void oracle_lusolve(const double* a, double* b, const int* p, double* x, int n) {
  for (int i = 0; i < n; i++) {
    double sum = 0.0;
    for (int j = 0; j < i; j++) sum += a[p[i] * n + j] * x[j];
    x[i] = b[p[i]] - sum;
  }
  for (int i = n - 1; i >= 0; i--) {
    double sum = 0.0;
    for (int j = n - 1; j > i; j--) sum += a[p[i] * n + j] * b[j];
    b[i] = (x[i] - sum) / a[p[i] * n + i];
  }
}

/* geometry primitives, ucs/geometry.h (CalcTriArea, CalcTetVol) */
void oracle_tri_area(const double* p1, const double* p2, const double* p3, double* r) {
  double v1[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
  double v2[3] = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
  r[0] = v1[1] * v2[2] - v2[1] * v1[2];
  r[1] = v1[2] * v2[0] - v2[2] * v1[0];
  r[2] = v1[0] * v2[1] - v2[0] * v1[1];
  r[0] = 0.5 * r[0]; r[1] = 0.5 * r[1]; r[2] = 0.5 * r[2];
}

double oracle_tet_vol(const double* p1, const double* p2, const double* p3, const double* p4) {
  double v1[3] = {p2[0] - p1[0], p2[1] - p1[1], p2[2] - p1[2]};
  double v2[3] = {p3[0] - p1[0], p3[1] - p1[1], p3[2] - p1[2]};
  double v3[3] = {p4[0] - p1[0], p4[1] - p1[1], p4[2] - p1[2]};
  double t[3];
  t[0] = v1[1] * v2[2] - v2[1] * v1[2];
  t[1] = v1[2] * v2[0] - v2[2] * v1[0];
  t[2] = v1[0] * v2[1] - v2[0] * v1[1];
  return (v3[0] * t[0] + v3[1] * t[1] + v3[2] * t[2]) / 6.0;
}

/* ---------------------------------------------------------------------- */
/* implicit part: time step, Jacobian, SGS, update                         */
/* ---------------------------------------------------------------------- */

/* MaxEigenvalue, ucs/compressible.tcc:799, on the face-averaged state */
static double max_eigenvalue(const pcfd_params* prm, const double* QL, const double* QR, const double* avec) {
  double t[NVARS];
  for (int i = 0; i < NEQN; i++) t[i] = 0.5 * (QL[i] + QR[i]);
  oracle_aux(prm->gamma, t);
  double gm1 = prm->gamma - 1.0;
  double rho = t[0], u = t[1] / rho, v = t[2] / rho, w = t[3] / rho;
  double v2h = 0.5 * (u * u + v * v + w * w);
  double P = gm1 * (t[4] - rho * v2h);
  double c = sqrt(prm->gamma * P / rho);
  double theta = u * avec[0] + v * avec[1] + w * avec[2];
  double e4 = fabs(theta + c), e5 = fabs(theta - c);
  return dmax(e4, e5);
}

/* ComputeTimesteps with local time stepping, ucs/timestep.tcc:7,80,115 */
double oracle_timestep(const pcfd_mesh_view* m, const pcfd_params* prm, const double* q, double cfl, double* dt) {
  const int nn = m->nnode;
  for (int i = 0; i < nn; i++) dt[i] = 0.0;
  for (int e = 0; e < m->nedge; e++) {
    int a = m->edges[2 * e], b = m->edges[2 * e + 1];
    const double* avec = &m->edge_area[4 * e];
    double s = max_eigenvalue(prm, &q[(size_t)a * NVARS], &q[(size_t)b * NVARS], avec) * avec[3];
    dt[b] += s;
    dt[a] += s;
  }
  for (int k = 0; k < m->nbedge; k++) {
    int a = m->bedges[2 * k], b = m->bedges[2 * k + 1];
    const double* avec = &m->bedge_area[4 * k];
    dt[a] += max_eigenvalue(prm, &q[(size_t)a * NVARS], &q[(size_t)b * NVARS], avec) * avec[3];
  }
  double dtmin = 0.0;
  for (int i = 0; i < nn; i++) {
    dt[i] = cfl * (m->vol[i] / dt[i]);
    dtmin = (i == 0) ? dt[i] : dmin(dtmin, dt[i]);
  }
  return dtmin;
}

/* CRSMatrix::Init, ucs/crsmatrix.tcc:48: diagonal first, then psp order */
void oracle_crs_init(const pcfd_mesh_view* m, int* ia, int* ja) {
  const int nn = m->nnode;
  ia[0] = 0;
  for (int i = 0; i < nn; i++) ia[i + 1] = ia[i] + (m->ipsp[i + 1] - m->ipsp[i]) + 1;
  for (int i = 0; i < nn; i++) {
    int c = ia[i];
    ja[c++] = i;
    for (int k = m->ipsp[i]; k < m->ipsp[i + 1]; k++) ja[c++] = m->psp[k];
  }
}

/* CRSMatrix::GetIndex, ucs/crsmatrix.tcc:740 (linear row search) */
static int crs_index(const int* ia, const int* ja, int row, int col) {
  if (row == col) return ia[row];
  for (int k = ia[row] + 1; k < ia[row + 1]; k++)
    if (ja[k] == col) return k;
  return -1;
}

static void numflux(const double* QL, const double* QR, const double* avec, double gamma, double* f) {
  oracle_roe_flux(QL, QR, avec, 0.0, gamma, f);
  kneecap(f);
}

/* CompressibleEqnSet::ViscousJacobian, ucs/compressible.tcc:1633 */
static void viscous_jacobian(const pcfd_params* prm, const double* QL, const double* QR, const double* dx, double s2,
                             const double* avec, double* aL, double* aR) {
  double Qavg[NVARS];
  for (int i = 0; i < NEQN; i++) Qavg[i] = 0.5 * (QL[i] + QR[i]);
  oracle_aux(prm->gamma, Qavg);
  double mu = viscosity(prm, Qavg);
  double tmut = mu;
  double ReTilde = prm->Re / prm->mach;
  double RK = avec[3] / ReTilde;
  double RKT = RK * tmut;
  double rhoL = QL[0], uL = QL[1] / rhoL, vL = QL[2] / rhoL, wL = QL[3] / rhoL, PL = QL[6];
  double rhoR = QR[0], uR = QR[1] / rhoR, vR = QR[2] / rhoR, wR = QR[3] / rhoR, PR = QR[6];
  double u = 0.5 * (uL + uR), v = 0.5 * (vL + vR), w = 0.5 * (wL + wR);
  double DxL[3], DxR[3];
  for (int i = 0; i < 3; i++) {
    DxL[i] = -dx[i] / (rhoL * s2);
    DxR[i] = dx[i] / (rhoR * s2);
  }
  double c43 = 4.0 / 3.0, mc23 = -2.0 / 3.0;
  double gamma = prm->gamma, gm1 = gamma - 1.0;
  double cp = 1.0 / gm1;
  double k = mu / prm->Pr * cp;
  double c1 = -(k + 0.0);
  for (int side = 1; side >= 0; side--) {
    const double* D = side ? DxR : DxL;
    double* A = side ? aR : aL;
    double rho = side ? rhoR : rhoL, P = side ? PR : PL;
    double us = side ? uR : uL, vs = side ? vR : vL, ws = side ? wR : wL;
    double dux = -u * D[0], duy = -u * D[1], duz = -u * D[2];
    double dvx = -v * D[0], dvy = -v * D[1], dvz = -v * D[2];
    double dwx = -w * D[0], dwy = -w * D[1], dwz = -w * D[2];
    double dfact = -2.0 / 3.0 * (dux + dvy + dwz);
    double dtxx = (2.0 * dux + dfact), dtyy = (2.0 * dvy + dfact), dtzz = (2.0 * dwz + dfact);
    double dtxy = duy + dvx, dtxz = duz + dwx, dtyz = dvz + dwy;
    double dtxn = dtxx * avec[0] + dtxy * avec[1] + dtxz * avec[2];
    double dtyn = dtxy * avec[0] + dtyy * avec[1] + dtyz * avec[2];
    double dtzn = dtxz * avec[0] + dtyz * avec[1] + dtzz * avec[2];
    double r2u = (c43 * D[0] * avec[0] + D[1] * avec[1] + D[2] * avec[2]);
    double r2v = (mc23 * D[1] * avec[0] + D[0] * avec[1]);
    double r2w = (mc23 * D[2] * avec[0] + D[0] * avec[2]);
    double r3u = (mc23 * D[0] * avec[1] + D[1] * avec[0]);
    double r3v = (D[0] * avec[0] + c43 * D[1] * avec[1] + D[2] * avec[2]);
    double r3w = (mc23 * D[2] * avec[1] + D[1] * avec[2]);
    double r4u = (mc23 * D[0] * avec[2] + D[2] * avec[0]);
    double r4v = (mc23 * D[1] * avec[2] + D[2] * avec[1]);
    double r4w = (D[0] * avec[0] + D[1] * avec[1] + c43 * D[2] * avec[2]);
    A[0] = A[1] = A[2] = A[3] = A[4] = 0.0;
    A[5] = -RKT * (dtxn); A[6] = -RKT * r2u; A[7] = -RKT * r2v; A[8] = -RKT * r2w; A[9] = 0.0;
    A[10] = -RKT * (dtyn); A[11] = -RKT * r3u; A[12] = -RKT * r3v; A[13] = -RKT * r3w; A[14] = 0.0;
    A[15] = -RKT * (dtzn); A[16] = -RKT * r4u; A[17] = -RKT * r4v; A[18] = -RKT * r4w; A[19] = 0.0;
    double v2 = (us * us + vs * vs + ws * ws);
    double dT_dP = gamma / rho;
    double dP_dr = +gm1 * 0.5 * v2, dP_dru = -gm1 * us, dP_drv = -gm1 * vs, dP_drw = -gm1 * ws, dP_dret = +gm1;
    double Tn = (D[0] * avec[0] + D[1] * avec[1] + D[2] * avec[2]) * dT_dP * c1;
    A[20] = -RKT * (dtxn * u + dtyn * v + dtzn * w) + RK * Tn * (dP_dr - P / rho);
    A[21] = -RKT * (r2u * u + r3u * v + r4u * w) + RK * Tn * dP_dru;
    A[22] = -RKT * (r2v * u + r3v * v + r4v * w) + RK * Tn * dP_drv;
    A[23] = -RKT * (r2w * u + r3w * v + r4w * w) + RK * Tn * dP_drw;
    A[24] = RK * Tn * dP_dret;
  }
  for (int i = 0; i < 25; i++) aL[i] = -aL[i];
}

/* One half-edge of CalculateBoundaryVariables on (QL, QR) in place */
static int apply_bc_one(const pcfd_mesh_view* m, const pcfd_params* prm, const double* q, const double* Qinf, int eid,
                        double* QL, double* QR) {
  const double* avec = &m->bedge_area[4 * eid];
  int bct = bc_of(prm, m->bfactag[eid]);
  const double gamma = prm->gamma;
  switch (bct) {
    case PCFD_BC_SONIC_INFLOW:
    case PCFD_BC_DIRICHLET:
      for (int i = 0; i < NVARS; i++) QR[i] = QL[i] = Qinf[i];
      break;
    case PCFD_BC_SONIC_OUTFLOW:
    case PCFD_BC_NEUMANN:
      for (int i = 0; i < NEQN; i++) QR[i] = QL[i];
      break;
    case PCFD_BC_FARFIELD:
      bc_farfield(gamma, QL, QR, Qinf, avec, 0.0);
      break;
    case PCFD_BC_IMPERMEABLE_WALL:
    case PCFD_BC_SYMMETRY:
      bc_inviscid_wall(gamma, prm->no_cvbc, QL, QR, avec, 0.0);
      break;
    case PCFD_BC_NOSLIP: {
      int nn = oracle_normal_node(m, m->bedges[2 * eid], avec);
      double nQ[NVARS];
      memcpy(nQ, &q[(size_t)nn * NVARS], sizeof(nQ));
      double Tw = prm->bc_twall[m->bfactag[eid]] / prm->ref_temperature;
      bc_viscous_wall(gamma, QL, QR, nQ, Tw);
      break;
    }
    default:
      return -1;
  }
  oracle_aux(gamma, QR);
  oracle_aux(gamma, QL);
  return 0;
}

/* LU in place of every diagonal block (PrepareSGS, ucs/crsmatrix.tcc:840) */
void oracle_prepare_sgs(int nnode, const int* ia, double* M, int* pv) {
  for (int i = 0; i < nnode; i++) oracle_lu(&M[(size_t)ia[i] * 25], &pv[(size_t)i * 5], 5);
}

/* ComputeJacobians (ucs/jacobian.tcc:13) for the ideal gas, steady:
 * Kernel_NumJac, Bkernel_NumJac (jacobianBoundaryEval = 0, which applies the
 * boundary conditions to the stored state as it goes), Kernel_Viscous_Jac,
 * Kernel_Diag_NumJac, ContributeTemporalTerms with dt, then the no-slip row
 * changes.  M [nblocks][25] in the reference layout; q is modified as the
 * reference modifies it. */
int oracle_jacobian(const pcfd_mesh_view* m, const pcfd_params* prm, double* q, const double* dt, const int* ia,
                    const int* ja, double* M) {
  const int nn = m->nnode;
  const double gamma = prm->gamma;
  const double h = 1.0e-8;
  memset(M, 0, sizeof(double) * (size_t)ia[nn] * 25);
  double Qinf[NVARS];
  oracle_qinf(prm, Qinf);
  /* Kernel_NumJac, :254 */
  for (int e = 0; e < m->nedge; e++) {
    int a = m->edges[2 * e], b = m->edges[2 * e + 1];
    const double* avec = &m->edge_area[4 * e];
    const double* QL = &q[(size_t)a * NVARS];
    const double* QR = &q[(size_t)b * NVARS];
    double fS[NEQN], fL[NEQN], fR[NEQN], QPL[NVARS], QPR[NVARS], tL[25], tR[25];
    numflux(QL, QR, avec, gamma, fS);
    for (int i = 0; i < NEQN; i++) {
      memcpy(QPL, QL, sizeof(QPL));
      memcpy(QPR, QR, sizeof(QPR));
      QPL[i] += h;
      QPR[i] += h;
      oracle_aux(gamma, QPL);
      oracle_aux(gamma, QPR);
      numflux(QPL, QR, avec, gamma, fL);
      numflux(QL, QPR, avec, gamma, fR);
      for (int j = 0; j < NEQN; j++) tL[j * NEQN + i] = (fS[j] - fL[j]) / h;
      for (int j = 0; j < NEQN; j++) tR[j * NEQN + i] = (fR[j] - fS[j]) / h;
    }
    double* pR = &M[(size_t)crs_index(ia, ja, a, b) * 25];
    double* pL = &M[(size_t)crs_index(ia, ja, b, a) * 25];
    for (int t = 0; t < 25; t++) pR[t] += tR[t];
    for (int t = 0; t < 25; t++) pL[t] += tL[t];
  }
  /* Bkernel_NumJac, :459 */
  for (int eid = 0; eid < m->nbedge; eid++) {
    int a = m->bedges[2 * eid], b = m->bedges[2 * eid + 1];
    const double* avec = &m->bedge_area[4 * eid];
    double* QL = &q[(size_t)a * NVARS];
    double* QR = &q[(size_t)b * NVARS];
    if (apply_bc_one(m, prm, q, Qinf, eid, QL, QR)) return -1;
    double fS[NEQN], fL[NEQN], QPL[NVARS], QPR[NVARS], tL[25];
    const int beval = prm->jac_boundary_eval;
    if (beval == 3) {
      /* build extension: base state through the same boundary map */
      double QBL[NVARS], QBR[NVARS];
      memcpy(QBL, QL, sizeof(QBL));
      memcpy(QBR, QR, sizeof(QBR));
      apply_bc_one(m, prm, q, Qinf, eid, QBL, QBR);
      numflux(QBL, QBR, avec, gamma, fS);
    } else {
      numflux(QL, QR, avec, gamma, fS);
    }
    for (int i = 0; i < NEQN; i++) {
      memcpy(QPL, QL, sizeof(QPL));
      memcpy(QPR, QR, sizeof(QPR));
      QPL[i] += h;
      QPR[i] += h;
      oracle_aux(gamma, QPL);
      oracle_aux(gamma, QPR);
      if (beval != 1) {
        memcpy(QPR, QR, sizeof(QPR));
        oracle_aux(gamma, QPR);
        apply_bc_one(m, prm, q, Qinf, eid, QPL, QPR);
        numflux(QPL, QPR, avec, gamma, fL);
      } else {
        numflux(QPL, QR, avec, gamma, fL);
      }
      for (int j = 0; j < NEQN; j++) tL[j * NEQN + i] = (fL[j] - fS[j]) / h;
    }
    double* d = &M[(size_t)ia[a] * 25];
    for (int t = 0; t < 25; t++) d[t] += tL[t];
  }
  /* Kernel_Viscous_Jac, :734 */
  if (prm->viscous) {
    for (int e = 0; e < m->nedge; e++) {
      int a = m->edges[2 * e], b = m->edges[2 * e + 1];
      const double* xL = &m->xyz[3 * a];
      const double* xR = &m->xyz[3 * b];
      double dx[3], s2 = 0.0, aL[25], aR[25];
      for (int i = 0; i < 3; i++) { dx[i] = (xR[i] - xL[i]); s2 += dx[i] * dx[i]; }
      viscous_jacobian(prm, &q[(size_t)a * NVARS], &q[(size_t)b * NVARS], dx, s2, &m->edge_area[4 * e], aL, aR);
      double* pR = &M[(size_t)crs_index(ia, ja, a, b) * 25];
      double* pL = &M[(size_t)crs_index(ia, ja, b, a) * 25];
      for (int t = 0; t < 25; t++) pR[t] += aR[t];
      for (int t = 0; t < 25; t++) pL[t] += aL[t];
    }
  }
  /* Kernel_Diag_NumJac, :437 */
  for (int e = 0; e < m->nedge; e++) {
    int a = m->edges[2 * e], b = m->edges[2 * e + 1];
    const double* jacL = &M[(size_t)crs_index(ia, ja, b, a) * 25];
    const double* jacR = &M[(size_t)crs_index(ia, ja, a, b) * 25];
    double* dR = &M[(size_t)ia[b] * 25];
    double* dL = &M[(size_t)ia[a] * 25];
    for (int t = 0; t < 25; t++) dR[t] += -jacR[t];
    for (int t = 0; t < 25; t++) dL[t] += -jacL[t];
  }
  /* ContributeTemporalTerms, ucs/jacobian.tcc:214 -> ucs/eqnset.tcc:195 */
  for (int i = 0; i < nn; i++) {
    double* d = &M[(size_t)ia[i] * 25];
    for (int r = 0; r < NEQN; r++) d[r * NEQN + r] += 1.0 * m->vol[i] / dt[i];
  }
  /* Bkernel_BC_Jac_Modify -> ModifyViscousWallJacobian */
  for (int eid = 0; eid < m->nbedge; eid++) {
    if (bc_of(prm, m->bfactag[eid]) != PCFD_BC_NOSLIP) continue;
    int a = m->bedges[2 * eid];
    double Tw = prm->bc_twall[m->bfactag[eid]] / prm->ref_temperature;
    int rows[5], nr = 0;
    rows[nr++] = 1; rows[nr++] = 2; rows[nr++] = 3;
    if (Tw < 0.0) { rows[nr++] = 0; rows[nr++] = 4; }
    else rows[nr++] = 4;
    for (int rr = 0; rr < nr; rr++) {
      int sr = rows[rr];
      for (int k = ia[a]; k < ia[a + 1]; k++)
        for (int c = 0; c < NEQN; c++) M[(size_t)k * 25 + sr * NEQN + c] = 0.0;
      M[(size_t)ia[a] * 25 + sr * NEQN + sr] = 1.0;
    }
    if (Tw < 0.0) {
      int nnrm = oracle_normal_node(m, a, &m->bedge_area[4 * eid]);
      double* off = &M[(size_t)crs_index(ia, ja, a, nnrm) * 25];
      off[0] = -1.0;
      off[24] = -1.0;
    } else {
      M[(size_t)ia[a] * 25 + 4 * NEQN + 0] = -(Tw / (gamma * (gamma - 1.0)) + 0.5 * 0.0);
    }
  }
  return 0;
}

/* One block Gauss-Seidel row update (the body of the loops in CRS::SGS) */
static void sgs_row(int node, const int* ia, const int* ja, const double* M, const int* pv, const double* b,
                    double* x) {
  double rhs[NEQN], vout[NEQN], tmp[NEQN];
  memcpy(rhs, &b[(size_t)node * NEQN], sizeof(rhs));
  for (int k = ia[node] + 1; k < ia[node + 1]; k++) {
    oracle_matvec(&M[(size_t)k * 25], &x[(size_t)ja[k] * NEQN], vout, NEQN);
    for (int c = 0; c < NEQN; c++) rhs[c] -= vout[c];
  }
  oracle_lusolve(&M[(size_t)ia[node] * 25], rhs, &pv[(size_t)node * NEQN], tmp, NEQN);
  memcpy(&x[(size_t)node * NEQN], rhs, sizeof(rhs));
}

/* CRS::SGS, ucs/crs.tcc:62: nSgs x (forward then backward lexicographic
 * sweeps); M's diagonal must hold its LU (oracle_prepare_sgs).  Returns
 * |norm(x) after the last sweep - after the one before|. */
double oracle_sgs(int nnode, const int* ia, const int* ja, const double* M, const int* pv, const double* b, double* x,
                  int nsweeps) {
  double xOld = 0.0, xNorm = 0.0;
  for (int s = 0; s < nsweeps; s++) {
    for (int i = 0; i < nnode; i++) sgs_row(i, ia, ja, M, pv, b, x);
    for (int i = nnode - 1; i >= 0; i--) sgs_row(i, ia, ja, M, pv, b, x);
    xOld = xNorm;
    double t = 0.0;
    for (size_t k = 0; k < (size_t)nnode * NEQN; k++) t += x[k] * x[k];
    xNorm = sqrt(t) / (double)((size_t)nnode * NEQN);
  }
  return fabs(xOld - xNorm);
}

/* The same sweeps over rows grouped by colour (rows[cptr[c]..cptr[c+1]]),
 * colours forward then backward: the order the GPU uses.  Test helper. */
void oracle_sgs_colored(int nnode, const int* ia, const int* ja, const double* M, const int* pv, const double* b,
                        double* x, int nsweeps, int ncolor, const int* cptr, const int* rows) {
  (void)nnode;
  for (int s = 0; s < nsweeps; s++) {
    for (int c = 0; c < ncolor; c++)
      for (int k = cptr[c]; k < cptr[c + 1]; k++) sgs_row(rows[k], ia, ja, M, pv, b, x);
    for (int c = ncolor - 1; c >= 0; c--)
      for (int k = cptr[c]; k < cptr[c + 1]; k++) sgs_row(rows[k], ia, ja, M, pv, b, x);
  }
}

/* NaN/Inf update zeroing and CompressibleEqnSet::ApplyDQ
 * (ucs/solutionSpace.tcc:774-804, ucs/compressible.tcc:929); returns the
 * update norm sqrt(sum x^2)/(nnode*5). */
double oracle_apply_dq(const pcfd_mesh_view* m, const pcfd_params* prm, double* x, double* q) {
  const int nn = m->nnode;
  const double gm1 = prm->gamma - 1.0;
  for (int j = 0; j < nn; j++) {
    int zero = 0;
    for (int k = 0; k < NEQN; k++)
      if (isnan(x[(size_t)j * NEQN + k]) || isinf(x[(size_t)j * NEQN + k])) { x[(size_t)j * NEQN + k] = 0.0; zero = 1; }
    if (zero)
      for (int k = 0; k < NEQN; k++) x[(size_t)j * NEQN + k] = 0.0;
  }
  for (int j = 0; j < nn; j++) {
    double* dQ = &x[(size_t)j * NEQN];
    double* Q = &q[(size_t)j * NVARS];
    double minP = 1.0e-10, minRho = 1.0e-10, minE = 1.0e-10;
    if (Q[0] + dQ[0] < 0.0) Q[0] = minRho; else Q[0] += dQ[0];
    if (Q[4] + dQ[4] < 0.0) Q[4] = minE; else Q[4] += dQ[4];
    double rho = Q[0], u = Q[1] / rho, v = Q[2] / rho, w = Q[3] / rho, E = Q[4];
    double v2 = u * u + v * v + w * w;
    if (E < 0.5 * rho * v2) {
      double v2mod = 2.0 * (E - minP / gm1);
      double frac = 0.0;
      if (v2mod > 0.0) frac = sqrt(v2mod / v2);
      u *= frac; v *= frac; w *= frac;
      Q[1] = rho * u; Q[2] = rho * v; Q[3] = rho * w;
    } else {
      Q[1] += dQ[1]; Q[2] += dQ[2]; Q[3] += dQ[3];
    }
    oracle_aux(prm->gamma, Q);
  }
  double t = 0.0;
  for (size_t k = 0; k < (size_t)nn * NEQN; k++) t += x[k] * x[k];
  return sqrt(t) / (double)((size_t)nn * NEQN);
}

/* Forces::ComputeYpCf -> FORCE_Kernel (ucs/forces.tcc:124-197, :376-408):
 * over the boundary half-edges in order, those whose tag belongs to the body
 * (in_body[factag] != 0) add p |a| n to the pressure force and, on no-slip
 * walls of a viscous run, the wall stress |a| to the viscous force.
 * ComputeStressVector (ucs/compressible.tcc:1113) reads the stress from
 * gradient entries 3..11, the gradients of the momentum components (the
 * velocity gradients sit at 18..26); this restates it as written.
 * out[0..2] pressure force, out[3..5] viscous force. */
void oracle_forces(const pcfd_mesh_view* m, const pcfd_params* prm, const double* q, const double* grad,
                   const int* in_body, double* out) {
  for (int j = 0; j < 6; j++) out[j] = 0.0;
  const double Sconst = 110.4 / prm->ref_temperature;
  const double retilde = prm->Re / prm->mach;
  for (int eid = 0; eid < m->nbedge; eid++) {
    const int tag = m->bfactag[eid];
    if (tag < 0 || tag >= prm->ntags || !in_body[tag]) continue;
    const int a = m->bedges[2 * eid];
    const double* avec = &m->bedge_area[4 * eid];
    const double* Q = &q[(size_t)a * NVARS];
    const double p = Q[6];
    for (int j = 0; j < 3; j++) out[j] += p * avec[j] * avec[3];
    if (prm->bc_type[tag] == PCFD_BC_NOSLIP && prm->viscous) {
      const double T = Q[5];
      const double mu = (1.0 + Sconst) * pow(T, 1.5) / (T + Sconst);
      const double* g = &grad[(size_t)a * NTERMS * 3];
      const double ux = g[3], uy = g[4], uz = g[5], vx = g[6], vy = g[7], vz = g[8], wx = g[9], wy = g[10],
                   wz = g[11];
      const double div = -2.0 / 3.0 * (ux + vy + wz);
      const double txx = 2.0 * ux + div, tyy = 2.0 * vy + div, tzz = 2.0 * wz + div;
      const double txy = uy + vx, txz = uz + wx, tyz = vz + wy;
      const double txn = txx * avec[0] + txy * avec[1] + txz * avec[2];
      const double tyn = txy * avec[0] + tyy * avec[1] + tyz * avec[2];
      const double tzn = txz * avec[0] + tyz * avec[1] + tzz * avec[2];
      const double s0 = -(mu / retilde) * txn, s1 = -(mu / retilde) * tyn, s2 = -(mu / retilde) * tzn;
      out[3] += s0 * avec[3];
      out[4] += s1 * avec[3];
      out[5] += s2 * avec[3];
    }
  }
}
