// Device-side equation-set math for the ideal-gas compressible path
// (CompressibleEqnSet<T>, ucs/compressible.tcc).  Operation order follows the
// reference; divisions by the same quantity are replaced by one reciprocal
// and multiplications, because FP64 division and square root are the
// scarcest resource on sm_103a.
#pragma once

#include <cuda_runtime.h>

namespace pcfd {

constexpr int NEQN = 5;
constexpr int NVARS = 10;   // rho, rho u, rho v, rho w, rho E | T, P, u, v, w
constexpr int NTERMS = 9;   // gradient terms: 0..5 and 7..9 of q (GetGradientsLocation)

__device__ __forceinline__ double dmax(double a, double b) { return (a > b) ? a : b; }

// Harten-Hyman entropy fix of one eigenvalue (ucs/compressible.tcc:148-185)
__device__ __forceinline__ double entropy_fix(double eig, double eigL, double eigR) {
  double eps = dmax(eig - eigL, eigR - eig);
  eps = dmax(0.0, eps);
  double a = fabs(eig);
  if (a < eps) a = 0.5 * (eig * eig / eps + eps);
  return a;
}

// Roe flux with the reference's eigen-decomposition: RoeVariables (:533),
// Eigensystem (:580), entropy fix, |A| dQ = T |L| Tinv dQ, and
// 0.5 area (F_L + F_R - |A| dQ) (RoeFlux, :93).  avec = (nx, ny, nz, area);
// static grid (vdotn = 0).
// Returns a mask of non-physical states in the sense of BadExtrapolation
// (ucs/compressible.tcc:1056: p < 1e-10, rho < 0 or rho E < 1e-10):
// bit 0 = left state, bit 1 = right state, bit 2 = Roe-averaged state.  The
// limiter's pressure clip (ucs/limiters.tcc:737) applies exactly these
// three tests to the same extrapolated states.
__device__ __forceinline__ int roe_flux(const double* QL, const double* QR, const double nx, const double ny,
                                        const double nz, const double area, const double gamma, double* flux) {
  const double gm1 = gamma - 1.0;
  const double rL = QL[0], irL = 1.0 / rL;
  const double uL = QL[1] * irL, vL = QL[2] * irL, wL = QL[3] * irL, EL = QL[4];
  const double PL = gm1 * (EL - 0.5 * rL * (uL * uL + vL * vL + wL * wL));
  const double hL = (EL + PL) * irL;
  const double rR = QR[0], irR = 1.0 / rR;
  const double uR = QR[1] * irR, vR = QR[2] * irR, wR = QR[3] * irR, ER = QR[4];
  const double PR = gm1 * (ER - 0.5 * rR * (uR * uR + vR * vR + wR * wR));
  const double hR = (ER + PR) * irR;

  // Roe-averaged state
  const double rho = sqrt(rL * rR);
  const double sigma = rho / (rL + rho);
  const double u = uL + sigma * (uR - uL);
  const double v = vL + sigma * (vR - vL);
  const double w = wL + sigma * (wR - wL);
  const double h = hL + sigma * (hR - hL);
  double v2h = 0.5 * (u * u + v * v + w * w);
  const double rE = rho * (1.0 / gamma) * (h + gm1 * v2h);
  const double irho = 1.0 / rho;
  const double P = gm1 * (rE - rho * v2h);
  const double c2 = gamma * P * irho;
  const double c = sqrt(c2);
  const double ic = 1.0 / c;
  const double ic2 = ic * ic;
  const double thetaf = u * nx + v * ny + w * nz;

  // entropy-fixed |eigenvalues|
  const double thetaL = uL * nx + vL * ny + wL * nz;
  const double thetaR = uR * nx + vR * ny + wR * nz;
  const double cL = sqrt(gamma * PL * irL);
  const double cR = sqrt(gamma * PR * irR);
  const double l0 = entropy_fix(thetaf, thetaL, thetaR);
  const double l3 = entropy_fix(thetaf + c, thetaL + cL, thetaR + cR);
  const double l4 = entropy_fix(thetaf - c, thetaL - cL, thetaR - cR);

  const double d0 = QR[0] - QL[0], d1 = QR[1] - QL[1], d2 = QR[2] - QL[2], d3 = QR[3] - QL[3],
               d4 = QR[4] - QL[4];

  // dv = Tinv dQ (rows of the left eigenvector matrix)
  const double gv = gm1 * v2h, gu = gm1 * u, gvv = gm1 * v, gw = gm1 * w;
  double dv0 = (nx - nz * v * irho + ny * w * irho - nx * ic2 * gv) * d0 + (nx * ic2 * gu) * d1 +
               (nz * irho + nx * ic2 * gvv) * d2 + (-ny * irho + nx * ic2 * gw) * d3 + (-nx * ic2 * gm1) * d4;
  double dv1 = (ny + nz * u * irho - nx * w * irho - ny * ic2 * gv) * d0 + (-nz * irho + ny * ic2 * gu) * d1 +
               (ny * ic2 * gvv) * d2 + (nx * irho + ny * ic2 * gw) * d3 + (-ny * ic2 * gm1) * d4;
  double dv2 = (nz - ny * u * irho + nx * v * irho - nz * ic2 * gv) * d0 + (ny * irho + nz * ic2 * gu) * d1 +
               (-nx * irho + nz * ic2 * gvv) * d2 + (nz * ic2 * gw) * d3 + (-nz * ic2 * gm1) * d4;
  const double hr = 0.5 * irho;
  double dv3 = (-hr * (thetaf - gv * ic)) * d0 + (hr * (nx - gu * ic)) * d1 + (hr * (ny - gvv * ic)) * d2 +
               (hr * (nz - gw * ic)) * d3 + (hr * (gm1 * ic)) * d4;
  double dv4 = (hr * (thetaf + gv * ic)) * d0 + (-hr * (nx + gu * ic)) * d1 + (-hr * (ny + gvv * ic)) * d2 +
               (-hr * (nz + gw * ic)) * d3 + (hr * (gm1 * ic)) * d4;
  dv0 *= l0; dv1 *= l0; dv2 *= l0; dv3 *= l3; dv4 *= l4;

  // dr = T dv (columns of the right eigenvector matrix)
  const double rc = rho * ic;
  const double cg = c * (1.0 / gm1);
  const double dr0 = nx * dv0 + ny * dv1 + nz * dv2 + rc * dv3 + rc * dv4;
  const double dr1 = (u * nx) * dv0 + (u * ny - rho * nz) * dv1 + (u * nz + rho * ny) * dv2 +
                     rho * (u * ic + nx) * dv3 + rho * (u * ic - nx) * dv4;
  const double dr2 = (v * nx + rho * nz) * dv0 + (v * ny) * dv1 + (v * nz - rho * nx) * dv2 +
                     rho * (v * ic + ny) * dv3 + rho * (v * ic - ny) * dv4;
  const double dr3 = (w * nx - rho * ny) * dv0 + (w * ny + rho * nx) * dv1 + (w * nz) * dv2 +
                     rho * (w * ic + nz) * dv3 + rho * (w * ic - nz) * dv4;
  const double dr4 = (v2h * nx + rho * (v * nz - w * ny)) * dv0 + (v2h * ny + rho * (w * nx - u * nz)) * dv1 +
                     (v2h * nz + rho * (u * ny - v * nx)) * dv2 + rho * (v2h * ic + thetaf + cg) * dv3 +
                     rho * (v2h * ic - thetaf + cg) * dv4;

  // physical fluxes (Flux, :686)
  const double rtL = rL * thetaL, rtR = rR * thetaR;
  const double ha = 0.5 * area;
  flux[0] = ha * (rtL + rtR - dr0);
  flux[1] = ha * ((uL * rtL + PL * nx) + (uR * rtR + PR * nx) - dr1);
  flux[2] = ha * ((vL * rtL + PL * ny) + (vR * rtR + PR * ny) - dr2);
  flux[3] = ha * ((wL * rtL + PL * nz) + (wR * rtR + PR * nz) - dr3);
  flux[4] = ha * (hL * rtL + hR * rtR - dr4);
  return ((rL < 0.0 || EL < 1.0e-10 || PL < 1.0e-10) ? 1 : 0) | ((rR < 0.0 || ER < 1.0e-10 || PR < 1.0e-10) ? 2 : 0) |
         ((P < 1.0e-10 || rE < 1.0e-10) ? 4 : 0);
}

// ComputeAuxiliaryVariables (ucs/compressible.tcc:1230) on a 10-wide record
__device__ __forceinline__ void aux_vars(double gamma, double* Q) {
  const double gm1 = gamma - 1.0;
  const double ir = 1.0 / Q[0];
  const double u = Q[1] * ir, v = Q[2] * ir, w = Q[3] * ir;
  const double P = gm1 * (Q[4] - 0.5 * Q[0] * (u * u + v * v + w * w));
  Q[6] = P;
  Q[5] = gamma * P * ir;
  Q[7] = u;
  Q[8] = v;
  Q[9] = w;
}

// Sutherland's law (EqnSet::ComputeViscosity, ucs/eqnset.h:251)
__device__ __forceinline__ double sutherland(double T, double S) { return (1.0 + S) * (T * sqrt(T)) / (T + S); }

// ViscousFlux (ucs/compressible.tcc:713) for laminar flow (mut = 0).
// Q: averaged conservative state; T: its temperature; grad: 27-wide face
// gradient; rk = area / ReTilde.
__device__ __forceinline__ void viscous_flux(const double u, const double v, const double w, const double T,
                                             const double* grad, const double nx, const double ny, const double nz,
                                             const double rk, const double S, const double cp_over_pr,
                                             double* flux) {
  const double Tx = grad[15], Ty = grad[16], Tz = grad[17];
  const double ux = grad[18], uy = grad[19], uz = grad[20];
  const double vx = grad[21], vy = grad[22], vz = grad[23];
  const double wx = grad[24], wy = grad[25], wz = grad[26];
  const double mu = sutherland(T, S);
  const double fact = -2.0 / 3.0 * (ux + vy + wz);
  const double tauxx = 2.0 * ux + fact, tauyy = 2.0 * vy + fact, tauzz = 2.0 * wz + fact;
  const double tauxy = uy + vx, tauxz = uz + wx, tauyz = vz + wy;
  const double RKT = rk * mu;
  const double c1 = -(mu * cp_over_pr);
  const double Tn = Tx * nx + Ty * ny + Tz * nz;
  const double tauxn = tauxx * nx + tauxy * ny + tauxz * nz;
  const double tauyn = tauxy * nx + tauyy * ny + tauyz * nz;
  const double tauzn = tauxz * nx + tauyz * ny + tauzz * nz;
  flux[0] = 0.0;
  flux[1] = -RKT * tauxn;
  flux[2] = -RKT * tauyn;
  flux[3] = -RKT * tauzn;
  flux[4] = -RKT * (tauxn * u + tauyn * v + tauzn * w) + rk * c1 * Tn;
}

}  // namespace pcfd
