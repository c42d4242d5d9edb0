// Device-side equation-set math for the ideal-gas compressible path
// (CompressibleEqnSet<T>, ucs/compressible.tcc), templated on the scalar type:
// S = double is the reference precision, S = dfl runs the same algebra in
// double-float on the FP32 pipes (dfloat.cuh).  Operation order follows the
// reference; divisions by the same quantity are replaced by one reciprocal
// and multiplications, because division and square root are the costliest
// operations on sm_103a.
#pragma once

#include <cuda_runtime.h>

#include "dfloat.cuh"

namespace pcfd {

constexpr int NEQN = 5;
constexpr int NVARS = 10;   // rho, rho u, rho v, rho w, rho E | T, P, u, v, w
constexpr int NTERMS = 9;   // gradient terms: 0..5 and 7..9 of q (GetGradientsLocation)

template <class S>
__device__ __forceinline__ S smax(S a, S b) { return (a > b) ? a : b; }

// Harten-Hyman entropy fix of one eigenvalue (ucs/compressible.tcc:148-185)
template <class S>
__device__ __forceinline__ S entropy_fix(S eig, S eigL, S eigR) {
  S eps = smax(eig - eigL, eigR - eig);
  eps = smax(Sc<S>::c(0.0), eps);
  S a = fabs(eig);
  if (a < eps) a = halve(eig * eig / eps + eps);
  return a;
}

// Primitive quantities of one side of a Roe flux (the per-state part of
// RoeVariables, Eigensystem and Flux).  A finite-difference Jacobian that
// perturbs one side reuses the other side's record.
template <class S>
struct RoeSide {
  S r, ir, u, v, w, E, P, h, c, th;
};

template <class S>
__device__ __forceinline__ RoeSide<S> roe_side(const S* Q, const S nx, const S ny, const S nz, const S gamma,
                                               const S gm1) {
  RoeSide<S> o;
  o.r = Q[0];
  o.ir = Sc<S>::c(1.0) / o.r;
  o.u = Q[1] * o.ir;
  o.v = Q[2] * o.ir;
  o.w = Q[3] * o.ir;
  o.E = Q[4];
  o.P = gm1 * (o.E - halve(o.r) * (o.u * o.u + o.v * o.v + o.w * o.w));
  o.h = (o.E + o.P) * o.ir;
  o.c = sqrt(gamma * o.P * o.ir);
  o.th = o.u * nx + o.v * ny + o.w * nz;
  return o;
}

template <class S>
__device__ __forceinline__ int roe_core(const RoeSide<S>& L, const RoeSide<S>& R, const S* QL, const S* QR,
                                        const S nx, const S ny, const S nz, const S area, const S gamma, const S gm1,
                                        const S igamma, S* flux);

// Roe flux with the reference's eigensystem: RoeVariables (:533),
// Eigensystem (:580), entropy fix, |A| dQ = T |L| Tinv dQ (evaluated in
// projector form, in roe_core), and 0.5 area (F_L + F_R - |A| dQ)
// (RoeFlux, :93).  (nx, ny, nz, area) is the edge's unit normal and area;
// static grid (vdotn = 0).
// Returns a mask of non-physical states in the sense of BadExtrapolation
// (ucs/compressible.tcc:1056: p < 1e-10, rho < 0 or rho E < 1e-10):
// bit 0 = left state, bit 1 = right state, bit 2 = Roe-averaged state.  The
// limiter's pressure clip (ucs/limiters.tcc:737) applies exactly these
// three tests to the same extrapolated states.
template <class S>
__device__ __forceinline__ int roe_flux(const S* QL, const S* QR, const S nx, const S ny, const S nz, const S area,
                                        const S gamma, const S gm1, const S igamma, const S igm1, S* flux) {
  return roe_core(roe_side(QL, nx, ny, nz, gamma, gm1), roe_side(QR, nx, ny, nz, gamma, gm1), QL, QR, nx, ny, nz,
                  area, gamma, gm1, igamma, flux);
}

template <class S>
__device__ __forceinline__ int roe_core(const RoeSide<S>& L, const RoeSide<S>& R, const S* QL, const S* QR,
                                        const S nx, const S ny, const S nz, const S area, const S gamma, const S gm1,
                                        const S igamma, S* flux) {
  const S one = Sc<S>::c(1.0);
  const S rL = L.r, uL = L.u, vL = L.v, wL = L.w, EL = L.E, PL = L.P, hL = L.h;
  const S rR = R.r, uR = R.u, vR = R.v, wR = R.w, ER = R.E, PR = R.P, hR = R.h;

  // Roe-averaged state
  const S rho = sqrt(rL * rR);
  const S sigma = rho / (rL + rho);
  const S u = uL + sigma * (uR - uL);
  const S v = vL + sigma * (vR - vL);
  const S w = wL + sigma * (wR - wL);
  const S h = hL + sigma * (hR - hL);
  S v2h = halve(u * u + v * v + w * w);
  const S rE = rho * igamma * (h + gm1 * v2h);
  const S P = gm1 * (rE - rho * v2h);
  const S c2 = gm1 * (h - v2h);  // = gamma P / rho with P and rE above
  const S c = sqrt(c2);
  const S ic2 = one / c2;
  const S thetaf = u * nx + v * ny + w * nz;

  // entropy-fixed |eigenvalues|
  const S thetaL = L.th, thetaR = R.th, cL = L.c, cR = R.c;
  const S l0 = entropy_fix(thetaf, thetaL, thetaR);
  const S l3 = entropy_fix(thetaf + c, thetaL + cL, thetaR + cR);
  const S l4 = entropy_fix(thetaf - c, thetaL - cL, thetaR - cR);

  const S d0 = QR[0] - QL[0], d1 = QR[1] - QL[1], d2 = QR[2] - QL[2], d3 = QR[3] - QL[3], d4 = QR[4] - QL[4];

  // |A| dQ = T |L| Tinv dQ.  The three entropy/shear columns of T share the
  // eigenvalue l0, so the product is l0 dQ + (l3 - l0) P+ dQ + (l4 - l0) P- dQ
  // with P+/- the projectors on the two acoustic eigenvectors
  // r+/- = (1, u +/- c n, h +/- c theta): the same value as the reference's
  // two 5x5 products (any basis of the l0 eigenspace gives it), in about a
  // third of the operations.  P+/- dQ = a+/- r+/- with
  // a+/- = (dp +/- c rho dVn) / (2 c^2), where rho dVn = n.d(rho u) - theta d(rho)
  // and dp = (gamma - 1)(d(rho E) - u.d(rho u) + |u|^2/2 d(rho)) at the Roe state.
  const S rdvn = (nx * d1 + ny * d2 + nz * d3) - thetaf * d0;
  const S dp = gm1 * (d4 - (u * d1 + v * d2 + w * d3) + v2h * d0);
  const S hic2 = halve(ic2);
  const S ap3 = (l3 - l0) * ((dp + c * rdvn) * hic2);
  const S ap4 = (l4 - l0) * ((dp - c * rdvn) * hic2);
  const S sp = ap3 + ap4, sm = c * (ap3 - ap4);
  const S dr0 = l0 * d0 + sp;
  const S dr1 = l0 * d1 + (u * sp + nx * sm);
  const S dr2 = l0 * d2 + (v * sp + ny * sm);
  const S dr3 = l0 * d3 + (w * sp + nz * sm);
  const S dr4 = l0 * d4 + (h * sp + thetaf * sm);

  // physical fluxes (Flux, :686)
  const S rtL = rL * thetaL, rtR = rR * thetaR;
  const S ha = halve(area);
  flux[0] = ha * (rtL + rtR - dr0);
  flux[1] = ha * ((uL * rtL + PL * nx) + (uR * rtR + PR * nx) - dr1);
  flux[2] = ha * ((vL * rtL + PL * ny) + (vR * rtR + PR * ny) - dr2);
  flux[3] = ha * ((wL * rtL + PL * nz) + (wR * rtR + PR * nz) - dr3);
  flux[4] = ha * (hL * rtL + hR * rtR - dr4);
  const S zero = Sc<S>::c(0.0), tiny = Sc<S>::c(1.0e-10);
  return ((rL < zero || EL < tiny || PL < tiny) ? 1 : 0) | ((rR < zero || ER < tiny || PR < tiny) ? 2 : 0) |
         ((P < tiny || rE < tiny) ? 4 : 0);
}

// ComputeAuxiliaryVariables (ucs/compressible.tcc:1230) on a 10-wide FP64 record
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
template <class S>
__device__ __forceinline__ S sutherland(S T, S S_) {
  return (Sc<S>::c(1.0) + S_) * (T * sqrt(T)) / (T + S_);
}

// ViscousFlux (ucs/compressible.tcc:713) for laminar flow (mut = 0).
// (u, v, w, T): the face-averaged state; grad: 27-wide face gradient;
// rk = area / ReTilde.
template <class S>
__device__ __forceinline__ void viscous_flux(const S u, const S v, const S w, const S T, const S* grad, const S nx,
                                             const S ny, const S nz, const S rk, const S Sconst, const S cp_over_pr,
                                             S* flux) {
  const S Tx = grad[15], Ty = grad[16], Tz = grad[17];
  const S ux = grad[18], uy = grad[19], uz = grad[20];
  const S vx = grad[21], vy = grad[22], vz = grad[23];
  const S wx = grad[24], wy = grad[25], wz = grad[26];
  const S two = Sc<S>::c(2.0);
  const S mu = sutherland(T, Sconst);
  const S fact = Sc<S>::c(-2.0 / 3.0) * (ux + vy + wz);
  const S tauxx = twice(ux) + fact, tauyy = twice(vy) + fact, tauzz = twice(wz) + fact;
  const S tauxy = uy + vx, tauxz = uz + wx, tauyz = vz + wy;
  const S RKT = rk * mu;
  const S c1 = -(mu * cp_over_pr);
  const S Tn = Tx * nx + Ty * ny + Tz * nz;
  const S tauxn = tauxx * nx + tauxy * ny + tauxz * nz;
  const S tauyn = tauxy * nx + tauyy * ny + tauyz * nz;
  const S tauzn = tauxz * nx + tauyz * ny + tauzz * nz;
  flux[0] = Sc<S>::c(0.0);
  flux[1] = -RKT * tauxn;
  flux[2] = -RKT * tauyn;
  flux[3] = -RKT * tauzn;
  flux[4] = -RKT * (tauxn * u + tauyn * v + tauzn * w) + rk * c1 * Tn;
}

}  // namespace pcfd
