// Implicit part of the path on sm_103a: Jacobian assembly into device block
// CRS, block LU of the diagonal, block Gauss-Seidel sweeps, the Newton
// update and the local time step.  Included by solver.cu inside its
// anonymous namespace (it uses the Solver state and the residual kernels).
//
// Block CRS layout: the reference's (CRSMatrix::Init, ucs/crsmatrix.tcc:48):
// row i = diagonal block first, then its psp neighbours in psp order; blocks
// are 5x5 row-major.  Off-diagonal blocks are stored in the Jacobian
// precision T (double, float or bfloat16); the diagonal is kept in FP64 in a
// separate array, before (d_diag) and after (d_dlu + pivots) its LU.
#pragma once

// (cuda_bf16.h is included by solver.cu at file scope)

template <class T>
__device__ __forceinline__ T to_store(double v);
template <>
__device__ __forceinline__ double to_store<double>(double v) { return v; }
template <>
__device__ __forceinline__ float to_store<float>(double v) { return (float)v; }
template <>
__device__ __forceinline__ __nv_bfloat16 to_store<__nv_bfloat16>(double v) { return __double2bfloat16(v); }

__device__ __forceinline__ double ld_blk(const double* p) { return *p; }
__device__ __forceinline__ double ld_blk(const float* p) { return (double)*p; }
__device__ __forceinline__ double ld_blk(const __nv_bfloat16* p) { return (double)__bfloat162float(*p); }
__device__ __forceinline__ float ld_blkf(const double* p) { return (float)*p; }
__device__ __forceinline__ float ld_blkf(const float* p) { return *p; }
__device__ __forceinline__ float ld_blkf(const __nv_bfloat16* p) { return __bfloat162float(*p); }

// NumericalFlux with the NaN kneecap (ucs/eqnset.tcc:55-90), Roe flux
__device__ __forceinline__ void numflux(const double* QL, const double* QR, const D4& a, double gamma, double* f,
                                        unsigned long long* health) {
  roe_flux(QL, QR, a.x, a.y, a.z, a.w, gamma, gamma - 1.0, 1.0 / gamma, 1.0 / (gamma - 1.0), f);
  if (kneecap5(f)) atomicAdd(&health[H_KNEECAP], 1ull);
}

// CompressibleEqnSet::ViscousJacobian (ucs/compressible.tcc:1633), laminar,
// in the scalar type R (FP64; FP32 when the blocks are stored in FP32 or BF16).
// QL/QR are the nodal 10-wide records (their stored pressure is used, as
// GetPressure reads it); aL/aR are the left/right blocks with the sign the
// reference scatters them with.
template <class R>
__device__ void viscous_jacobian(const R* QL, const R* QR, const R* dx, R s2, R ax, R ay, R az, R aw, R gamma, R Pr,
                                 R inv_retilde, R S, R* aL, R* aR) {
  const R half = R(0.5), one = R(1.0), two = R(2.0);
  R Q0 = half * (QL[0] + QR[0]), Q1 = half * (QL[1] + QR[1]), Q2 = half * (QL[2] + QR[2]),
         Q3 = half * (QL[3] + QR[3]), Q4 = half * (QL[4] + QR[4]);
  R gm1 = gamma - one;
  R iQ0 = one / Q0;
  R ua = Q1 * iQ0, va = Q2 * iQ0, wa = Q3 * iQ0;
  R Pa = gm1 * (Q4 - half * Q0 * (ua * ua + va * va + wa * wa));
  R Ta = gamma * Pa * iQ0;
  R mu = sutherland(Ta, S);
  R RK = aw * inv_retilde;
  R RKT = RK * mu;
  R rhoL = QL[0], uL = QL[1] / rhoL, vL = QL[2] / rhoL, wL = QL[3] / rhoL, PL = QL[6];
  R rhoR = QR[0], uR = QR[1] / rhoR, vR = QR[2] / rhoR, wR = QR[3] / rhoR, PR = QR[6];
  R u = half * (uL + uR), v = half * (vL + vR), w = half * (wL + wR);
  R DxL[3], DxR[3];
  for (int i = 0; i < 3; i++) {
    DxL[i] = -dx[i] / (rhoL * s2);
    DxR[i] = dx[i] / (rhoR * s2);
  }
  const R c43 = R(4.0 / 3.0), mc23 = R(-2.0 / 3.0);
  R cp = one / gm1;
  R c1 = -(mu / Pr * cp);
  for (int side = 0; side < 2; side++) {
    const R* D = side ? DxR : DxL;
    R* A = side ? aR : aL;
    R rho = side ? rhoR : rhoL, P = side ? PR : PL;
    R us = side ? uR : uL, vs = side ? vR : vL, ws = side ? wR : wL;
    R dux = -u * D[0], duy = -u * D[1], duz = -u * D[2];
    R dvx = -v * D[0], dvy = -v * D[1], dvz = -v * D[2];
    R dwx = -w * D[0], dwy = -w * D[1], dwz = -w * D[2];
    R dfact = R(-2.0 / 3.0) * (dux + dvy + dwz);
    R dtxx = (two * dux + dfact), dtyy = (two * dvy + dfact), dtzz = (two * dwz + dfact);
    R dtxy = duy + dvx, dtxz = duz + dwx, dtyz = dvz + dwy;
    R dtxn = dtxx * ax + dtxy * ay + dtxz * az;
    R dtyn = dtxy * ax + dtyy * ay + dtyz * az;
    R dtzn = dtxz * ax + dtyz * ay + dtzz * az;
    R r2u = (c43 * D[0] * ax + D[1] * ay + D[2] * az);
    R r2v = (mc23 * D[1] * ax + D[0] * ay);
    R r2w = (mc23 * D[2] * ax + D[0] * az);
    R r3u = (mc23 * D[0] * ay + D[1] * ax);
    R r3v = (D[0] * ax + c43 * D[1] * ay + D[2] * az);
    R r3w = (mc23 * D[2] * ay + D[1] * az);
    R r4u = (mc23 * D[0] * az + D[2] * ax);
    R r4v = (mc23 * D[1] * az + D[2] * ay);
    R r4w = (D[0] * ax + D[1] * ay + c43 * D[2] * az);
    A[0] = A[1] = A[2] = A[3] = A[4] = R(0);
    A[5] = -RKT * dtxn; A[6] = -RKT * r2u; A[7] = -RKT * r2v; A[8] = -RKT * r2w; A[9] = R(0);
    A[10] = -RKT * dtyn; A[11] = -RKT * r3u; A[12] = -RKT * r3v; A[13] = -RKT * r3w; A[14] = R(0);
    A[15] = -RKT * dtzn; A[16] = -RKT * r4u; A[17] = -RKT * r4v; A[18] = -RKT * r4w; A[19] = R(0);
    R v2 = (us * us + vs * vs + ws * ws);
    R dT_dP = gamma / rho;
    R dP_dr = +gm1 * half * v2, dP_dru = -gm1 * us, dP_drv = -gm1 * vs, dP_drw = -gm1 * ws, dP_dret = +gm1;
    R Tn = (D[0] * ax + D[1] * ay + D[2] * az) * dT_dP * c1;
    A[20] = -RKT * (dtxn * u + dtyn * v + dtzn * w) + RK * Tn * (dP_dr - P / rho);
    A[21] = -RKT * (r2u * u + r3u * v + r4u * w) + RK * Tn * dP_dru;
    A[22] = -RKT * (r2v * u + r3v * v + r4v * w) + RK * Tn * dP_drv;
    A[23] = -RKT * (r2w * u + r3w * v + r4w * w) + RK * Tn * dP_drw;
    A[24] = RK * Tn * dP_dret;
  }
  for (int i = 0; i < 25; i++) aL[i] = -aL[i];
}

struct JacConst {
  double gamma, Pr, inv_retilde, S;
  int viscous;
};

// Kernel_NumJac (ucs/jacobian.tcc:254): one-sided finite differences of the
// Roe flux (h = 1e-8, 11 flux evaluations per edge) into A(R,L) and A(L,R),
// plus Kernel_Viscous_Jac (:734) when viscous.
// q is the state the inviscid differences see (the state before the boundary
// conditions: ComputeSpatialJacobian runs Kernel_NumJac before Bkernel_NumJac
// applies them, ucs/jacobian.tcc:186-188); qv the state after them, which
// the viscous blocks see (Kernel_Viscous_Jac runs after, :190-194).
template <class T>
__global__ void __launch_bounds__(128) k_jac_edge(int nedge, const int2* __restrict__ en, const D4* __restrict__ ea,
                                                  const double* __restrict__ eh, const double* __restrict__ q,
                                                  const double* __restrict__ qv,
                                                  const int* __restrict__ pos_lr, const int* __restrict__ pos_rl,
                                                  JacConst k, T* __restrict__ M, unsigned long long* health) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nedge) return;
  const int2 n = en[e];
  const D4 a = ea[e];
  double QL[NVARS], QR[NVARS];
#pragma unroll
  for (int t = 0; t < NVARS; t++) { QL[t] = q[(size_t)n.x * NVARS + t]; QR[t] = q[(size_t)n.y * NVARS + t]; }
  const double h = 1.0e-8;
  const double ih = 1.0 / h;
  const double g = k.gamma, gm1 = k.gamma - 1.0, ig = 1.0 / k.gamma;
  // each perturbation changes one side; the other side's primitives are reused
  const RoeSide<double> sL = roe_side(QL, a.x, a.y, a.z, g, gm1), sR = roe_side(QR, a.x, a.y, a.z, g, gm1);
  double fS[NEQN];
  roe_core(sL, sR, QL, QR, a.x, a.y, a.z, a.w, g, gm1, ig, fS);
  if (kneecap5(fS)) atomicAdd(&health[H_KNEECAP], 1ull);
  double tL[25], tR[25];
  for (int i = 0; i < NEQN; i++) {
    double QP[NEQN], fP[NEQN];
#pragma unroll
    for (int t = 0; t < NEQN; t++) QP[t] = QL[t];
    QP[i] += h;
    roe_core(roe_side(QP, a.x, a.y, a.z, g, gm1), sR, QP, QR, a.x, a.y, a.z, a.w, g, gm1, ig, fP);
    if (kneecap5(fP)) atomicAdd(&health[H_KNEECAP], 1ull);
#pragma unroll
    for (int j = 0; j < NEQN; j++) tL[j * 5 + i] = (fS[j] - fP[j]) * ih;
#pragma unroll
    for (int t = 0; t < NEQN; t++) QP[t] = QR[t];
    QP[i] += h;
    roe_core(sL, roe_side(QP, a.x, a.y, a.z, g, gm1), QL, QP, a.x, a.y, a.z, a.w, g, gm1, ig, fP);
    if (kneecap5(fP)) atomicAdd(&health[H_KNEECAP], 1ull);
#pragma unroll
    for (int j = 0; j < NEQN; j++) tR[j * 5 + i] = (fP[j] - fS[j]) * ih;
  }
  if (k.viscous) {
    double dx[3] = {2.0 * eh[3 * (size_t)e], 2.0 * eh[3 * (size_t)e + 1], 2.0 * eh[3 * (size_t)e + 2]};
    double s2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
    double vL[25], vR[25];
#pragma unroll
    for (int t = 0; t < NVARS; t++) {
      QL[t] = qv[(size_t)n.x * NVARS + t];
      QR[t] = qv[(size_t)n.y * NVARS + t];
    }
    viscous_jacobian<double>(QL, QR, dx, s2, a.x, a.y, a.z, a.w, k.gamma, k.Pr, k.inv_retilde, k.S, vL, vR);
#pragma unroll
    for (int t = 0; t < 25; t++) { tL[t] += vL[t]; tR[t] += vR[t]; }
  }
  T* bl = &M[(size_t)pos_rl[e] * 25];  // A(R, L)
  T* br = &M[(size_t)pos_lr[e] * 25];  // A(L, R)
#pragma unroll
  for (int t = 0; t < 25; t++) { bl[t] = to_store<T>(tL[t]); br[t] = to_store<T>(tR[t]); }
}

// The same differences with the eleven Roe flux evaluations in double-float
// (the residual's alternative arithmetic, on the FP32 pipes).  A flux
// carries ~2^-48 relative error there, so the quotient over h = 1e-8 has
// ~1e-6 relative error: the Jacobian is only the Newton iteration matrix,
// the residual (evaluated separately) decides the converged answer.  The
// analytic viscous blocks stay FP64.
// difference quotient of two double-float fluxes in the block type's
// arithmetic (h = 1e-8, whose reciprocal 1e8 is exact in FP32)
__device__ __forceinline__ double df_quot(dfl d, double) { return to_dbl(d) * 1.0e8; }
__device__ __forceinline__ float df_quot(dfl d, float) { return __fmul_rn(__fadd_rn(d.hi, d.lo), 1.0e8f); }
__device__ __forceinline__ __nv_bfloat16 store_blk(__nv_bfloat16*, float v) { return __float2bfloat16(v); }
__device__ __forceinline__ float store_blk(float*, float v) { return v; }
__device__ __forceinline__ double store_blk(double*, double v) { return v; }

template <class T>
__global__ void __launch_bounds__(128, 3) k_jac_edge_df(int nedge, const int2* __restrict__ en,
                                                     const D4* __restrict__ ea, const double* __restrict__ eh,
                                                     const double* __restrict__ q, const double* __restrict__ qv,
                                                     const int* __restrict__ pos_lr,
                                                     const int* __restrict__ pos_rl, JacConst k, T* __restrict__ M,
                                                     unsigned long long* health) {
  // FP64 blocks keep FP64 quotients and viscous blocks; FP32 and BF16
  // blocks get them in FP32, so no FP64 instruction is spent on a value
  // that is rounded to FP32 or coarser anyway
  typedef typename std::conditional<std::is_same<T, double>::value, double, float>::type VR;
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nedge) return;
  const int2 n = en[e];
  const D4 a = ea[e];
  dfl QL[NEQN], QR[NEQN];
#pragma unroll
  for (int t = 0; t < NEQN; t++) {
    QL[t] = to_df(q[(size_t)n.x * NVARS + t]);
    QR[t] = to_df(q[(size_t)n.y * NVARS + t]);
  }
  const dfl nx = to_df(a.x), ny = to_df(a.y), nz = to_df(a.z), ar = to_df(a.w);
  const dfl g = to_df(k.gamma), gm1 = to_df(k.gamma - 1.0), ig = to_df(1.0 / k.gamma);
  const dfl h = to_df(1.0e-8);
  // each perturbation changes one side; the other side's primitives are reused
  const RoeSide<dfl> sL = roe_side(QL, nx, ny, nz, g, gm1), sR = roe_side(QR, nx, ny, nz, g, gm1);
  dfl fS[NEQN];
  roe_core(sL, sR, QL, QR, nx, ny, nz, ar, g, gm1, ig, fS);
  if (kneecap5(fS)) atomicAdd(&health[H_KNEECAP], 1ull);
  VR tL[25], tR[25];
  for (int i = 0; i < NEQN; i++) {
    dfl QP[NEQN], fP[NEQN];
#pragma unroll
    for (int t = 0; t < NEQN; t++) QP[t] = QL[t];
    QP[i] = QP[i] + h;
    roe_core(roe_side(QP, nx, ny, nz, g, gm1), sR, QP, QR, nx, ny, nz, ar, g, gm1, ig, fP);
    if (kneecap5(fP)) atomicAdd(&health[H_KNEECAP], 1ull);
#pragma unroll
    for (int j = 0; j < NEQN; j++) tL[j * 5 + i] = df_quot(fS[j] - fP[j], VR(0));
#pragma unroll
    for (int t = 0; t < NEQN; t++) QP[t] = QR[t];
    QP[i] = QP[i] + h;
    roe_core(sL, roe_side(QP, nx, ny, nz, g, gm1), QL, QP, nx, ny, nz, ar, g, gm1, ig, fP);
    if (kneecap5(fP)) atomicAdd(&health[H_KNEECAP], 1ull);
#pragma unroll
    for (int j = 0; j < NEQN; j++) tR[j * 5 + i] = df_quot(fP[j] - fS[j], VR(0));
  }
  if (k.viscous) {
    VR QLv[NVARS], QRv[NVARS];
#pragma unroll
    for (int t = 0; t < NVARS; t++) {
      QLv[t] = (VR)qv[(size_t)n.x * NVARS + t];
      QRv[t] = (VR)qv[(size_t)n.y * NVARS + t];
    }
    VR dx[3] = {(VR)(2.0 * eh[3 * (size_t)e]), (VR)(2.0 * eh[3 * (size_t)e + 1]), (VR)(2.0 * eh[3 * (size_t)e + 2])};
    VR s2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
    VR vL[25], vR[25];
    viscous_jacobian<VR>(QLv, QRv, dx, s2, (VR)a.x, (VR)a.y, (VR)a.z, (VR)a.w, (VR)k.gamma, (VR)k.Pr,
                         (VR)k.inv_retilde, (VR)k.S, vL, vR);
#pragma unroll
    for (int t = 0; t < 25; t++) { tL[t] += vL[t]; tR[t] += vR[t]; }
  }
  T* bl = &M[(size_t)pos_rl[e] * 25];  // A(R, L)
  T* br = &M[(size_t)pos_lr[e] * 25];  // A(L, R)
#pragma unroll
  for (int t = 0; t < 25; t++) { bl[t] = store_blk(bl, tL[t]); br[t] = store_blk(br, tR[t]); }
}

// The differences of one boundary half-edge from its post-condition states
// QL, QR (Bkernel_NumJac's loop, ucs/jacobian.tcc:470-520).
__device__ void jac_bedge_fd(int he, int bct, const D4 a, double Tw, const double* nQ, const BcConst& bk, int beval,
                             const double* QL, const double* QR, double* __restrict__ bblk,
                             unsigned long long* health) {
  const double h = 1.0e-8;
  const double ih = 1.0 / h;
  double fS[NEQN];
  if (beval == 3) {
    // base state through the same boundary-condition map as the perturbed ones
    double QBL[NVARS], QBR[NVARS];
    for (int t = 0; t < NVARS; t++) { QBL[t] = QL[t]; QBR[t] = QR[t]; }
    apply_bc(bk, bct, QBL, QBR, a, Tw, nQ);
    numflux(QBL, QBR, a, bk.gamma, fS, health);
  } else {
    numflux(QL, QR, a, bk.gamma, fS, health);
  }
  double* out = &bblk[(size_t)he * 25];
  for (int i = 0; i < NEQN; i++) {
    double QPL[NVARS], QPR[NVARS], fL[NEQN];
    for (int t = 0; t < NVARS; t++) { QPL[t] = QL[t]; QPR[t] = QR[t]; }
    QPL[i] += h;
    aux_vars(bk.gamma, QPL);
    aux_vars(bk.gamma, QPR);
    if (beval != 1) apply_bc(bk, bct, QPL, QPR, a, Tw, nQ);
    numflux(QPL, QPR, a, bk.gamma, fL, health);
    for (int j = 0; j < NEQN; j++) out[j * 5 + i] = (fL[j] - fS[j]) * ih;
  }
}

// The node and phantom states one boundary half-edge of Bkernel_NumJac
// (ucs/jacobian.tcc:459) works on.  Thread t < nind takes an independent
// half-edge (its node has no hard-setting condition); the rest take slot
// p = t - nind of a hard-set node's ordered list, whose earlier slots'
// hard sets are replayed on the node state first - the reference applies the
// conditions in place, half-edge after half-edge, before each difference.
// The states are read from q as it was before this pass.
struct BedgeSlots {
  int nind;
  const int* ind;     // [nind] independent half-edges
  const int* slot_group, *gnode, *gptr, *ghe;
};

__device__ __forceinline__ int bedge_states(const BedgeSlots& sl, int t, const BcConst& k, const int2* __restrict__ bn,
                                            const int* __restrict__ bbc, const double* __restrict__ btw,
                                            const int* __restrict__ bnrm, const double* __restrict__ q, double* QL,
                                            double* QR) {
  int he;
  if (t < sl.nind) {
    he = sl.ind[t];
    for (int j = 0; j < NVARS; j++) QL[j] = q[(size_t)bn[he].x * NVARS + j];
  } else {
    const int p = t - sl.nind;
    he = sl.ghe[p];
    const int g = sl.slot_group[p];
    for (int j = 0; j < NVARS; j++) QL[j] = q[(size_t)sl.gnode[g] * NVARS + j];
    replay_group(k, sl.gptr[g], p, sl.ghe, bn, bbc, btw, bnrm, q, QL);
  }
  for (int j = 0; j < NVARS; j++) QR[j] = q[(size_t)bn[he].y * NVARS + j];
  return he;
}

// Bkernel_NumJac (ucs/jacobian.tcc:459) with jacobianBoundaryEval = 0: the
// condition is applied to the half-edge's states (CalculateBoundaryVariables,
// which the reference runs inside this kernel), the phantom state is
// re-derived from each perturbed interior state through the condition, and
// the difference quotient goes to the diagonal.
__global__ void __launch_bounds__(128) k_jac_bedge(int nthreads, BedgeSlots sl, const int2* __restrict__ bn,
                                                   const D4* __restrict__ ba, const int* __restrict__ bbc,
                                                   const double* __restrict__ btw, const int* __restrict__ bnrm,
                                                   BcConst bk, int beval, const double* __restrict__ q,
                                                   double* __restrict__ bblk, unsigned long long* health) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nthreads) return;
  double QL[NVARS], QR[NVARS], nQ[NVARS];
  const int he = bedge_states(sl, t, bk, bn, bbc, btw, bnrm, q, QL, QR);
  const D4 a = ba[he];
  const int bct = bbc[he];
  for (int j = 0; j < NVARS; j++) nQ[j] = 0.0;
  if (bct == PCFD_BC_NOSLIP && bnrm[he] >= 0)
    for (int j = 0; j < NVARS; j++) nQ[j] = q[(size_t)bnrm[he] * NVARS + j];
  if (!apply_bc(bk, bct, QL, QR, a, btw[he], nQ)) atomicAdd(&health[H_BADBC], 1ull);
  jac_bedge_fd(he, bct, a, btw[he], nQ, bk, beval, QL, QR, bblk, health);
}

// One thread walking the half-edges in order on a private copy of the state
// (the exact reference order when a no-slip normal node is itself hard-set
// by a condition, so a condition reads a state an earlier one wrote).
__global__ void k_jac_bedge_sequential(int nbedge, const int2* __restrict__ bn, const D4* __restrict__ ba,
                                       const int* __restrict__ bbc, const double* __restrict__ btw,
                                       const int* __restrict__ bnrm, BcConst bk, int beval, double* __restrict__ qw,
                                       double* __restrict__ bblk, unsigned long long* health) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int he = 0; he < nbedge; he++) {
    const int2 n = bn[he];
    double* QL = &qw[(size_t)n.x * NVARS];
    double* QR = &qw[(size_t)n.y * NVARS];
    double nQ[NVARS];
    const int bct = bbc[he];
    for (int j = 0; j < NVARS; j++) nQ[j] = 0.0;
    if (bct == PCFD_BC_NOSLIP && bnrm[he] >= 0)
      for (int j = 0; j < NVARS; j++) nQ[j] = qw[(size_t)bnrm[he] * NVARS + j];
    if (!apply_bc(bk, bct, QL, QR, ba[he], btw[he], nQ)) atomicAdd(&health[H_BADBC], 1ull);
    double L[NVARS], R[NVARS];
    for (int j = 0; j < NVARS; j++) { L[j] = QL[j]; R[j] = QR[j]; }
    jac_bedge_fd(he, bct, ba[he], btw[he], nQ, bk, beval, L, R, bblk, health);
  }
}

// The boundary-condition map and auxiliary variables in double-float, for
// the double-float form of the boundary Jacobian below (the same operations
// as apply_bc and aux_vars).
__device__ __forceinline__ void aux_vars_df(dfl gamma, dfl* Q) {
  const dfl one = Sc<dfl>::c(1.0), half = Sc<dfl>::c(0.5);
  const dfl gm1 = gamma - one;
  const dfl ir = one / Q[0];
  const dfl u = Q[1] * ir, v = Q[2] * ir, w = Q[3] * ir;
  const dfl P = gm1 * (Q[4] - half * Q[0] * (u * u + v * v + w * w));
  Q[6] = P;
  Q[5] = gamma * P * ir;
  Q[7] = u;
  Q[8] = v;
  Q[9] = w;
}

__device__ int apply_bc_df(int bct, dfl gamma, int no_cvbc, const dfl* qinf, dfl* QL, dfl* QR, dfl ax, dfl ay, dfl az,
                           dfl Tw, const dfl* nQ) {
  const dfl zero = Sc<dfl>::c(0.0), one = Sc<dfl>::c(1.0);
  switch (bct) {
    case PCFD_BC_SONIC_INFLOW:
    case PCFD_BC_DIRICHLET:
      for (int i = 0; i < NVARS; i++) QR[i] = QL[i] = qinf[i];
      break;
    case PCFD_BC_SONIC_OUTFLOW:
    case PCFD_BC_NEUMANN:
      for (int i = 0; i < NEQN; i++) QR[i] = QL[i];
      break;
    case PCFD_BC_FARFIELD:
      bc_farfield<dfl>(gamma, qinf, QL, QL[6], QR, ax, ay, az);
      break;
    case PCFD_BC_IMPERMEABLE_WALL:
    case PCFD_BC_SYMMETRY:
      bc_inviscid_wall<dfl>(gamma, no_cvbc, QL, QL[6], QR, ax, ay, az);
      break;
    case PCFD_BC_NOSLIP:
      if (Tw < zero) {
        QR[0] = QL[0] = nQ[0];
        QR[4] = QL[4] = nQ[4];
      } else {
        const dfl gm1 = gamma - one;
        const dfl rhoEt = Tw * QL[0] / (gamma * gm1) + Sc<dfl>::c(0.5) * QR[0] * zero;
        QR[0] = QL[0];
        QR[4] = QL[4] = rhoEt;
      }
      QR[1] = QL[1] = QL[0] * zero;
      QR[2] = QL[2] = QL[0] * zero;
      QR[3] = QL[3] = QL[0] * zero;
      break;
    default:
      return 0;
  }
  aux_vars_df(gamma, QR);
  aux_vars_df(gamma, QL);
  return 1;
}

// Bkernel_NumJac in double-float: the six boundary-condition maps with their
// ten far-field or wall sub-iterations and the six Roe fluxes of a
// half-edge on the FP32 pipes; the difference quotients (FP64 diagonal
// contributions) carry ~1e-6 relative error, as in k_jac_edge_df.
__global__ void __launch_bounds__(128) k_jac_bedge_df(int nthreads, BedgeSlots sl, const int2* __restrict__ bn,
                                                      const D4* __restrict__ ba, const int* __restrict__ bbc,
                                                      const double* __restrict__ btw, const int* __restrict__ bnrm,
                                                      BcConst bk, int beval, const double* __restrict__ q,
                                                      double* __restrict__ bblk, unsigned long long* health) {
  const int tt = blockIdx.x * blockDim.x + threadIdx.x;
  if (tt >= nthreads) return;
  double QL0[NVARS], QR0[NVARS], nQ0[NVARS];
  const int he = bedge_states(sl, tt, bk, bn, bbc, btw, bnrm, q, QL0, QR0);
  const int bct = bbc[he];
  for (int t = 0; t < NVARS; t++) nQ0[t] = 0.0;
  if (bct == PCFD_BC_NOSLIP && bnrm[he] >= 0)
    for (int t = 0; t < NVARS; t++) nQ0[t] = q[(size_t)bnrm[he] * NVARS + t];
  // the condition on the stored state, in FP64 as the boundary update does
  if (!apply_bc(bk, bct, QL0, QR0, ba[he], btw[he], nQ0)) atomicAdd(&health[H_BADBC], 1ull);
  const D4 a = ba[he];
  dfl QL[NVARS], QR[NVARS], nQ[NVARS], qinf[NVARS];
  for (int t = 0; t < NVARS; t++) {
    QL[t] = to_df(QL0[t]);
    QR[t] = to_df(QR0[t]);
    qinf[t] = to_df(bk.qinf[t]);
    nQ[t] = to_df(nQ0[t]);
  }
  const dfl gamma = to_df(bk.gamma), gm1 = to_df(bk.gamma - 1.0), ig = to_df(1.0 / bk.gamma),
            igm1 = to_df(1.0 / (bk.gamma - 1.0));
  const dfl ax = to_df(a.x), ay = to_df(a.y), az = to_df(a.z), aw = to_df(a.w), Tw = to_df(btw[he]);
  const dfl h = to_df(1.0e-8);
  dfl fS[NEQN];
  if (beval == 3) {
    dfl QBL[NVARS], QBR[NVARS];
    for (int t = 0; t < NVARS; t++) { QBL[t] = QL[t]; QBR[t] = QR[t]; }
    apply_bc_df(bct, gamma, bk.no_cvbc, qinf, QBL, QBR, ax, ay, az, Tw, nQ);
    roe_flux<dfl>(QBL, QBR, ax, ay, az, aw, gamma, gm1, ig, igm1, fS);
  } else {
    roe_flux<dfl>(QL, QR, ax, ay, az, aw, gamma, gm1, ig, igm1, fS);
  }
  if (kneecap5(fS)) atomicAdd(&health[H_KNEECAP], 1ull);
  double* out = &bblk[(size_t)he * 25];
  for (int i = 0; i < NEQN; i++) {
    dfl QPL[NVARS], QPR[NVARS], fL[NEQN];
    for (int t = 0; t < NVARS; t++) { QPL[t] = QL[t]; QPR[t] = QR[t]; }
    QPL[i] = QPL[i] + h;
    aux_vars_df(gamma, QPL);
    aux_vars_df(gamma, QPR);
    if (beval != 1) apply_bc_df(bct, gamma, bk.no_cvbc, qinf, QPL, QPR, ax, ay, az, Tw, nQ);
    roe_flux<dfl>(QPL, QPR, ax, ay, az, aw, gamma, gm1, ig, igm1, fL);
    if (kneecap5(fL)) atomicAdd(&health[H_KNEECAP], 1ull);
    for (int j = 0; j < NEQN; j++) out[j * 5 + i] = to_dbl(fL[j] - fS[j]) * 1.0e8;
  }
}

// Diagonal blocks: boundary contributions in half-edge order, minus the
// column of off-diagonal blocks in edge order (Kernel_Diag_NumJac,
// ucs/jacobian.tcc:437), plus vol/dtau on the diagonal
// (EqnSet::ContributeTemporalTerms, ucs/eqnset.tcc:195, steady: cnp1 = 1).
template <class T>
__global__ void __launch_bounds__(128) k_jac_diag(int nnode, const int* __restrict__ nptr, const int* __restrict__ nedg,
                                                  const int* __restrict__ pos_lr, const int* __restrict__ pos_rl,
                                                  const int* __restrict__ bptr, const int* __restrict__ bhe,
                                                  const double* __restrict__ bblk, const T* __restrict__ M,
                                                  const double* __restrict__ vol, const double* __restrict__ dt,
                                                  double* __restrict__ diag) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nnode) return;
  double D[25];
#pragma unroll
  for (int t = 0; t < 25; t++) D[t] = 0.0;
  for (int p = bptr[i]; p < bptr[i + 1]; p++) {
    const double* B = &bblk[(size_t)bhe[p] * 25];
#pragma unroll
    for (int t = 0; t < 25; t++) D[t] += B[t];
  }
  for (int k = nptr[i]; k < nptr[i + 1]; k++) {
    int se = nedg[k];
    // column block A(j, i): i is the left node -> A(R, L); else A(L, R)
    const T* A = (se < 0) ? &M[(size_t)pos_rl[~se] * 25] : &M[(size_t)pos_lr[se] * 25];
#pragma unroll
    for (int t = 0; t < 25; t++) D[t] += -ld_blk(&A[t]);
  }
  double vd = 1.0 * vol[i] / dt[i];
#pragma unroll
  for (int r = 0; r < NEQN; r++) D[r * 5 + r] += vd;
#pragma unroll
  for (int t = 0; t < 25; t++) diag[(size_t)i * 25 + t] = D[t];
}

// LU (ucs/matrix.h:111) in place with row pivots, on a 5x5 block.
__device__ __forceinline__ int lu5(double* a, int* p) {
  int bad = 0, row = 0;
  for (int i = 0; i < 5; i++) p[i] = i;
  for (int i = 0; i < 5; i++) {
    double large = 0.0;
    for (int j = i; j < 5; j++)
      if (fabs(a[p[j] * 5 + i]) > fabs(large)) { large = a[p[j] * 5 + i]; row = j; }
    if (large == 0.0 || fabs(large) < 1.0e-15) bad = 1;
    int t = p[i]; p[i] = p[row]; p[row] = t;
    large = 1.0 / large;
    for (int j = i + 1; j < 5; j++) a[p[j] * 5 + i] *= large;
    for (int j = i + 1; j < 5; j++)
      for (int kk = i + 1; kk < 5; kk++) a[p[j] * 5 + kk] -= a[p[j] * 5 + i] * a[p[i] * 5 + kk];
  }
  return bad;
}

// No-slip row modifications (Bkernel_BC_Jac_Modify, ucs/bc.tcc:748 ->
// ModifyViscousWallJacobian, ucs/compressible.tcc:1577) on the node's own
// row, then PrepareSGS's LU of the diagonal (ucs/crsmatrix.tcc:840).
template <class T>
__global__ void __launch_bounds__(128) k_jac_finish(int nnode, const int* __restrict__ ia, const int* __restrict__ ja,
                                                    const int* __restrict__ bptr, const int* __restrict__ bhe,
                                                    const int* __restrict__ bbc, const double* __restrict__ btw,
                                                    const int* __restrict__ bnrm, double gamma, T* __restrict__ M,
                                                    double* __restrict__ diag, double* __restrict__ dlu,
                                                    int* __restrict__ piv, unsigned long long* health) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nnode) return;
  double D[25];
#pragma unroll
  for (int t = 0; t < 25; t++) D[t] = diag[(size_t)i * 25 + t];
  bool mod = false;
  for (int p = bptr[i]; p < bptr[i + 1]; p++) {
    int he = bhe[p];
    if (bbc[he] != PCFD_BC_NOSLIP) continue;
    mod = true;
    double Tw = btw[he];
    int rows[5];
    int nr = 0;
    rows[nr++] = 1; rows[nr++] = 2; rows[nr++] = 3;
    if (Tw < 0.0) { rows[nr++] = 0; rows[nr++] = 4; }
    else rows[nr++] = 4;
    for (int rr = 0; rr < nr; rr++) {
      int sr = rows[rr];
      for (int b = ia[i] + 1; b < ia[i + 1]; b++)
        for (int c = 0; c < 5; c++) M[(size_t)b * 25 + sr * 5 + c] = to_store<T>(0.0);
      for (int c = 0; c < 5; c++) D[sr * 5 + c] = 0.0;
      D[sr * 5 + sr] = 1.0;
    }
    if (Tw < 0.0) {
      int nn = bnrm[he];
      for (int b = ia[i] + 1; b < ia[i + 1]; b++)
        if (ja[b] == nn) {
          M[(size_t)b * 25 + 0] = to_store<T>(-1.0);
          M[(size_t)b * 25 + 24] = to_store<T>(-1.0);
        }
    } else {
      D[4 * 5 + 0] = -(Tw / (gamma * (gamma - 1.0)) + 0.5 * 0.0);
    }
  }
  if (mod)
    for (int t = 0; t < 25; t++) diag[(size_t)i * 25 + t] = D[t];
  int pv[5];
  if (lu5(D, pv)) atomicAdd(&health[H_BADLU], 1ull);
  // store reciprocals of the U diagonal for the solves
#pragma unroll
  for (int r = 0; r < 5; r++) D[pv[r] * 5 + r] = 1.0 / D[pv[r] * 5 + r];
#pragma unroll
  for (int t = 0; t < 25; t++) dlu[(size_t)i * 25 + t] = D[t];
#pragma unroll
  for (int r = 0; r < 5; r++) piv[(size_t)i * 5 + r] = pv[r];
}

// LuSolve (ucs/matrix.h:238) with the U-diagonal reciprocals stored by
// k_jac_finish; b is overwritten with the solution.
__device__ __forceinline__ void lusolve5(const double* a, double* b, const int* p) {
  double x[5];
  for (int i = 0; i < 5; i++) {
    double sum = 0.0;
    for (int j = 0; j < i; j++) sum += a[p[i] * 5 + j] * x[j];
    x[i] = b[p[i]] - sum;
  }
  for (int i = 4; i >= 0; i--) {
    double sum = 0.0;
    for (int j = 4; j > i; j--) sum += a[p[i] * 5 + j] * b[j];
    b[i] = (x[i] - sum) * a[p[i] * 5 + i];
  }
}

// Explicit inverse of each LU-factored diagonal block, column c = LuSolve of
// the unit vector e_c, so that a sweep's diagonal solve is one 25-lane
// product instead of a serial substitution on one lane (FP64 runs at 2
// operations per clock per SM on GB300).  Same values as LuSolve in exact
// arithmetic; the rounding differs at the level of cond(D) * 1e-16.
__global__ void k_diag_inverse(int nnode, const double* __restrict__ dlu, const int* __restrict__ piv,
                               double* __restrict__ dinv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nnode) return;
  double a[25];
  int p[5];
#pragma unroll
  for (int t = 0; t < 25; t++) a[t] = dlu[(size_t)i * 25 + t];
#pragma unroll
  for (int r = 0; r < 5; r++) p[r] = piv[(size_t)i * 5 + r];
  for (int c = 0; c < 5; c++) {
    double b[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    b[c] = 1.0;
    lusolve5(a, b, p);
    for (int r = 0; r < 5; r++) dinv[(size_t)i * 25 + r * 5 + c] = b[r];
  }
}

// Arithmetic of the off-diagonal products: FP64 for the FP64 matrix; FP32
// for the FP32 and BF16 storage (whose coefficients carry FP32 or coarser
// rounding already), reading an FP32 copy of x, so that no per-coefficient
// FP64 instruction (a double-to-float conversion runs on the FP64 pipe) is
// left.  The diagonal blocks and the LU stay FP64.
template <class T>
struct OffAcc {
  typedef float type;
};
template <>
struct OffAcc<double> {
  typedef double type;
};
__device__ __forceinline__ double off_val(double a) { return a; }
__device__ __forceinline__ float off_val(float a) { return a; }
__device__ __forceinline__ float off_val(__nv_bfloat16 a) { return __bfloat162float(a); }

// Sum over lanes 5r .. 5r+4 of v, left in lane 5r (r = 0..4).
template <class A>
__device__ __forceinline__ A sum5(A v) {
  const unsigned full = 0xffffffffu;
  return v + __shfl_down_sync(full, v, 1) + __shfl_down_sync(full, v, 2) + __shfl_down_sync(full, v, 3) +
         __shfl_down_sync(full, v, 4);
}

// Off-diagonal part of a block row of A x.  The row's blocks are contiguous
// in CRS order, 25 coefficients each (row-major), so lane l < 25 takes
// coefficient (l / 5, l % 5) of every block: each warp load reads 25
// consecutive coefficients.  The row's column indices come in with one
// coalesced load (lane b holds block b's).  A row is handled in two phases
// so that a warp can overlap rows: row_issue starts the coefficient and x
// loads of the first 16 blocks (8 in FP64), row_finish consumes them (and walks any
// further blocks).  Lane 5r receives row r's sum.
// blocks whose loads are issued together: 16 in FP32, 8 in FP64 (registers)
template <class T>
struct RowBatch {
  static constexpr int n = sizeof(typename OffAcc<T>::type) == 8 ? 8 : 16;
};

// x gathers: through L1, or (CG) from L2 for kernels in which other blocks
// write x between reads (L1 is not coherent across SMs within a launch)
template <bool CG, class A>
__device__ __forceinline__ A ldx(const A* p) {
  if (CG) return __ldcg(p);
  return *p;
}

template <class T, bool CG = false>
__device__ __forceinline__ void row_issue(int b0, int nb, int jl, int lane, const T* __restrict__ M,
                                          const typename OffAcc<T>::type* __restrict__ xa,
                                          typename OffAcc<T>::type (&av)[RowBatch<T>::n],
                                          typename OffAcc<T>::type (&xv)[RowBatch<T>::n]) {
  constexpr int kRowBatch = RowBatch<T>::n;
  typedef typename OffAcc<T>::type A;
  const int c = lane % 5;
  const bool active = lane < 25;
#pragma unroll
  for (int u = 0; u < kRowBatch; u++) {
    const int j = __shfl_sync(0xffffffffu, jl, u);
    const bool ok = active && u < nb;
    av[u] = ok ? off_val(M[(size_t)(b0 + u) * 25 + lane]) : A(0);
    xv[u] = ok ? ldx<CG>(&xa[(size_t)j * 5 + c]) : A(0);
  }
}

template <class T, bool CG = false>
__device__ __forceinline__ typename OffAcc<T>::type row_finish(int b0, int nb, int jl, int lane,
                                                               const int* __restrict__ ja, const T* __restrict__ M,
                                                               const typename OffAcc<T>::type* __restrict__ xa,
                                                               const typename OffAcc<T>::type (&av)[RowBatch<T>::n],
                                                               const typename OffAcc<T>::type (&xv)[RowBatch<T>::n]) {
  typedef typename OffAcc<T>::type A;
  constexpr int kRowBatch = RowBatch<T>::n;
  A acc = A(0);
#pragma unroll
  for (int u = 0; u < kRowBatch; u++) acc = fma(av[u], xv[u], acc);
  // blocks past the first batch
  const int c = lane % 5;
  const bool active = lane < 25;
  for (int k = kRowBatch; k < nb; k++) {
    const int j = k < 32 ? __shfl_sync(0xffffffffu, jl, k & 31) : ja[b0 + k];
    if (active) acc = fma(off_val(M[(size_t)(b0 + k) * 25 + lane]), ldx<CG>(&xa[(size_t)j * 5 + c]), acc);
  }
  return sum5(acc);
}

// the next row's block range and column indices
__device__ __forceinline__ void row_meta(const int* __restrict__ ia, const int* __restrict__ ja, int i, int lane,
                                         int& b0, int& nb, int& jl) {
  b0 = ia[i] + 1;
  nb = ia[i + 1] - b0;
  jl = lane < nb ? ja[b0 + lane] : 0;
}

// FP64 copy of an FP32 vector
__global__ void k_f32_to_f64(long long n, const float* __restrict__ x, double* __restrict__ y) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = (double)x[i];
}

// FP32 copy of an FP64 vector (once per product or sweep)
__global__ void k_to_f32(long long n, const double* __restrict__ x, float* __restrict__ xf) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    xf[i] = (float)x[i];
}

// One colour of a block Gauss-Seidel sweep (CRS::SGS, ucs/crs.tcc:62):
// warps stride over the colour's rows; for each, rhs = b_i - sum_j A_ij x_j
// over the off-diagonal blocks, then x_i = D_i^-1 rhs as a 25-lane product
// with the stored inverse.  desc holds each row's (id, first off-diagonal
// block, block count) in colour order, read two rows ahead; while a row's
// coefficients are in flight the warp already loads the next row's column
// indices, so a row costs about one memory latency.  K is the vector type
// (FP64, or FP32 inside the FP32 Krylov solver); xa is x in the products'
// accumulation type (x itself, or its FP32 copy, which the sweep keeps
// current).  Rows of one colour share no block, so no row reads an x written
// in the same colour.  g is the warp's first row, W the number of warps.
template <class T, class K, bool CG>
__device__ __forceinline__ void sgs_rows(int nrows, const int4* __restrict__ desc, const int* __restrict__ ja,
                                         const T* __restrict__ M,
                                         const K* __restrict__ dinv, const K* __restrict__ b, K* x,
                                         typename OffAcc<T>::type* xa, int g, const int W) {
  typedef typename OffAcc<T>::type A;
  const int lane = threadIdx.x & 31;
  if (g >= nrows) return;
  const int4 none = make_int4(-1, 0, 0, 0);
  int4 d = desc[g];
  int i = d.x, b0 = d.y, nb = d.z;
  int jl = lane < nb ? ja[b0 + lane] : 0;
  int4 dn = g + W < nrows ? desc[g + W] : none;
  const int r = lane / 5, c = lane % 5;
  while (true) {
    A av[RowBatch<T>::n], xv[RowBatch<T>::n];
    row_issue<T, CG>(b0, nb, jl, lane, M, xa, av, xv);
    // the row's right-hand side and inverse diagonal block travel with its
    // coefficients instead of after the sum
    const K bi = (lane < 25 && c == 0) ? b[(size_t)i * 5 + r] : K(0);
    const K di = lane < 25 ? dinv[(size_t)i * 25 + lane] : K(0);
    const int4 dnn = g + 2 * W < nrows ? desc[g + 2 * W] : none;
    const int jln = (dn.x >= 0 && lane < dn.z) ? ja[dn.y + lane] : 0;
    const K s = (K)row_finish<T, CG>(b0, nb, jl, lane, ja, M, xa, av, xv);
    // rhs_r = b_r - s_r on lane 5r; lane l = 5r + c then forms D^-1[r][c] rhs_c
    const K rhs = (lane < 25 && c == 0) ? bi - s : K(0);
    const K rc = __shfl_sync(0xffffffffu, rhs, (5 * c) & 31);
    K v = di * rc;
    v = sum5(v);
    if (lane < 25 && c == 0) {
      x[(size_t)i * 5 + r] = v;
      if ((const void*)xa != (const void*)x) xa[(size_t)i * 5 + r] = (A)v;
    }
    if (dn.x < 0) break;
    g += W;
    i = dn.x;
    b0 = dn.y;
    nb = dn.z;
    jl = jln;
    dn = dnn;
  }
}


// Grid-wide barrier of a cooperative launch (all blocks co-resident): a
// counter and a generation word.  The wait is bounded; on time-out the
// block sets *err and the caller returns.
constexpr long long kBarrierSpins = 1LL << 22;

__device__ __forceinline__ bool grid_barrier(unsigned int* __restrict__ bar, unsigned int nblocks,
                                             int* __restrict__ err) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* gen = bar + 1;
    const unsigned int g0 = *gen;
    __threadfence();
    int ok = 1;
    if (atomicAdd(bar, 1u) == nblocks - 1) {
      atomicExch(bar, 0u);
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      long long spins = 0;
      while (*gen == g0) {
        if (++spins > kBarrierSpins) {
          atomicExch(err, 1);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

// Colour of phase p of symmetric sweeps (colours forward, then backward).
__device__ __forceinline__ int sgs_colour(int p, int ncolor) {
  const int cc = p % ncolor, dir = (p / ncolor) & 1;
  return dir == 0 ? cc : ncolor - 1 - cc;
}
// The phase after p, skipping a phase of the colour just swept (the last
// colour of a forward sweep opens the backward one, the first colour of a
// backward sweep opens the next forward one): a colour's rows read only
// other colours' x, unchanged in between, so the repeat would write the
// same values.
__device__ __forceinline__ int sgs_next_phase(int p, int nphase, int ncolor) {
  int q = p + 1;
  while (q < nphase && sgs_colour(q, ncolor) == sgs_colour(p, ncolor)) q++;
  return q;
}

// nsweeps symmetric sweeps (all colours forward, then backward) in one
// cooperative launch: the colours are separated by grid barriers instead of
// kernel boundaries, and x is gathered from L2.  Each row's arithmetic does
// not depend on which warp takes it, so the result is that of per-colour
// launches.
template <class T, class K>
__global__ void __launch_bounds__(256, 3) k_sgs_sweep(int ncolor, const int* __restrict__ cptr,
                                                      const int4* __restrict__ desc, const int* __restrict__ ja,
                                                      const T* __restrict__ M,
                                                      const K* __restrict__ dinv, const K* __restrict__ b,
                                                      K* x, typename OffAcc<T>::type* xa,
                                                      int nsweeps, unsigned int* __restrict__ bar,
                                                      int* __restrict__ err) {
  const int g = blockIdx.x * 8 + (threadIdx.x >> 5), W = gridDim.x * 8;
  const int nphase = nsweeps * 2 * ncolor;
  for (int p = 0; p < nphase; p = sgs_next_phase(p, nphase, ncolor)) {
    const int c = sgs_colour(p, ncolor);
    const int r0 = cptr[c], nr = cptr[c + 1] - r0;
    sgs_rows<T, K, true>(nr, desc + r0, ja, M, dinv, b, x, xa, g, W);
    if (sgs_next_phase(p, nphase, ncolor) < nphase && !grid_barrier(bar, gridDim.x, err)) return;
  }
}

// Block sparse matrix-vector product y = A x (CRS MatVecMultiply,
// ucs/crs.tcc:484), warps striding over the rows with the same overlap of
// the next row's indices, diagonal in the vector type.
template <class T, class K>
__global__ void __launch_bounds__(256, 3) k_spmv(int nnode, const int* __restrict__ ia, const int* __restrict__ ja,
                                                 const T* __restrict__ M, const K* __restrict__ diag,
                                                 const K* __restrict__ x,
                                                 const typename OffAcc<T>::type* __restrict__ xa, K* __restrict__ y) {
  typedef typename OffAcc<T>::type A;
  const int lane = threadIdx.x & 31;
  const int W = gridDim.x * 8;
  int i = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (i >= nnode) return;
  // row pointers are read two rows ahead, column indices one row ahead
  int b0, nb, jl;
  row_meta(ia, ja, i, lane, b0, nb, jl);
  int i1 = i + W, b01 = 0, nb1 = 0;
  if (i1 < nnode) {
    b01 = ia[i1] + 1;
    nb1 = ia[i1 + 1] - b01;
  }
  while (true) {
    A av[RowBatch<T>::n], xv[RowBatch<T>::n];
    row_issue<T>(b0, nb, jl, lane, M, xa, av, xv);
    K d = lane < 25 ? diag[(size_t)i * 25 + lane] * x[(size_t)i * 5 + lane % 5] : K(0);
    const int i2 = i1 + W;
    int b02 = 0, nb2 = 0;
    if (i2 < nnode) {
      b02 = ia[i2] + 1;
      nb2 = ia[i2 + 1] - b02;
    }
    const int jl1 = (i1 < nnode && lane < nb1) ? ja[b01 + lane] : 0;
    const K s = (K)row_finish<T>(b0, nb, jl, lane, ja, M, xa, av, xv);
    d = sum5(d);
    if (lane < 25 && lane % 5 == 0) y[(size_t)i * 5 + lane / 5] = s + d;
    if (i1 >= nnode) break;
    i = i1;
    b0 = b01;
    nb = nb1;
    jl = jl1;
    i1 = i2;
    b01 = b02;
    nb1 = nb2;
  }
}

// ---- asynchronous-copy row pipeline (FP32 blocks and vectors) ------------
// A warp streams its rows through a ring of kRowStages shared-memory stages
// filled by 16-byte cp.async.cg copies (L2 only): the row's contiguous
// off-diagonal blocks (one aligned window) and, per block, the aligned
// 32-byte window holding the 5 entries of x it multiplies.  The data of the
// next rows are in flight while the current row is summed, without holding
// registers, so a warp keeps several rows' loads outstanding.  Every copy
// stays inside its array: the allocations carry 16 bytes of tail padding.
constexpr int kRowStages = 3;
constexpr int kStageBlocks = 16;  // blocks staged per row; further blocks are read directly

// Window sizes of one stage in elements of E (float or double): a 16-byte
// chunk holds C elements, so an aligned window of a k-element run starting
// anywhere in a chunk holds k + C - 1 elements, rounded up to whole chunks.
template <class E>
struct StageGeom {
  static constexpr int C = 16 / (int)sizeof(E);
  static constexpr int XCH = (5 + C - 1 + C - 1) / C;    // chunks of one block's x window
  static constexpr int DCH = (25 + C - 1 + C - 1) / C;   // chunks of the inverse diagonal block
  static constexpr int BCH = (5 + C - 1 + C - 1) / C;    // chunks of the right-hand side
};

template <class E>
struct RowStage {
  E m[kStageBlocks * 25 + StageGeom<E>::C];       // window of the row's blocks
  E x[kStageBlocks * StageGeom<E>::XCH * StageGeom<E>::C];  // per block: a window holding its 5 x entries
  E dinv[StageGeom<E>::DCH * StageGeom<E>::C];    // window of the row's inverse diagonal block (sweeps)
  E b[StageGeom<E>::BCH * StageGeom<E>::C];       // window of the row's right-hand side (sweeps)
};
static_assert(sizeof(RowStage<float>) % 16 == 0 && sizeof(RowStage<double>) % 16 == 0, "stage size");

__device__ __forceinline__ void cp_async16(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// element offset of p inside its 16-byte chunk
template <class E>
__device__ __forceinline__ int chunk_off(const E* p) {
  return (int)((reinterpret_cast<uintptr_t>(p) & 15) / sizeof(E));
}
__device__ __forceinline__ const void* chunk_of(const void* p, int k) {
  return reinterpret_cast<const void*>((reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)15) + 16 * (uintptr_t)k);
}

// start the copies of row (b0, nb, jl) into stage st, and with dinv the
// windows of row i's inverse diagonal block and right-hand side; always
// commits a group.  PARTS selects the copies: 1 the matrix, inverse
// diagonal and right-hand side (constant during a sweep), 2 the x windows.
template <class E, int PARTS = 3>
__device__ __forceinline__ void row_stage_issue(bool valid, int b0, int nb, int jl, int lane,
                                                const E* __restrict__ M, const E* xa, RowStage<E>* st, int i = 0,
                                                const E* __restrict__ dinv = nullptr, const E* __restrict__ b = nullptr) {
  typedef StageGeom<E> G;
  const int ns = min(nb, kStageBlocks);
  // column ids of the blocks whose x chunks this lane copies (two passes)
  int j0 = 0, j1 = 0;
  if (PARTS & 2) {
    j0 = __shfl_sync(0xffffffffu, jl, min(lane / G::XCH, 31));
    j1 = __shfl_sync(0xffffffffu, jl, min((lane + 32) / G::XCH, 31));
  }
  if (valid) {
    if (PARTS & 1) {
      const E* g = M + (size_t)b0 * 25;
      const int n16 = (int)(((reinterpret_cast<uintptr_t>(g) & 15) + (uintptr_t)ns * 25 * sizeof(E) + 15) >> 4);
      const uint32_t sm = umma::smem_addr(st->m);
      for (int c = lane; c < n16; c += 32) cp_async16(sm + 16 * c, chunk_of(g, c));
    }
    if (PARTS & 2) {
      const uint32_t sx = umma::smem_addr(st->x);
#pragma unroll
      for (int pass = 0; pass < 2; pass++) {
        const int c = lane + 32 * pass;
        const int u = c / G::XCH;
        if (u < ns) cp_async16(sx + 16 * c, chunk_of(xa + (size_t)(pass ? j1 : j0) * 5, c % G::XCH));
      }
    }
    if ((PARTS & 1) && dinv) {
      if (lane < G::DCH) cp_async16(umma::smem_addr(st->dinv) + 16 * lane, chunk_of(dinv + (size_t)i * 25, lane));
      else if (lane < G::DCH + G::BCH)
        cp_async16(umma::smem_addr(st->b) + 16 * (lane - G::DCH), chunk_of(b + (size_t)i * 5, lane - G::DCH));
    }
  }
  cp_async_commit();
}

// off-diagonal sum of a staged row; lane 5r receives row r's sum
template <class E>
__device__ __forceinline__ E row_stage_sum(int b0, int nb, int jl, int lane, const RowStage<E>* st,
                                           const int* __restrict__ ja, const E* __restrict__ M, const E* xa) {
  typedef StageGeom<E> G;
  const int c = lane % 5;
  const bool active = lane < 25;
  const int ns = min(nb, kStageBlocks);
  const int mo = chunk_off(M + (size_t)b0 * 25);
  // lane u's block: where its x entries start in the stage (formed once per
  // row, one shuffle per block below)
  const int xoff = lane * G::XCH * G::C + chunk_off(xa + (size_t)jl * 5);
  E acc = E(0);
#pragma unroll
  for (int u = 0; u < kStageBlocks; u++) {
    if (u >= ns) break;
    const int xo = __shfl_sync(0xffffffffu, xoff, u);
    if (active) acc = fma(st->m[mo + u * 25 + lane], st->x[xo + c], acc);
  }
  for (int k = kStageBlocks; k < nb; k++) {
    const int j = k < 32 ? __shfl_sync(0xffffffffu, jl, k & 31) : ja[b0 + k];
    if (active) acc = fma(M[(size_t)(b0 + k) * 25 + lane], __ldcg(&xa[(size_t)j * 5 + c]), acc);
  }
  return sum5(acc);
}

// y = A x with FP32 blocks and vectors through the staged pipeline: warps
// stride over rows, each row's copies issued two rows before its sum, its
// row pointers and column indices one row before that.
__global__ void __launch_bounds__(256, 4) k_spmv_staged(int nnode, const int* __restrict__ ia,
                                                        const int* __restrict__ ja, const float* __restrict__ M,
                                                        const float* __restrict__ diag, const float* __restrict__ x,
                                                        float* __restrict__ y) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  RowStage<float>* st = reinterpret_cast<RowStage<float>*>(smem_raw) + wid * kRowStages;
  const int W = gridDim.x * 8;
  int iA = blockIdx.x * 8 + wid;
  if (iA >= nnode) return;
  // rows A (summed this iteration), B (in flight), C (issued this
  // iteration), N (next; its bounds and column indices are read ahead)
  auto bounds = [&](int i, int& b0, int& nb) {
    if (i < nnode) {
      b0 = ia[i] + 1;
      nb = ia[i + 1] - b0;
    } else {
      b0 = 0;
      nb = 0;
    }
  };
  auto cols = [&](int i, int b0, int nb) { return (i < nnode && lane < nb) ? ja[b0 + lane] : 0; };
  int bA, nA, bB, nB, bC, nC, bN, nN;
  bounds(iA, bA, nA);
  int jA = cols(iA, bA, nA);
  int iB = iA + W;
  bounds(iB, bB, nB);
  int jB = cols(iB, bB, nB);
  row_stage_issue(true, bA, nA, jA, lane, M, x, &st[0]);
  row_stage_issue(iB < nnode, bB, nB, jB, lane, M, x, &st[1]);
  int iC = iB + W;
  bounds(iC, bC, nC);
  int jC = cols(iC, bC, nC);
  int iN = iC + W;
  bounds(iN, bN, nN);
  int sA = 0, sB = 1, sC = 2;
  while (true) {
    row_stage_issue(iC < nnode, bC, nC, jC, lane, M, x, &st[sC]);
    const int jN = cols(iN, bN, nN);
    const int iNN = iN + W;
    int bNN, nNN;
    bounds(iNN, bNN, nNN);
    const float d = lane < 25 ? diag[(size_t)iA * 25 + lane] * x[(size_t)iA * 5 + lane % 5] : 0.f;
    cp_async_wait<2>();
    __syncwarp();
    const float sum = row_stage_sum(bA, nA, jA, lane, &st[sA], ja, M, x);
    const float dd = sum5(d);
    if (lane < 25 && lane % 5 == 0) y[(size_t)iA * 5 + lane / 5] = sum + dd;
    __syncwarp();
    if (iB >= nnode) break;
    iA = iB; bA = bB; nA = nB; jA = jB;
    iB = iC; bB = bC; nB = nC; jB = jC;
    iC = iN; bC = bN; nC = nN; jC = jN;
    iN = iNN; bN = bNN; nN = nNN;
    const int t = sA;
    sA = sB;
    sB = sC;
    sC = t;
  }
  cp_async_wait<0>();
}

// The first two rows of a warp in one colour of a sweep: their descriptors
// and column indices, and the copies that do not depend on x (matrix,
// inverse diagonal, right-hand side; two groups when the warp has rows).
// Issued before the barrier that ends the previous colour.
template <class E>
__device__ __forceinline__ void sgs_head(int nrows, const int4* __restrict__ desc, const int* __restrict__ ja,
                                         const E* __restrict__ M, const E* __restrict__ dinv,
                                         const E* __restrict__ b, int g, const int W, RowStage<E>* st, int4& dA,
                                         int& jA, int4& dB, int& jB) {
  const int lane = threadIdx.x & 31;
  const int4 none = make_int4(-1, 0, 0, 0);
  dA = g < nrows ? desc[g] : none;
  dB = g + W < nrows ? desc[g + W] : none;
  jA = (dA.x >= 0 && lane < dA.z) ? ja[dA.y + lane] : 0;
  jB = (dB.x >= 0 && lane < dB.z) ? ja[dB.y + lane] : 0;
  if (g >= nrows) return;
  row_stage_issue<E, 1>(true, dA.y, dA.z, jA, lane, M, nullptr, &st[0], dA.x, dinv, b);
  row_stage_issue<E, 1>(dB.x >= 0, dB.y, dB.z, jB, lane, M, nullptr, &st[1], dB.x, dinv, b);
}

// The rows of one colour of a sweep through the staged pipeline (sgs_rows'
// arithmetic on staged data), E the element type of blocks and vectors:
// desc gives the rows in colour order, g the warp's first row, W the number
// of warps, and (dA, jA, dB, jB) the head sgs_head read and started.
// Drains its copies before returning.
template <class E>
__device__ __forceinline__ void sgs_rows_staged(int nrows, const int4* __restrict__ desc, const int* __restrict__ ja,
                                                const E* __restrict__ M, const E* __restrict__ dinv,
                                                const E* __restrict__ b, E* x, int g, const int W, RowStage<E>* st,
                                                int4 dA, int jA, int4 dB, int jB) {
  const int lane = threadIdx.x & 31;
  if (g >= nrows) return;
  const int r = lane / 5, c = lane % 5;
  const int4 none = make_int4(-1, 0, 0, 0);
  auto cols = [&](const int4& d) { return (d.x >= 0 && lane < d.z) ? ja[d.y + lane] : 0; };
  // groups: head A, head B, x of A, x of B, then one per further row, so
  // the wait for all but the two newest completes row A's copies
  row_stage_issue<E, 2>(true, dA.y, dA.z, jA, lane, M, x, &st[0]);
  row_stage_issue<E, 2>(dB.x >= 0, dB.y, dB.z, jB, lane, M, x, &st[1]);
  int gC = g + 2 * W;
  int4 dC = gC < nrows ? desc[gC] : none;
  int jC = cols(dC);
  int4 dN = gC + W < nrows ? desc[gC + W] : none;
  int sA = 0, sB = 1, sC = 2;
  while (true) {
    row_stage_issue<E>(dC.x >= 0, dC.y, dC.z, jC, lane, M, x, &st[sC], dC.x, dinv, b);
    const int jN = cols(dN);
    const int gNN = gC + 2 * W;
    const int4 dNN = gNN < nrows ? desc[gNN] : none;
    cp_async_wait<2>();
    __syncwarp();
    const RowStage<E>* sa = &st[sA];
    const E s = row_stage_sum<E>(dA.y, dA.z, jA, lane, sa, ja, M, x);
    const int i = dA.x;
    const int bo = chunk_off(b + (size_t)i * 5);
    const int dof = chunk_off(dinv + (size_t)i * 25);
    // rhs_r = b_r - s_r on lane 5r; lane l = 5r + c then forms D^-1[r][c] rhs_c
    const E rhs = (lane < 25 && c == 0) ? sa->b[bo + r] - s : E(0);
    const E rc = __shfl_sync(0xffffffffu, rhs, (5 * c) & 31);
    E v = lane < 25 ? sa->dinv[dof + lane] * rc : E(0);
    v = sum5(v);
    if (lane < 25 && c == 0) x[(size_t)i * 5 + r] = v;
    __syncwarp();
    if (dB.x < 0) break;
    dA = dB; jA = jB;
    dB = dC; jB = jC;
    dC = dN; jC = jN;
    dN = dNN;
    gC += W;
    const int t = sA;
    sA = sB;
    sB = sC;
    sC = t;
  }
  cp_async_wait<0>();
  __syncwarp();
}

// nsweeps sweeps in one cooperative launch through the staged pipeline
// (k_sgs_sweep's phases and barriers); FP32 or FP64 blocks and vectors.
// Each warp starts the x-independent copies of its first two rows of the
// next colour before the barrier, so they overlap the wait.
template <class E>
__global__ void __launch_bounds__(256, sizeof(E) == 8 ? 2 : 4) k_sgs_sweep_staged(int ncolor, const int* __restrict__ cptr,
                                                          const int4* __restrict__ desc, const int* __restrict__ ja,
                                                          const E* __restrict__ M, const E* __restrict__ dinv,
                                                          const E* __restrict__ b, E* x, int nsweeps,
                                                          unsigned int* __restrict__ bar, int* __restrict__ err) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  RowStage<E>* st = reinterpret_cast<RowStage<E>*>(smem_raw) + (threadIdx.x >> 5) * kRowStages;
  const int g = blockIdx.x * 8 + (threadIdx.x >> 5), W = gridDim.x * 8;
  const int nphase = nsweeps * 2 * ncolor;
  if (nphase <= 0) return;
  int c = sgs_colour(0, ncolor);
  int r0 = cptr[c], nr = cptr[c + 1] - r0;
  int4 dA, dB;
  int jA, jB;
  sgs_head<E>(nr, desc + r0, ja, M, dinv, b, g, W, st, dA, jA, dB, jB);
  for (int p = 0; p < nphase;) {
    sgs_rows_staged<E>(nr, desc + r0, ja, M, dinv, b, x, g, W, st, dA, jA, dB, jB);
    p = sgs_next_phase(p, nphase, ncolor);
    if (p < nphase) {
      c = sgs_colour(p, ncolor);
      r0 = cptr[c];
      nr = cptr[c + 1] - r0;
      sgs_head<E>(nr, desc + r0, ja, M, dinv, b, g, W, st, dA, jA, dB, jB);
      if (!grid_barrier(bar, gridDim.x, err)) {
        cp_async_wait<0>();
        return;
      }
    }
  }
}

// FP32 copies of the diagonal blocks and their inverses (FP32 Krylov solver)
__global__ void k_diag_f32(long long n25, const double* __restrict__ diag, const double* __restrict__ dinv,
                           float* __restrict__ diagf, float* __restrict__ dinvf) {
  for (long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x; k < n25; k += (long long)gridDim.x * blockDim.x) {
    diagf[k] = (float)diag[k];
    dinvf[k] = (float)dinv[k];
  }
}

// Newton update (NewtonIterate, ucs/solutionSpace.tcc:772-818): NaN/Inf
// updates are zeroed per node, CompressibleEqnSet::ApplyDQ
// (ucs/compressible.tcc:929) clips density, energy and pressure, the
// auxiliary variables are recomputed, and b-style partial sums of dq^2 are
// formed for the update norm.
// fq, when given, is the double-float copy of q, updated with each row.
__global__ void __launch_bounds__(kNormThreads) k_apply_dq(int nnode, double gamma, double* __restrict__ x,
                                                            double* __restrict__ q, dfl* __restrict__ fq,
                                                            double* __restrict__ part, unsigned long long* health) {
  __shared__ double red[kNormThreads / 32];
  double acc = 0.0;
  const double gm1 = gamma - 1.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnode; i += gridDim.x * blockDim.x) {
    double dQ[5];
    bool zero = false;
    for (int k = 0; k < 5; k++) {
      dQ[k] = x[(size_t)i * 5 + k];
      if (isnan(dQ[k]) || isinf(dQ[k])) zero = true;
    }
    if (zero) {
      for (int k = 0; k < 5; k++) { dQ[k] = 0.0; x[(size_t)i * 5 + k] = 0.0; }
      atomicAdd(&health[H_NANDQ], 1ull);
    }
    double* Q = &q[(size_t)i * NVARS];
    const double minP = 1.0e-10, minRho = 1.0e-10, minE = 1.0e-10;
    if (Q[0] + dQ[0] < 0.0) { Q[0] = minRho; atomicAdd(&health[H_RHOCLIP], 1ull); }
    else Q[0] += dQ[0];
    if (Q[4] + dQ[4] < 0.0) { Q[4] = minE; atomicAdd(&health[H_ECLIP], 1ull); }
    else Q[4] += dQ[4];
    double rho = Q[0];
    double u = Q[1] / rho, v = Q[2] / rho, w = Q[3] / rho;
    double E = Q[4];
    double v2 = u * u + v * v + w * w;
    if (E < 0.5 * rho * v2) {
      atomicAdd(&health[H_PCLIP], 1ull);
      double v2mod = 2.0 * (E - minP / gm1);
      double frac = 0.0;
      if (v2mod > 0.0) frac = sqrt(v2mod / v2);
      u *= frac; v *= frac; w *= frac;
      Q[1] = rho * u; Q[2] = rho * v; Q[3] = rho * w;
    } else {
      Q[1] += dQ[1]; Q[2] += dQ[2]; Q[3] += dQ[3];
    }
    aux_vars(gamma, Q);
    if (fq)
      for (int j = 0; j < NVARS; j++) fq[(size_t)i * NVARS + j] = to_df(Q[j]);
    for (int k = 0; k < 5; k++) acc += dQ[k] * dQ[k];
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double v = 0.0;
    for (int k = 0; k < kNormThreads / 32; k++) v += red[k];
    part[blockIdx.x] = v;
  }
}

// Sum of squares of a vector in fixed order (deterministic), per block.
__global__ void __launch_bounds__(kNormThreads) k_sumsq(long long n, const double* __restrict__ v,
                                                         double* __restrict__ part) {
  __shared__ double red[kNormThreads / 32];
  double acc = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    acc += v[i] * v[i];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int k = 0; k < kNormThreads / 32; k++) s += red[k];
    part[blockIdx.x] = s;
  }
}

__global__ void k_sum_final(int nblocks, const double* __restrict__ part, double* __restrict__ out) {
  if (threadIdx.x >= 32) return;
  const double s = warp_col_sum(part, nblocks, 1, 0, threadIdx.x);
  if (threadIdx.x == 0) *out = s;
}

// MaxEigenvalue (ucs/compressible.tcc:799) of the face-averaged state, in
// the residual's scalar type S (FP64, or double-float)
template <class S, class V>
__device__ __forceinline__ S max_eig(const S* QL, const S* QR, const V& a, S gamma) {
  const S Q0 = halve(QL[0] + QR[0]), Q1 = halve(QL[1] + QR[1]), Q2 = halve(QL[2] + QR[2]),
          Q3 = halve(QL[3] + QR[3]), Q4 = halve(QL[4] + QR[4]);
  const S gm1 = gamma - Sc<S>::c(1.0);
  const S ir = Sc<S>::c(1.0) / Q0;
  const S u = Q1 * ir, v = Q2 * ir, w = Q3 * ir;
  const S v2h = halve(u * u + v * v + w * w);
  const S P = gm1 * (Q4 - Q0 * v2h);
  const S c = sqrt(gamma * P * ir);
  const S theta = u * a.x + v * a.y + w * a.z;
  const S e4 = fabs(theta + c), e5 = fabs(theta - c);
  return e4 > e5 ? e4 : e5;
}

// ComputeTimesteps (ucs/timestep.tcc:7) with local time stepping:
// dt_i = CFL vol_i / sum(max eigenvalue * area) over the node's faces.
template <class S>
__global__ void __launch_bounds__(128) k_timestep(int nnode, const int* __restrict__ nptr, const int* __restrict__ nedg,
                                                  const int* __restrict__ nnbr,
                                                  const typename V4<S>::type* __restrict__ ea,
                                                  const int* __restrict__ bptr, const int* __restrict__ bhe,
                                                  const int2* __restrict__ bn,
                                                  const typename V4<S>::type* __restrict__ ba, const S* __restrict__ q,
                                                  const double* __restrict__ vol, double gamma_d, double cfl,
                                                  double* __restrict__ dt) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nnode) return;
  const S gamma = Sc<S>::from(gamma_d);
  S s = Sc<S>::c(0.0);
  const S* qi = &q[(size_t)i * NVARS];
  for (int k = nptr[i]; k < nptr[i + 1]; k++) {
    int se = nedg[k];
    int e = se < 0 ? ~se : se;
    const S* qj = &q[(size_t)nnbr[k] * NVARS];
    const typename V4<S>::type a = ea[e];
    // the reference averages left and right in edge orientation
    s += (se < 0 ? max_eig(qi, qj, a, gamma) : max_eig(qj, qi, a, gamma)) * a.w;
  }
  for (int p = bptr[i]; p < bptr[i + 1]; p++) {
    int he = bhe[p];
    const typename V4<S>::type a = ba[he];
    s += max_eig(qi, &q[(size_t)bn[he].y * NVARS], a, gamma) * a.w;
  }
  dt[i] = cfl * (vol[i] / Sc<S>::to(s));
}

__global__ void __launch_bounds__(kNormThreads) k_min_part(int n, const double* __restrict__ v,
                                                            double* __restrict__ part) {
  __shared__ double red[kNormThreads / 32];
  double m = 1.0e300;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) m = fmin(m, v[i]);
  for (int o = 16; o > 0; o >>= 1) m = fmin(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 1.0e300;
    for (int k = 0; k < kNormThreads / 32; k++) r = fmin(r, red[k]);
    part[blockIdx.x] = r;
  }
}

__global__ void k_min_final(int nblocks, const double* __restrict__ part, double* __restrict__ out) {
  if (threadIdx.x >= 32) return;
  double r = 1.0e300;
  for (int i = threadIdx.x; i < nblocks; i += 32) r = fmin(r, part[i]);
  for (int o = 16; o > 0; o >>= 1) r = fmin(r, __shfl_xor_sync(0xffffffffu, r, o));
  if (threadIdx.x == 0) *out = r;
}

// ---- FGMRES vector kernels (deterministic reductions) ----------------------

// part[block][k] = partial sums of (w, V_k) for k < nv; V_k = V + k*n
template <class K>
__global__ void __launch_bounds__(kNormThreads) k_mdot(long long n, int nv, const K* __restrict__ V,
                                                        const K* __restrict__ w, double* __restrict__ part,
                                                        unsigned int* __restrict__ done,
                                                        double* __restrict__ out, float* __restrict__ outf) {
  // eight vectors per pass over w: w is read nv/8 times, each V_k once;
  // per-thread sums in the vector type, block sums in FP64, stored dot-major
  // ([k][block]) for the final sums
  __shared__ double red[kNormThreads / 32][8];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k0 = 0; k0 < nv; k0 += 8) {
    const int nk = min(8, nv - k0);
    K acc[8];
#pragma unroll
    for (int u = 0; u < 8; u++) acc[u] = K(0);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
      const K wi = w[i];
#pragma unroll
      for (int u = 0; u < 8; u++)
        if (u < nk) acc[u] = fma(wi, V[(size_t)(k0 + u) * n + i], acc[u]);
    }
#pragma unroll
    for (int u = 0; u < 8; u++) {
      K a = acc[u];
      for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
      if (lane == 0) red[wid][u] = (double)a;
    }
    __syncthreads();
    if (threadIdx.x < nk) {
      double sacc = 0.0;
      for (int q = 0; q < kNormThreads / 32; q++) sacc += red[q][threadIdx.x];
      part[(size_t)(k0 + threadIdx.x) * gridDim.x + blockIdx.x] = sacc;
    }
    __syncthreads();
  }
  // the last block to finish sums the partials (a warp per dot product, in
  // a fixed order) and re-arms the counter
  __threadfence();
  if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (last) {
    __threadfence();
    for (int k = wid; k < nv; k += kNormThreads / 32) {
      const double sum = warp_col_sum(part + (size_t)k * gridDim.x, (int)gridDim.x, 1, 0, lane);
      if (lane == 0) {
        out[k] = sum;
        outf[k] = (float)sum;
      }
    }
    if (threadIdx.x == 0) *done = 0u;
  }
}

// w -= sum_k h[k] V_k   (h on the device, in the vector type)
template <class K>
__global__ void k_orth_update(long long n, int nv, const K* __restrict__ V, const K* __restrict__ h,
                              K* __restrict__ w) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    K v = w[i];
    for (int k = 0; k < nv; k++) v -= h[k] * V[(size_t)k * n + i];
    w[i] = v;
  }
}

// w -= sum_k h[k] V_k (the first Gram-Schmidt pass), then dots[k] =
// (w, V_k) of the result (the second pass's coefficients), nv <= 32, in one
// pass over V: the update as in k_orth_update, the dot products with the
// per-thread, per-block and final summation orders of k_mdot.  Partials are
// stored dot-major ([k][block]).
template <class K, int NV>
__global__ void __launch_bounds__(kNormThreads) k_orth_mdot(long long n, int nv, const K* __restrict__ V,
                                                             const K* __restrict__ h, K* __restrict__ w,
                                                             double* __restrict__ part,
                                                             unsigned int* __restrict__ done,
                                                             double* __restrict__ out, float* __restrict__ outf) {
  __shared__ double red[kNormThreads / 32][32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  K acc[NV], hh[NV];
#pragma unroll
  for (int u = 0; u < NV; u++) {
    acc[u] = K(0);
    hh[u] = u < nv ? h[u] : K(0);
  }
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    // the element's V entries loaded ahead (independent loads in flight),
    // then the update in the sequential order and the dot products
    K vv[NV];
    const K* vp = V + i;
#pragma unroll
    for (int u = 0; u < NV; u++) vv[u] = u < nv ? vp[(size_t)u * n] : K(0);
    K v = w[i];
#pragma unroll
    for (int u = 0; u < NV; u++)
      if (u < nv) v -= hh[u] * vv[u];
    w[i] = v;
#pragma unroll
    for (int u = 0; u < NV; u++)
      if (u < nv) acc[u] = fma(v, vv[u], acc[u]);
  }
#pragma unroll
  for (int u = 0; u < NV; u++) {
    if (u >= nv) break;
    K a = acc[u];
    for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
    if (lane == 0) red[wid][u] = (double)a;
  }
  __syncthreads();
  if (threadIdx.x < nv) {
    double sacc = 0.0;
    for (int q = 0; q < kNormThreads / 32; q++) sacc += red[q][threadIdx.x];
    part[(size_t)threadIdx.x * gridDim.x + blockIdx.x] = sacc;
  }
  __threadfence();
  if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (last) {
    __threadfence();
    for (int k = wid; k < nv; k += kNormThreads / 32) {
      const double sum = warp_col_sum(part + (size_t)k * gridDim.x, (int)gridDim.x, 1, 0, lane);
      if (lane == 0) {
        out[k] = sum;
        outf[k] = (float)sum;
      }
    }
    if (threadIdx.x == 0) *done = 0u;
  }
}

// w -= sum_k h[k] V_k (the second Gram-Schmidt pass) with (w, w) of the
// result: per-thread sums in the vector type and FP64 block sums as in
// k_mdot, the last block writing the total to out[0]
template <class K, int NV>
__global__ void __launch_bounds__(kNormThreads) k_orth_norm(long long n, int nv, const K* __restrict__ V,
                                                             const K* __restrict__ h, K* __restrict__ w,
                                                             double* __restrict__ part,
                                                             unsigned int* __restrict__ done,
                                                             double* __restrict__ out) {
  __shared__ double red[kNormThreads / 32];
  __shared__ bool last;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  K acc = K(0);
  if (nv <= NV) {
    // up to NV vectors: V entries and coefficients in registers, loaded ahead
    K hh[NV];
#pragma unroll
    for (int u = 0; u < NV; u++) hh[u] = u < nv ? h[u] : K(0);
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
      K vv[NV];
      const K* vp = V + i;
#pragma unroll
      for (int u = 0; u < NV; u++) vv[u] = u < nv ? vp[(size_t)u * n] : K(0);
      K v = w[i];
#pragma unroll
      for (int u = 0; u < NV; u++)
        if (u < nv) v -= hh[u] * vv[u];
      w[i] = v;
      acc = fma(v, v, acc);
    }
  } else {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
      K v = w[i];
      for (int k = 0; k < nv; k++) v -= h[k] * V[(size_t)k * n + i];
      w[i] = v;
      acc = fma(v, v, acc);
    }
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if (lane == 0) red[wid] = (double)acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double sacc = 0.0;
    for (int q = 0; q < kNormThreads / 32; q++) sacc += red[q];
    part[blockIdx.x] = sacc;
  }
  __threadfence();
  if (threadIdx.x == 0) last = atomicAdd(done, 1u) == gridDim.x - 1;
  __syncthreads();
  if (last) {
    __threadfence();
    if (wid == 0) {
      const double sum = warp_col_sum(part, (int)gridDim.x, 1, 0, lane);
      if (lane == 0) out[0] = sum;
    }
    if (threadIdx.x == 0) *done = 0u;
  }
}

// y = a * x
template <class K>
__global__ void k_scale_copy(long long n, K a, const K* __restrict__ x, K* __restrict__ y) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    y[i] = a * x[i];
}

// x += sum_k c[k] Z_k  (x FP64; the sum in the vector type)
template <class K>
__global__ void k_combine(long long n, int nv, const K* __restrict__ Z, const K* __restrict__ c,
                          double* __restrict__ x) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    K v = K(0);
    for (int k = 0; k < nv; k++) v += c[k] * Z[(size_t)k * n + i];
    x[i] += (double)v;
  }
}

// FP32 vector from an FP64 one, or b - r into FP32 (r = A x on entry)
__global__ void k_residual_vec_f32(long long n, const double* __restrict__ b, const double* __restrict__ r,
                                   float* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = (float)(b[i] - (r ? r[i] : 0.0));
}

// r = b - r   (r holds A x on entry)
__global__ void k_residual_vec(long long n, const double* __restrict__ b, double* __restrict__ r) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    r[i] = b[i] - r[i];
}
