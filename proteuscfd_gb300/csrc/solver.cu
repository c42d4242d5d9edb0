// Device solver for the edge-based implicit finite-volume path on sm_103a:
// C ABI (include/pcfd.h), device-resident mesh and fields, and the kernels
// for boundary conditions, LSQ gradient, limiter and residual.
//
// Design (GB300-first, one GPU):
//  * Every field lives in HBM for the life of the handle; host copies happen
//    only in set/get calls.
//  * The edge loops of the reference (Driver/Bdriver, ucs/driver.tcc:6,70)
//    become (a) one edge kernel that evaluates each edge's flux once and
//    stores it, and (b) a node kernel that gathers, for every node, its
//    incident edge fluxes in ascending edge order - the order in which the
//    reference's sequential scatter adds them - so the sum is deterministic
//    and free of atomics.
//  * Node-centred passes (gradient, limiter) gather over a node->edge CSR in
//    the same ascending edge order; the static per-edge-end LSQ weights and
//    edge half-vectors are computed once at set-up, because the mesh does
//    not move.
//  * FP64 throughout the residual path.
#include "../../include/pcfd.h"
#include "flux_device.cuh"
#include "umma.cuh"

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

using namespace pcfd;

// 32-byte aligned edge area record (unit normal + magnitude), one 256-bit load
struct __align__(32) D4 {
  double x, y, z, w;
};
struct __align__(32) DF4 {
  dfl x, y, z, w;
};
template <class S>
struct V4;
template <>
struct V4<double> {
  using type = D4;
};
template <>
struct V4<dfl> {
  using type = DF4;
};

namespace {

thread_local std::string g_err;

int set_err(int code, const std::string& msg) {
  g_err = msg;
  return code;
}

#define CUDA_TRY(call)                                                                 \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      return set_err(PCFD_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

enum HealthSlot {
  H_KNEECAP = 0,  // NaN flux components zeroed (ucs/eqnset.tcc:73-88)
  H_LIMCLIP = 1,  // nodes whose limiter the pressure clip zeroed
  H_RHOCLIP = 2,  // ApplyDQ density clips
  H_ECLIP = 3,    // ApplyDQ energy clips
  H_PCLIP = 4,    // ApplyDQ pressure clips
  H_NANDQ = 5,    // nodes whose NaN/Inf update was zeroed
  H_BADBC = 6,    // half-edges with an unknown boundary condition type
  H_BADLU = 7     // ill-conditioned diagonal blocks in the LU
};

// Kernel timers, one per launch site (TimerList analogue)
enum TimerId {
  T_BC = 0, T_GRAD, T_LIMITER, T_EDGEFLUX, T_CLIP, T_BEDGEFLUX, T_GATHER, T_NORM, T_SETUP,
  T_JAC_EDGE, T_JAC_BEDGE, T_JAC_DIAG, T_JAC_FINISH, T_SGS, T_SPMV, T_KRYLOV, T_UPDATE, T_TIMESTEP, T_LP_FWD,
  T_LP_BWD, T_EDGEVISC, T_COUNT
};
const char* kTimerNames[T_COUNT] = {"bc_update", "lsq_gradient", "venkat_limiter", "edge_flux", "pressure_clip",
                                    "bedge_flux", "residual_gather", "norm_reduce", "setup", "jac_edge",
                                    "jac_bedge", "jac_diag", "jac_finish_lu", "sgs_sweep", "spmv",
                                    "krylov_vec", "apply_dq", "timestep", "learned_forward",
                                    "learned_backward", "edge_viscous"};

struct Learned;

struct Solver {
  // sizes
  int nnode = 0, nbnode = 0, nedge = 0, nbedge = 0, ntot = 0;
  int nbgroup = 0;  // boundary nodes
  pcfd_params prm{};
  std::vector<int> bc_type;
  std::vector<double> bc_twall;
  double qinf[NVARS];
  int bc_sequential = 0;  // 1: a no-slip normal node is itself hard-set; run BCs in order

  cudaStream_t stream = nullptr;
  // mesh
  int2* d_en = nullptr;         // [nedge] edge nodes
  D4* d_ea = nullptr;      // [nedge] unit normal + area
  double* d_eh = nullptr;       // [nedge][3] 0.5 (xR - xL)
  int2* d_bn = nullptr;         // [nbedge]
  D4* d_ba = nullptr;      // [nbedge]
  int* d_bbc = nullptr;         // [nbedge] bc type
  double* d_btw = nullptr;      // [nbedge] non-dimensional wall temperature
  int* d_bfactag = nullptr;     // [nbedge] boundary tag
  int* d_bnrm = nullptr;        // [nbedge] no-slip normal node (or -1)
  double* d_xyz = nullptr;      // [nnode][3]
  double* d_vol = nullptr;      // [nnode]
  int* d_nptr = nullptr;        // [nnode+1] node -> incident edges
  int* d_nedg = nullptr;        // [2 nedge] signed edge id (~e when the node is the left node)
  int* d_nnbr = nullptr;        // [2 nedge] neighbour node of that entry
  double* d_lsq = nullptr;      // [2 nedge][3] LSQ weights per edge end
  int* d_bptr = nullptr;        // [nnode+1] node -> boundary half-edges (bedge order)
  int* d_bhe = nullptr;         // [nbedge]
  int* d_bgnode = nullptr;      // [nbgroup] boundary nodes
  int* d_bgptr = nullptr;       // [nbgroup+1] -> d_bghe
  int* d_bghe = nullptr;        // [nbgslot] half-edges of the hard-set nodes, bedge order per node
  int nbgslot = 0;
  int* d_bgslot = nullptr;      // [nbgslot] -> group
  double* d_bgqr = nullptr;     // [nbgslot][NVARS] new phantom states
  // fields
  double* d_q = nullptr;        // [ntot][10]
  double* d_grad = nullptr;     // [nnode][27]
  double* d_lim = nullptr;      // [nnode][5]
  double* d_b = nullptr;        // [nnode][5]
  double* d_qold = nullptr;     // [nnode][5] conservative state at the start of the step (STATE_N)
  double* d_qpre = nullptr;     // [ntot][10] state before the Jacobian's boundary pass
  double* d_ef = nullptr;       // [nedge][5] edge flux scratch
  double* d_bf = nullptr;       // [nbedge][5] half-edge flux scratch
  double* d_part = nullptr;     // [kNormBlocks][6] norm partial sums (scratch)
  double* d_norms = nullptr;    // [6]
  unsigned long long* d_health = nullptr;  // [8]
  double* d_limraw = nullptr;   // [nnode][5] limiter before the clamp to zero
  int* d_clipflag = nullptr;    // [nnode] bit 0 clip, bit 1 negative raw limiter
  int* d_clipany = nullptr;     // [1]
  int* d_bind = nullptr;        // half-edges of nodes without hard-set BCs
  int nbind = 0;
  int have_grad = 0, have_lim = 0;
  int lim_clipped = 0;  // 1: d_lim already went through the explicit pressure clip
  int grad_arith = 0, lim_arith = 0;
  int lim_fresh = 0;    // the limiter was computed since the last residual (its clip is pending)
  // each edge end's MUSCL correction grad.dx ([nedge][2][5], left end
  // first), written by the limiter pass that forms it anyway; valid for the
  // gradient it was formed from until the next residual (chi = 0 only)
  double* d_ext = nullptr;
  dfl* f_ext = nullptr;
  int ext_ready = 0, ext_arith = 0;

  // residual arithmetic of the composite calls: 0 FP64, 1 double-float on the
  // FP32 pipes; the double-float copies of the residual-path arrays
  int arith = 0;
  int f_q_valid = 0;
  dfl *f_q = nullptr, *f_grad = nullptr, *f_lim = nullptr, *f_limraw = nullptr, *f_eh = nullptr, *f_lsq = nullptr,
      *f_ef = nullptr, *f_bf = nullptr;
  DF4 *f_ea = nullptr, *f_ba = nullptr;

  // implicit system (block CRS in the reference layout)
  long long nblocks = 0;
  int* d_ia = nullptr;          // [nnode+1]
  int* d_ja = nullptr;          // [nblocks]
  int* d_pos_lr = nullptr;      // [nedge] block index of A(L,R)
  int* d_pos_rl = nullptr;      // [nedge] block index of A(R,L)
  int jac_prec = -1;            // 0 FP64, 1 FP32, 2 BF16 off-diagonal storage
  void* d_M = nullptr;          // [nblocks][25] off-diagonal blocks (diagonal slots unused)
  double* d_diag = nullptr;     // [nnode][25] diagonal blocks before the LU
  double* d_dlu = nullptr;      // [nnode][25] LU of the diagonal, U reciprocals on its diagonal
  double* d_dinv = nullptr;     // [nnode][25] inverse of the diagonal block (from the LU)
  float* d_diagf = nullptr;     // [nnode][25] FP32 copies of diag and dinv (FP32 Krylov solver)
  float* d_dinvf = nullptr;
  double* d_wd = nullptr;       // [nnode][5] FP64 scratch of the Krylov solver
  double* d_mv = nullptr;       // pcfd_matvec / pcfd_sgs_rhs scratch (two FP64 vectors, two padded FP32)
  float* d_dotsf = nullptr;     // FP32 copies of the Krylov dot results
  unsigned int* d_mdot_done = nullptr;  // blocks finished in k_mdot (re-armed by its last block)
  int* d_piv = nullptr;         // [nnode][5]
  double* d_bblk = nullptr;     // [nbedge][25] boundary contributions to the diagonal
  double* d_dt = nullptr;       // [nnode] local pseudo time step
  double* d_x = nullptr;        // [nnode][5] linear solution (dq)
  float* d_xf = nullptr;        // [nnode][5] FP32 copy of the vector the FP32/BF16 products read
  double* d_scal = nullptr;     // [16] scalar results
  int have_dt = 0, have_jac = 0;
  int ncolor = 0;
  std::vector<int> color_ptr;   // [ncolor+1] into d_color_rows
  int* d_color_rows = nullptr;  // [nnode]
  int* d_cptr = nullptr;        // [ncolor+1] colour pointers on the device
  int4* d_rowdesc = nullptr;    // [nnode] (row, first off-diagonal block, block count) in colour order
  unsigned int* d_gbar = nullptr;  // grid barrier of the SGS sweep kernel (count, generation)
  int* d_sgs_err = nullptr;     // set when a sweep's grid barrier timed out
  int nsm = 0;                  // multiprocessors of the device
  int orth_grid[16] = {};  // one-wave grids of k_orth_norm / k_orth_mdot per type and register width
  // FGMRES work space (allocated on first use)
  int fg_m = 0;
  double* d_V = nullptr;        // [m+1][nnode*5]
  double* d_Z = nullptr;        // [m][nnode*5]
  double* d_w = nullptr;        // [nnode*5]
  double* d_dots = nullptr;     // [kKrylovBlocks][m+2] partial dot products

  // profiling
  int profile = 0;
  // learned preconditioner (pcfd_lp_*), with the mesh means its features use
  Learned* lp = nullptr;
  double lp_lmean = 1.0, lp_vmean = 1.0;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  double t_ms[T_COUNT] = {0};
  long long t_n[T_COUNT] = {0};
  long long launches = 0;
};

constexpr int kNormBlocks = 304;  // 2 x 152 SMs
// Krylov vector kernels (dot products, orthogonalisation, scaling, the
// solution update) stream several vectors per element: 8 blocks of 256
// threads per SM keep enough loads in flight
constexpr int kKrylovBlocks = 8 * 152;
constexpr int kNormThreads = 256;

template <class F>
int launch(Solver* s, int timer, F&& f) {
  if (s->profile) cudaEventRecord(s->ev0, s->stream);
  f();
  s->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return set_err(PCFD_ERR_CUDA, std::string("kernel launch: ") + cudaGetErrorString(e));
  if (s->profile) {
    cudaEventRecord(s->ev1, s->stream);
    cudaEventSynchronize(s->ev1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, s->ev0, s->ev1);
    s->t_ms[timer] += ms;
    s->t_n[timer]++;
  }
  return PCFD_OK;
}

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

// Blocks of the row kernels (8 warps each, warps striding over rows): three
// resident blocks per SM on 152 SMs, fewer when there are fewer rows.
inline int row_grid(long long nrows) { return std::max(1, std::min(nblk(nrows, 8), 3 * 152)); }

// -------------------------------------------------------------------------
// set-up kernels
// -------------------------------------------------------------------------

// ComputeLSQCoefficients (ucs/gradient.tcc:141) for every (node, edge) entry
// of the node->edge CSR, with the inverse-distance weighting of
// Kernel_LSQ_Gradient (:251): grad_i += -we(s_i, w (x_i - x_j)) w (q_j - q_i).
// The stored triple is -we * w.
__global__ void k_lsq_weights(int nnode, const int* __restrict__ nptr, const int* __restrict__ nnbr,
                              const double* __restrict__ xyz, const double* __restrict__ sw,
                              double* __restrict__ lsq) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nnode) return;
  const double* s = &sw[6 * i];
  double s11 = s[0], s12 = s[1], s13 = s[2], s22 = s[3], s23 = s[4], s33 = s[5];
  double r11 = s11, r12 = s12, r13 = s13;
  double r12_r11 = (r11 == 0.0) ? 0.0 : r12 / r11;
  double r22 = s22 - r12 * r12_r11;
  double r23 = s23 - r12_r11 * r13;
  double r13_r11 = (r11 == 0.0) ? 0.0 : r13 / r11;
  double r23_r22 = (r22 == 0.0) ? 0.0 : r23 / r22;
  double r33 = s33 - r13 * r13_r11 - r23 * r23_r22;
  double xi0 = xyz[3 * i], xi1 = xyz[3 * i + 1], xi2 = xyz[3 * i + 2];
  for (int k = nptr[i]; k < nptr[i + 1]; k++) {
    int j = nnbr[k];
    double dx0 = xi0 - xyz[3 * j], dx1 = xi1 - xyz[3 * j + 1], dx2 = xi2 - xyz[3 * j + 2];
    double d2 = dx0 * dx0 + dx1 * dx1 + dx2 * dx2;
    double weight = 1.0 / sqrt(d2);
    dx0 *= weight; dx1 *= weight; dx2 *= weight;
    double dykdx = (dx1 - r12_r11 * dx0);
    double we2 = (r33 == 0.0) ? 0.0 : (dx2 - r13_r11 * dx0 - r23_r22 * dykdx) / r33;
    double we1 = (r22 == 0.0) ? 0.0 : (dykdx - r23 * we2) / r22;
    double we0 = (r11 == 0.0) ? 0.0 : (dx0 - r12 * we1 - r13 * we2) / r11;
    lsq[3 * (size_t)k + 0] = -we0 * weight;
    lsq[3 * (size_t)k + 1] = -we1 * weight;
    lsq[3 * (size_t)k + 2] = -we2 * weight;
  }
}

__global__ void k_edge_half(int nedge, const int2* __restrict__ en, const double* __restrict__ xyz,
                            double* __restrict__ eh) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nedge) return;
  int2 n = en[e];
  for (int c = 0; c < 3; c++) eh[3 * (size_t)e + c] = 0.5 * (xyz[3 * n.y + c] - xyz[3 * n.x + c]);
}

__global__ void k_fill_state(int nrows, const double* __restrict__ qinf, double* __restrict__ q) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nrows) return;
  for (int j = 0; j < NVARS; j++) q[(size_t)i * NVARS + j] = qinf[j];
}

// -------------------------------------------------------------------------
// boundary conditions (UpdateBCs, ucs/bc.tcc:1400)
// -------------------------------------------------------------------------

struct BcConst {
  double gamma;
  int no_cvbc;
  double qinf[NVARS];
};

// Arithmetic at the reference's decision points (a limiter's "does the
// extrapolation raise the value", the far field's "is there flow through
// the face") in the reference's rounding: each product and sum rounded on its
// own, in its order, no fused multiply-add.  A state whose answer sits on
// the tie (a zero velocity component, a flat field) then takes the
// reference's branch; the double-float arithmetic keeps its own forms.
template <class S>
__device__ __forceinline__ S dot3_ref(S a0, S b0, S a1, S b1, S a2, S b2) {
  return a0 * b0 + a1 * b1 + a2 * b2;
}
template <>
__device__ __forceinline__ double dot3_ref<double>(double a0, double b0, double a1, double b1, double a2, double b2) {
  return __dadd_rn(__dadd_rn(__dmul_rn(a0, b0), __dmul_rn(a1, b1)), __dmul_rn(a2, b2));
}
// q + ExtrapolateCorrection(dq, grad, dx) (ucs/eqnset.h:231) with a limiter of one
template <class S>
__device__ __forceinline__ S extrap_ref(S qi, S dq, S gdx, S hchi, S omc, bool chi0) {
  return chi0 ? qi + gdx : qi + (hchi * dq + omc * gdx);
}
template <>
__device__ __forceinline__ double extrap_ref<double>(double qi, double dq, double gdx, double hchi, double omc,
                                                     bool chi0) {
  return chi0 ? __dadd_rn(qi, gdx) : __dadd_rn(qi, __dadd_rn(__dmul_rn(hchi, dq), __dmul_rn(omc, gdx)));
}
// GetTheta (ucs/compressible.tcc:996): u nx + v ny + w nz of the averaged state
template <class S>
__device__ __forceinline__ S theta_ref(S t0, S t1, S t2, S t3, S ax, S ay, S az) {
  const S it0 = Sc<S>::c(1.0) / t0;
  return t1 * it0 * ax + t2 * it0 * ay + t3 * it0 * az;
}
template <>
__device__ __forceinline__ double theta_ref<double>(double t0, double t1, double t2, double t3, double ax, double ay,
                                                    double az) {
  return dot3_ref<double>(__ddiv_rn(t1, t0), ax, __ddiv_rn(t2, t0), ay, __ddiv_rn(t3, t0), az);
}

// GetFarfieldBoundaryVariables (ucs/compressible.tcc:1246), static grid;
// S = double, or dfl for the double-float residual arithmetic.  qinf and
// the stored pressure pi come in as S.
template <class S>
__device__ void bc_farfield(S gamma, const S* Qinf, const S* QL, S pi, S* QR, const S ax, const S ay, const S az) {
  const S half = Sc<S>::c(0.5), one = Sc<S>::c(1.0), zero = Sc<S>::c(0.0);
  const S gm1 = gamma - one;
  for (int subit = 0; subit < 10; subit++) {
    S t0 = (QL[0] + QR[0]) * half, t1 = (QL[1] + QR[1]) * half, t2 = (QL[2] + QR[2]) * half,
      t3 = (QL[3] + QR[3]) * half, t4 = (QL[4] + QR[4]) * half;
    S it0 = one / t0;
    S theta = theta_ref<S>(t0, t1, t2, t3, ax, ay, az);
    S rhoi = QL[0];
    S iri = one / QL[0];
    S ui = QL[1] * iri, vi = QL[2] * iri, wi = QL[3] * iri;
    S rhoinf = Qinf[0];
    S uinf = Qinf[1] / Qinf[0], vinf = Qinf[2] / Qinf[0], winf = Qinf[3] / Qinf[0];
    S pinf = Qinf[6];
    S tu = t1 * it0, tv = t2 * it0, tw = t3 * it0;
    S pavg = gm1 * (t4 - t0 * (half * (tu * tu + tv * tv + tw * tw)));
    S rhoavg = t0;
    S c2avg = gamma * (pavg / rhoavg);
    S cavg = sqrt(c2avg);
    S mach = fabs(theta / cavg);
    if (theta == zero) {
      return;
    } else if (theta > zero && mach >= one) {
      for (int i = 0; i < NEQN; i++) QR[i] = QL[i];
    } else if (theta < zero && mach >= one) {
      for (int i = 0; i < NEQN; i++) QR[i] = Qinf[i];
    } else if (theta > zero && mach < one) {
      S pb = pinf;
      S rhob = rhoi + (pb - pi) / c2avg;
      S t = (pb - pi) / (rhoavg * cavg);
      S ub = ui - ax * t, vb = vi - ay * t, wb = wi - az * t;
      QR[0] = rhob; QR[1] = rhob * ub; QR[2] = rhob * vb; QR[3] = rhob * wb;
      QR[4] = pb / gm1 + half * rhob * (ub * ub + vb * vb + wb * wb);
    } else if (theta < zero && mach < one) {
      S pb = half * (pinf + pi + rhoavg * cavg * (ax * (uinf - ui) + ay * (vinf - vi) + az * (winf - wi)));
      S rhob = rhoinf + (pb - pinf) / c2avg;
      S t = (pb - pinf) / (rhoavg * cavg);
      S ub = uinf + ax * t, vb = vinf + ay * t, wb = winf + az * t;
      QR[0] = rhob; QR[1] = rhob * ub; QR[2] = rhob * vb; QR[3] = rhob * wb;
      QR[4] = pb / gm1 + half * rhob * (ub * ub + vb * vb + wb * wb);
    } else {
      return;
    }
  }
}

// GetInviscidWallBoundaryVariables (ucs/compressible.tcc:1375), static grid
template <class S>
__device__ void bc_inviscid_wall(S gamma, int no_cvbc, const S* QL, S pi, S* QR, const S ax, const S ay,
                                 const S az) {
  const S half = Sc<S>::c(0.5), one = Sc<S>::c(1.0), two = Sc<S>::c(2.0);
  const S gm1 = gamma - one;
  const S rhoi = QL[0];
  const S iri = one / rhoi;
  const S ui = QL[1] * iri, vi = QL[2] * iri, wi = QL[3] * iri;
  if (no_cvbc) {
    S dot = QL[1] * ax + QL[2] * ay + QL[3] * az;
    for (int i = 0; i < NEQN; i++) QR[i] = QL[i];
    QR[1] = QL[1] - two * dot * ax;
    QR[2] = QL[2] - two * dot * ay;
    QR[3] = QL[3] - two * dot * az;
    return;
  }
  const S thetaL = ui * ax + vi * ay + wi * az;
  for (int subit = 0; subit < 10; subit++) {
    S t0 = (QL[0] + QR[0]) * half, t1 = (QL[1] + QR[1]) * half, t2 = (QL[2] + QR[2]) * half,
      t3 = (QL[3] + QR[3]) * half, t4 = (QL[4] + QR[4]) * half;
    S it0 = one / t0;
    S tu = t1 * it0, tv = t2 * it0, tw = t3 * it0;
    S rhoavg = t0;
    S pavg = gm1 * (t4 - t0 * (half * (tu * tu + tv * tv + tw * tw)));
    S c2avg = gamma * (pavg / rhoavg);
    S cavg = sqrt(c2avg);
    S pb = pi + rhoavg * cavg * thetaL;
    S rhob = rhoi + (pb - pi) / c2avg;
    S t = (pb - pi) / (rhoavg * cavg);
    S ub = ui - ax * t, vb = vi - ay * t, wb = wi - az * t;
    QR[0] = rhob; QR[1] = rhob * ub; QR[2] = rhob * vb; QR[3] = rhob * wb;
    QR[4] = pb / gm1 + half * rhob * (ub * ub + vb * vb + wb * wb);
  }
}

// FP64 entry points used by the ordered kernels and the boundary Jacobian
__device__ void bc_farfield(const BcConst& k, const double* QL, double* QR, const D4 a) {
  bc_farfield<double>(k.gamma, k.qinf, QL, QL[6], QR, a.x, a.y, a.z);
}
__device__ void bc_inviscid_wall(const BcConst& k, const double* QL, double* QR, const D4 a) {
  bc_inviscid_wall<double>(k.gamma, k.no_cvbc, QL, QL[6], QR, a.x, a.y, a.z);
}

// One boundary half-edge of CalculateBoundaryVariables (ucs/bc.tcc:1059).
// Returns 0 on an unknown BC type.
__device__ int apply_bc(const BcConst& k, int bct, double* QL, double* QR, const D4 a, double Tw,
                        const double* nQ) {
  switch (bct) {
    case PCFD_BC_SONIC_INFLOW:
    case PCFD_BC_DIRICHLET:
      for (int i = 0; i < NVARS; i++) QR[i] = QL[i] = k.qinf[i];
      break;
    case PCFD_BC_SONIC_OUTFLOW:
    case PCFD_BC_NEUMANN:
      for (int i = 0; i < NEQN; i++) QR[i] = QL[i];
      break;
    case PCFD_BC_FARFIELD:
      bc_farfield(k, QL, QR, a);
      break;
    case PCFD_BC_IMPERMEABLE_WALL:
    case PCFD_BC_SYMMETRY:
      bc_inviscid_wall(k, QL, QR, a);
      break;
    case PCFD_BC_NOSLIP:
      // GetViscousWallBoundaryVariables (ucs/compressible.tcc:1545), static wall
      if (Tw < 0.0) {
        QR[0] = QL[0] = nQ[0];
        QR[4] = QL[4] = nQ[4];
      } else {
        double gm1 = k.gamma - 1.0;
        double rhoEt = (Tw * QL[0] / (k.gamma * gm1) + 0.5 * QR[0] * 0.0);
        QR[0] = QL[0];
        QR[4] = QL[4] = rhoEt;
      }
      QR[1] = QL[1] = QL[0] * 0.0;
      QR[2] = QL[2] = QL[0] * 0.0;
      QR[3] = QL[3] = QL[0] * 0.0;
      break;
    default:
      return 0;
  }
  aux_vars(k.gamma, QR);
  aux_vars(k.gamma, QL);
  return 1;
}

// Nodes that a condition hard-sets (no-slip, Dirichlet, sonic inflow) see
// their half-edges in bedge order: a half-edge's phantom state depends on
// the node state left by the hard-set half-edges before it.  The work is
// split so that every half-edge still gets its own thread:
//   k_bc_group_halfedges  one thread per half-edge of a hard-set node; it
//                         replays the node-state changes of the earlier
//                         hard-set half-edges of its node (cheap assignments)
//                         and then runs its own condition, writing the new
//                         phantom state to a scratch row;
//   k_bc_group_nodes      one thread per hard-set node; it replays all its
//                         half-edges' node-state changes, writes the node,
//                         then moves its phantoms from scratch into q.
// Reads of q in the first kernel therefore all see the state before the
// update, as in the reference's sequential loop (ucs/bc.tcc:1400).

// Writes one state row; fq, when given, is the double-float copy of q the
// residual reads, kept current row by row instead of converted again whole.
__device__ __forceinline__ void store_row(double* __restrict__ q, dfl* __restrict__ fq, int row, const double* Q) {
  for (int j = 0; j < NVARS; j++) q[(size_t)row * NVARS + j] = Q[j];
  if (fq)
    for (int j = 0; j < NVARS; j++) fq[(size_t)row * NVARS + j] = to_df(Q[j]);
}

__device__ __forceinline__ bool hardsets(int bct) {
  return bct == PCFD_BC_NOSLIP || bct == PCFD_BC_SONIC_INFLOW || bct == PCFD_BC_DIRICHLET;
}

// The node-state half of apply_bc for the hard-setting conditions; qr0 is
// the phantom density before the update (it enters the isothermal wall's
// energy multiplied by the zero wall velocity).
__device__ void hardset_node(const BcConst& k, int bct, double* QL, double Tw, const double* nQ, double qr0) {
  if (bct == PCFD_BC_NOSLIP) {
    if (Tw < 0.0) {
      QL[0] = nQ[0];
      QL[4] = nQ[4];
    } else {
      double gm1 = k.gamma - 1.0;
      QL[4] = (Tw * QL[0] / (k.gamma * gm1) + 0.5 * qr0 * 0.0);
    }
    QL[1] = QL[0] * 0.0;
    QL[2] = QL[0] * 0.0;
    QL[3] = QL[0] * 0.0;
  } else {
    for (int i = 0; i < NVARS; i++) QL[i] = k.qinf[i];
  }
}

// Node state seen by slot p1 of a group whose slots start at p0.  Each
// half-edge ends with a recompute of the node's auxiliary variables, which
// depend only on its conservative values, so one recompute at the end
// stands for all of them.
__device__ void replay_group(const BcConst& k, int p0, int p1, const int* __restrict__ ghe,
                             const int2* __restrict__ bn, const int* __restrict__ bbc,
                             const double* __restrict__ btw, const int* __restrict__ bnrm,
                             const double* __restrict__ q, double* QL) {
  for (int p = p0; p < p1; p++) {
    const int he = ghe[p];
    const int bct = bbc[he];
    if (!hardsets(bct)) continue;
    double nQ[NVARS] = {0};
    if (bct == PCFD_BC_NOSLIP && bnrm[he] >= 0)
      for (int j = 0; j < NVARS; j++) nQ[j] = q[(size_t)bnrm[he] * NVARS + j];
    hardset_node(k, bct, QL, btw[he], nQ, q[(size_t)bn[he].y * NVARS]);
  }
  if (p1 > p0) aux_vars(k.gamma, QL);
}

template <bool DF>
__global__ void k_bc_group_halfedges(int nslot, const int* __restrict__ slot_group, const int* __restrict__ gnode,
                                     const int* __restrict__ gptr, const int* __restrict__ ghe,
                                     const int2* __restrict__ bn, const D4* __restrict__ ba,
                                     const int* __restrict__ bbc, const double* __restrict__ btw,
                                     const int* __restrict__ bnrm, BcConst k, const double* __restrict__ q,
                                     double* __restrict__ qr_out, unsigned long long* health) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nslot) return;
  const int g = slot_group[t];
  const int node = gnode[g];
  double QL[NVARS];
  for (int j = 0; j < NVARS; j++) QL[j] = q[(size_t)node * NVARS + j];
  replay_group(k, gptr[g], t, ghe, bn, bbc, btw, bnrm, q, QL);
  const int he = ghe[t];
  const int ph = bn[he].y;
  const int bct = bbc[he];
  double QR[NVARS];
  for (int j = 0; j < NVARS; j++) QR[j] = q[(size_t)ph * NVARS + j];
  if (DF && (bct == PCFD_BC_FARFIELD || bct == PCFD_BC_IMPERMEABLE_WALL || bct == PCFD_BC_SYMMETRY)) {
    dfl L[NEQN], R[NEQN], Qinf[NVARS];
    for (int j = 0; j < NEQN; j++) L[j] = to_df(QL[j]);
    for (int j = 0; j < NEQN; j++) R[j] = to_df(QR[j]);
    for (int j = 0; j < NVARS; j++) Qinf[j] = to_df(k.qinf[j]);
    const D4 a = ba[he];
    const dfl ax = to_df(a.x), ay = to_df(a.y), az = to_df(a.z), gamma = to_df(k.gamma);
    if (bct == PCFD_BC_FARFIELD) bc_farfield<dfl>(gamma, Qinf, L, to_df(QL[6]), R, ax, ay, az);
    else bc_inviscid_wall<dfl>(gamma, k.no_cvbc, L, to_df(QL[6]), R, ax, ay, az);
    for (int j = 0; j < NEQN; j++) QR[j] = to_dbl(R[j]);
    aux_vars(k.gamma, QR);
  } else {
    double nQ[NVARS] = {0};
    if (bct == PCFD_BC_NOSLIP && bnrm[he] >= 0)
      for (int j = 0; j < NVARS; j++) nQ[j] = q[(size_t)bnrm[he] * NVARS + j];
    if (!apply_bc(k, bct, QL, QR, ba[he], btw[he], nQ)) atomicAdd(&health[H_BADBC], 1ull);
  }
  for (int j = 0; j < NVARS; j++) qr_out[(size_t)t * NVARS + j] = QR[j];
}

__global__ void k_bc_group_nodes(int ngroup, const int* __restrict__ gnode, const int* __restrict__ gptr,
                                 const int* __restrict__ ghe, const int2* __restrict__ bn,
                                 const int* __restrict__ bbc, const double* __restrict__ btw,
                                 const int* __restrict__ bnrm, BcConst k, const double* __restrict__ qr_in,
                                 double* __restrict__ q, dfl* __restrict__ fq) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= ngroup) return;
  const int node = gnode[g];
  double QL[NVARS];
  for (int j = 0; j < NVARS; j++) QL[j] = q[(size_t)node * NVARS + j];
  replay_group(k, gptr[g], gptr[g + 1], ghe, bn, bbc, btw, bnrm, q, QL);
  store_row(q, fq, node, QL);
  for (int p = gptr[g]; p < gptr[g + 1]; p++) store_row(q, fq, bn[ghe[p]].y, &qr_in[(size_t)p * NVARS]);
}

// Half-edges of boundary nodes that no condition hard-sets (far field, walls,
// symmetry, outflow): each writes only its own phantom state, so every
// half-edge is independent.  The node's stored auxiliary variables are left
// as they are (the reference recomputes them from unchanged conservative
// values).
__global__ void k_bc_halfedges(int n, const int* __restrict__ list, const int2* __restrict__ bn,
                               const D4* __restrict__ ba, const int* __restrict__ bbc,
                               const double* __restrict__ btw, BcConst k, double* __restrict__ q,
                               dfl* __restrict__ fq, unsigned long long* health) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  int he = list[t];
  int2 nd = bn[he];
  double QL[NVARS], QR[NVARS];
  for (int j = 0; j < NVARS; j++) QL[j] = q[(size_t)nd.x * NVARS + j];
  for (int j = 0; j < NVARS; j++) QR[j] = q[(size_t)nd.y * NVARS + j];
  double nQ[NVARS] = {0};
  if (!apply_bc(k, bbc[he], QL, QR, ba[he], btw[he], nQ)) atomicAdd(&health[H_BADBC], 1ull);
  store_row(q, fq, nd.y, QR);
}

// The same for the double-float residual arithmetic: far-field and wall
// sub-iterations in double-float, the phantom state written back in FP64.
__global__ void k_bc_halfedges_df(int n, const int* __restrict__ list, const int2* __restrict__ bn,
                                  const D4* __restrict__ ba, const int* __restrict__ bbc, BcConst k,
                                  double* __restrict__ q, dfl* __restrict__ fq, unsigned long long* health) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  int he = list[t];
  int2 nd = bn[he];
  const int bct = bbc[he];
  if (bct != PCFD_BC_FARFIELD && bct != PCFD_BC_IMPERMEABLE_WALL && bct != PCFD_BC_SYMMETRY) {
    // outflow / Neumann: a copy, done in FP64
    double QL[NVARS], QR[NVARS], nQ[NVARS] = {0};
    for (int j = 0; j < NVARS; j++) QL[j] = q[(size_t)nd.x * NVARS + j];
    for (int j = 0; j < NVARS; j++) QR[j] = q[(size_t)nd.y * NVARS + j];
    if (!apply_bc(k, bct, QL, QR, ba[he], 0.0, nQ)) atomicAdd(&health[H_BADBC], 1ull);
    store_row(q, fq, nd.y, QR);
    return;
  }
  dfl QL[NEQN], QR[NEQN], Qinf[NVARS];
  for (int j = 0; j < NEQN; j++) QL[j] = to_df(q[(size_t)nd.x * NVARS + j]);
  for (int j = 0; j < NEQN; j++) QR[j] = to_df(q[(size_t)nd.y * NVARS + j]);
  for (int j = 0; j < NVARS; j++) Qinf[j] = to_df(k.qinf[j]);
  const dfl pi = to_df(q[(size_t)nd.x * NVARS + 6]);
  const D4 a = ba[he];
  const dfl ax = to_df(a.x), ay = to_df(a.y), az = to_df(a.z), gamma = to_df(k.gamma);
  if (bct == PCFD_BC_FARFIELD) bc_farfield<dfl>(gamma, Qinf, QL, pi, QR, ax, ay, az);
  else bc_inviscid_wall<dfl>(gamma, k.no_cvbc, QL, pi, QR, ax, ay, az);
  double Q[NVARS];
  for (int j = 0; j < NEQN; j++) Q[j] = to_dbl(QR[j]);
  aux_vars(k.gamma, Q);
  store_row(q, fq, nd.y, Q);
}

// Exact reference order when a no-slip normal node is itself hard-set by a
// boundary condition: a single thread walks the half-edges in bedge order.
__global__ void k_bc_sequential(int nbedge, const int2* __restrict__ bn, const D4* __restrict__ ba,
                                const int* __restrict__ bbc, const double* __restrict__ btw,
                                const int* __restrict__ bnrm, BcConst k, double* __restrict__ q,
                                unsigned long long* health) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  for (int he = 0; he < nbedge; he++) {
    int2 n = bn[he];
    double* QL = &q[(size_t)n.x * NVARS];
    double* QR = &q[(size_t)n.y * NVARS];
    double nQ[NVARS] = {0};
    int bct = bbc[he];
    if (bct == PCFD_BC_NOSLIP && bnrm[he] >= 0)
      for (int j = 0; j < NVARS; j++) nQ[j] = q[(size_t)bnrm[he] * NVARS + j];
    if (!apply_bc(k, bct, QL, QR, ba[he], btw[he], nQ)) atomicAdd(&health[H_BADBC], 1ull);
  }
}

// -------------------------------------------------------------------------
// weighted LSQ gradient (Gradient::Compute, ucs/gradient.tcc:57)
// Residual-path kernels are templated on the scalar type S: double (the
// reference precision) or dfl (double-float on the FP32 pipes).
// -------------------------------------------------------------------------

__constant__ int c_gradlist[NTERMS] = {0, 1, 2, 3, 4, 5, 7, 8, 9};

template <class S>
__global__ void __launch_bounds__(128) k_gradient(int nnode, const int* __restrict__ nptr,
                                                  const int* __restrict__ nnbr, const S* __restrict__ lsq,
                                                  const S* __restrict__ q, const int* __restrict__ bptr,
                                                  const int* __restrict__ bhe, const int* __restrict__ bbc,
                                                  const typename V4<S>::type* __restrict__ ba, S* __restrict__ grad) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nnode) return;
  S qi[NTERMS];
  for (int t = 0; t < NTERMS; t++) qi[t] = q[(size_t)i * NVARS + c_gradlist[t]];
  S g[NTERMS * 3];
  for (int t = 0; t < NTERMS * 3; t++) g[t] = Sc<S>::c(0.0);
  for (int k = nptr[i]; k < nptr[i + 1]; k++) {
    int j = nnbr[k];
    S c0 = lsq[3 * (size_t)k], c1 = lsq[3 * (size_t)k + 1], c2 = lsq[3 * (size_t)k + 2];
    const S* qj = &q[(size_t)j * NVARS];
#pragma unroll
    for (int t = 0; t < NTERMS; t++) {
      S dq = qj[c_gradlist[t]] - qi[t];
      g[3 * t + 0] += c0 * dq;
      g[3 * t + 1] += c1 * dq;
      g[3 * t + 2] += c2 * dq;
    }
  }
  // Bkernel_Symmetry_Fix (ucs/gradient.tcc:545), in half-edge order
  for (int p = bptr[i]; p < bptr[i + 1]; p++) {
    int he = bhe[p];
    if (bbc[he] != PCFD_BC_SYMMETRY) continue;
    typename V4<S>::type a = ba[he];
#pragma unroll
    for (int t = 0; t < NTERMS; t++) {
      S dot = g[3 * t] * a.x + g[3 * t + 1] * a.y + g[3 * t + 2] * a.z;
      g[3 * t + 0] -= dot * a.x;
      g[3 * t + 1] -= dot * a.y;
      g[3 * t + 2] -= dot * a.z;
    }
  }
  for (int t = 0; t < NTERMS * 3; t++) grad[(size_t)i * NTERMS * 3 + t] = g[t];
}

// -------------------------------------------------------------------------
// limiter (Limiter::Compute, ucs/limiters.tcc:53; limiter = 1, 2, 3)
// -------------------------------------------------------------------------

// The limiter of node i from its state qi, its gradient gi (first NEQN
// terms) and the neighbour bounds qmin/qmax (Kernel_FindMinMax, :135,
// initialised to zero as the reference does): LIM 1 Barth (Kernel_Barth,
// ucs/limiters.tcc:194), 2 Venkatakrishnan (Kernel_Venkat, :372), 3 modified
// Venkatakrishnan (Kernel_VenkatMod, :534).  The half-edge vector of each
// incident edge gives dx = 0.5 (x_j - x_i) (its sign flips when the node is
// the edge's right end).  Writes the raw value, the clamped value (lim may
// be null) and the clip flag.  CHI0: chi = 0, so the extrapolation is
// q + grad.dx exactly and the 0.5 chi dQ term is skipped (bit-identical).
// a fused multiply-add for the FP64 path of the limiter (the double-float
// path never reaches it)
template <class S>
__device__ __forceinline__ S fma_s(S a, S b, S c) { return a * b + c; }
template <>
__device__ __forceinline__ double fma_s<double>(double a, double b, double c) { return fma(a, b, c); }

// Neighbour bounds (Kernel_FindMinMax: qmax = v unless qmax > v, qmin = v
// unless qmin < v).  In FP64 the comparisons run on the integer pipes, on
// keys that order doubles as their values (sign bit flips the magnitude),
// so the FP64 pipe the limiter is bound by does not spend two comparisons
// per neighbour and equation on them; the double-float path compares values.
__device__ __forceinline__ long long dkey(double v) {
  const long long b = __double_as_longlong(v);
  return b ^ ((b >> 63) & 0x7fffffffffffffffLL);
}
template <class S>
__device__ __forceinline__ void bound_upd(S v, S& mn, S& mx, long long&, long long&) {
  mx = (mx > v) ? mx : v;
  mn = (mn < v) ? mn : v;
}
template <>
__device__ __forceinline__ void bound_upd<double>(double v, double& mn, double& mx, long long& kmn, long long& kmx) {
  const long long kv = dkey(v);
  if (!(kmx > kv)) { kmx = kv; mx = v; }
  if (!(kmn < kv)) { kmn = kv; mn = v; }
}

template <class S, int LIM, bool CHI0>
__device__ __forceinline__ void limit_node(int i, int k0, int k1, const int* __restrict__ nedg,
                                           const int* __restrict__ nnbr, const S* __restrict__ q,
                                           const S* __restrict__ eh, const double* __restrict__ vol, double chi_d,
                                           double K3, const S* qi, const S* gi, const S* qmin, const S* qmax,
                                           S* __restrict__ limraw, S* __restrict__ lim, int* __restrict__ clipflag,
                                           S* __restrict__ ext) {
  const S zero = Sc<S>::c(0.0);
  const S chi = Sc<S>::from(chi_d), hchi = Sc<S>::c(0.5) * chi, omc = Sc<S>::c(1.0) - chi;
  const S one = Sc<S>::c(1.0), two = Sc<S>::c(2.0);
  if (LIM != 3) {
    // t = (allowed change) / (extrapolated change), 1 where the extrapolation
    // leaves the value unchanged; Barth clamps t to [0, 1], Venkatakrishnan
    // maps it through (t^2 + 2t) / (t^2 + t + 2) (positive denominator).
    S lm[NEQN];
    for (int t = 0; t < NEQN; t++) lm[t] = one;
    for (int k = k0; k < k1; k++) {
      int se = nedg[k];
      const S* qj = &q[(size_t)nnbr[k] * NVARS];
      const S* hv = &eh[3 * (size_t)(se < 0 ? ~se : se)];
      S dx0 = hv[0], dx1 = hv[1], dx2 = hv[2];
      if (se >= 0) { dx0 = -dx0; dx1 = -dx1; dx2 = -dx2; }
      S* xo = (CHI0 && ext) ? &ext[(size_t)(se < 0 ? ~se : se) * (2 * NEQN) + (se < 0 ? 0 : NEQN)] : nullptr;
#pragma unroll
      for (int t = 0; t < NEQN; t++) {
        S gdx = dot3_ref<S>(gi[3 * t], dx0, gi[3 * t + 1], dx1, gi[3 * t + 2], dx2);
        if (xo) xo[t] = gdx;
        S Q = extrap_ref<S>(qi[t], qj[t] - qi[t], gdx, hchi, omc, CHI0);
        S r = one;
        if (Q > qi[t]) r = (qmax[t] - qi[t]) / (Q - qi[t]);
        else if (Q < qi[t]) r = (qmin[t] - qi[t]) / (Q - qi[t]);
        if (LIM == 1) {
          r = (r > zero) ? r : zero;
          r = (r < one) ? r : one;
        } else {
          r = (r * r + two * r) / (r * r + r + two);
        }
        if (r < lm[t]) lm[t] = r;
      }
    }
    int neg = 0;
    for (int t = 0; t < NEQN; t++) {
      S v = lm[t];
      limraw[(size_t)i * NEQN + t] = v;
      if (v < zero) neg = 1;
      if (lim) lim[(size_t)i * NEQN + t] = (v < zero) ? zero : v;
    }
    clipflag[i] = neg ? 2 : 0;
    return;
  }
  const S ep2 = Sc<S>::from(6.0 * 3.141592653589793 * vol[i] * K3);
  // The limiter is min(1, min_k num_k / den_k) with every den_k > 0
  // (den = (DP + DM/2)^2 + 7/4 DM^2 + eps^2).  The running minimum is kept
  // as a fraction and compared by cross-multiplication, so only one
  // division per equation remains instead of one per edge and equation.
  // DP takes one of two values per equation (qmax - q or qmin - q, by the
  // sign of DM); both and their squares are formed once, outside the
  // neighbour loop together with DP^2 + eps^2.  FP64 forms DM as the
  // reference does (extrapolated value minus node value, in its rounding,
  // since the sign of DM picks DP) and then num = DP^2 + eps^2 + 2 DM DP and
  // den = DP^2 + eps^2 + DM (DP + 2 DM) with fused multiply-adds: three FP64
  // instructions where the reference's expression order takes eight (the
  // FP64 pipe bounds this kernel); double-float forms DM as the
  // extrapolation's correction itself.
  constexpr bool F64 = std::is_same<S, double>::value;
  S dpp[NEQN], dpm[NEQN], bp[NEQN], bm[NEQN], bn[NEQN], bd[NEQN];
  for (int t = 0; t < NEQN; t++) {
    dpp[t] = qmax[t] - qi[t];
    dpm[t] = qmin[t] - qi[t];
    bp[t] = dpp[t] * dpp[t] + ep2;
    bm[t] = dpm[t] * dpm[t] + ep2;
    bn[t] = one;
    bd[t] = one;
  }
  for (int k = k0; k < k1; k++) {
    int se = nedg[k];
    const S* qj = &q[(size_t)nnbr[k] * NVARS];
    const S* hv = &eh[3 * (size_t)(se < 0 ? ~se : se)];
    S dx0 = hv[0], dx1 = hv[1], dx2 = hv[2];
    if (se >= 0) { dx0 = -dx0; dx1 = -dx1; dx2 = -dx2; }
    S* xo = (CHI0 && ext) ? &ext[(size_t)(se < 0 ? ~se : se) * (2 * NEQN) + (se < 0 ? 0 : NEQN)] : nullptr;
#pragma unroll
    for (int t = 0; t < NEQN; t++) {
      S gdx = dot3_ref<S>(gi[3 * t], dx0, gi[3 * t + 1], dx1, gi[3 * t + 2], dx2);
      if (xo) xo[t] = gdx;
      S corr = CHI0 ? gdx : hchi * (qj[t] - qi[t]) + omc * gdx;
      S num, den;
      if (F64) {
        S Q = extrap_ref<S>(qi[t], qj[t] - qi[t], gdx, hchi, omc, CHI0);
        S DM = Q - qi[t];
        bool pos = Q > qi[t];
        S DP = pos ? dpp[t] : dpm[t];
        S C1 = pos ? bp[t] : bm[t];
        num = fma_s(DM, DP + DP, C1);
        den = fma_s(DM, fma_s(Sc<S>::c(2.0), DM, DP), C1);
      } else {
        S DM = corr;
        bool pos = DM > zero;
        S DP = pos ? dpp[t] : dpm[t];
        S P2 = pos ? bp[t] : bm[t];
        S mp = DM * DP;
        num = P2 + twice(mp);
        den = P2 + twice(DM * DM) + mp;
      }
      if (num * bd[t] < bn[t] * den) { bn[t] = num; bd[t] = den; }
    }
  }
  // raw values (possibly negative) feed the pressure clip; the clamp to
  // zero comes after it (ucs/limiters.tcc:110-124)
  int neg = 0;
  for (int t = 0; t < NEQN; t++) {
    S v = (bd[t] == one) ? bn[t] : bn[t] / bd[t];
    limraw[(size_t)i * NEQN + t] = v;
    if (v < zero) neg = 1;
    if (lim) lim[(size_t)i * NEQN + t] = (v < zero) ? zero : v;
  }
  clipflag[i] = neg ? 2 : 0;
}

// Standalone limiter (Limiter<T>::Compute after a separate gradient): the
// neighbour bounds, then limit_node.
template <class S, int LIM, bool CHI0>
__global__ void __launch_bounds__(128) k_venkat(int nnode, const int* __restrict__ nptr,
                                                const int* __restrict__ nedg, const int* __restrict__ nnbr,
                                                const S* __restrict__ q, const S* __restrict__ grad,
                                                const S* __restrict__ eh, const double* __restrict__ vol, double chi_d,
                                                double K3, S* __restrict__ limraw, S* __restrict__ lim,
                                                int* __restrict__ clipflag, S* __restrict__ ext) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nnode) return;
  const S zero = Sc<S>::c(0.0);
  S qi[NEQN], qmin[NEQN], qmax[NEQN], gi[NEQN * 3];
  for (int t = 0; t < NEQN; t++) {
    qi[t] = q[(size_t)i * NVARS + t];
    qmin[t] = zero;
    qmax[t] = zero;
  }
  for (int t = 0; t < NEQN * 3; t++) gi[t] = grad[(size_t)i * NTERMS * 3 + t];
  const int k0 = nptr[i], k1 = nptr[i + 1];
  long long kmn[NEQN], kmx[NEQN];
  for (int t = 0; t < NEQN; t++) kmn[t] = kmx[t] = 0;  // the key of +0.0, the bounds' start
  for (int k = k0; k < k1; k++) {
    const S* qj = &q[(size_t)nnbr[k] * NVARS];
    for (int t = 0; t < NEQN; t++) bound_upd<S>(qj[t], qmin[t], qmax[t], kmn[t], kmx[t]);
  }
  limit_node<S, LIM, CHI0>(i, k0, k1, nedg, nnbr, q, eh, vol, chi_d, K3, qi, gi, qmin, qmax, limraw, lim, clipflag,
                           ext);
}

// BadExtrapolation (ucs/compressible.tcc:1056)
template <class S>
__device__ __forceinline__ int bad_extrap(S gamma, const S* Q) {
  S r = Q[0];
  S ir = Sc<S>::c(1.0) / r;
  S u = Q[1] * ir, v = Q[2] * ir, w = Q[3] * ir;
  S p = (gamma - Sc<S>::c(1.0)) * (Q[4] - r * (Sc<S>::c(0.5) * (u * u + v * v + w * w)));
  const S tiny = Sc<S>::c(1.0e-10);
  return (p < tiny) || (r < Sc<S>::c(0.0)) || (Q[4] < tiny);
}

// Extrapolated states of one edge with the given limiters and the three
// BadExtrapolation tests of Kernel_PressureClip (ucs/limiters.tcc:737):
// bit 0 left, bit 1 right, bit 2 Roe average.  h = 0.5 (x_R - x_L).
template <class S>
__device__ int clip_check(const S* qL, const S* qR, const S* gL, const S* gR, const S* lL, const S* lR, S h0, S h1,
                          S h2, S chi, S gamma) {
  const S hchi = Sc<S>::c(0.5) * chi, omc = Sc<S>::c(1.0) - chi;
  S Qi[NEQN], Qj[NEQN];
  for (int t = 0; t < NEQN; t++) {
    S dQ = qR[t] - qL[t];
    Qi[t] = qL[t] + (hchi * dQ + omc * (gL[3 * t] * h0 + gL[3 * t + 1] * h1 + gL[3 * t + 2] * h2)) * lL[t];
    Qj[t] = qR[t] + (hchi * (-dQ) + omc * (gR[3 * t] * (-h0) + gR[3 * t + 1] * (-h1) + gR[3 * t + 2] * (-h2))) * lR[t];
  }
  int m = 0;
  if (bad_extrap(gamma, Qi)) m |= 1;
  if (bad_extrap(gamma, Qj)) m |= 2;
  const S gm1 = gamma - Sc<S>::c(1.0), half = Sc<S>::c(0.5);
  S rL = Qi[0], rR = Qj[0];
  S uL = Qi[1] / rL, vL = Qi[2] / rL, wL = Qi[3] / rL;
  S uR = Qj[1] / rR, vR = Qj[2] / rR, wR = Qj[3] / rR;
  S PL = gm1 * (Qi[4] - half * rL * (uL * uL + vL * vL + wL * wL));
  S PR = gm1 * (Qj[4] - half * rR * (uR * uR + vR * vR + wR * wR));
  S hL = (Qi[4] + PL) / rL, hR = (Qj[4] + PR) / rR;
  S rho = sqrt(rL * rR);
  S sg = rho / (rL + rho);
  S u = uL + sg * (uR - uL), v = vL + sg * (vR - vL), w = wL + sg * (wR - wL), h = hL + sg * (hR - hL);
  S v2h = half * (u * u + v * v + w * w);
  S Qr[NEQN] = {rho, rho * u, rho * v, rho * w, rho / gamma * (h + gm1 * v2h)};
  if (bad_extrap(gamma, Qr)) m |= 4;
  return m;
}

// The three BadExtrapolation tests of clip_check for the states built from
// stored MUSCL corrections c (the limiter pass's grad.dx of each end):
// Q = q + c * l with the raw limiter l, then the Roe average.
template <class S>
__device__ int clip_check_ext(const S* qL, const S* qR, const S* c, const S* lL, const S* lR, S gamma) {
  S Qi[NEQN], Qj[NEQN];
  for (int t = 0; t < NEQN; t++) {
    Qi[t] = qL[t] + c[t] * lL[t];
    Qj[t] = qR[t] + c[NEQN + t] * lR[t];
  }
  int m = 0;
  if (bad_extrap(gamma, Qi)) m |= 1;
  if (bad_extrap(gamma, Qj)) m |= 2;
  const S gm1 = gamma - Sc<S>::c(1.0), half = Sc<S>::c(0.5);
  S rL = Qi[0], rR = Qj[0];
  S uL = Qi[1] / rL, vL = Qi[2] / rL, wL = Qi[3] / rL;
  S uR = Qj[1] / rR, vR = Qj[2] / rR, wR = Qj[3] / rR;
  S PL = gm1 * (Qi[4] - half * rL * (uL * uL + vL * vL + wL * wL));
  S PR = gm1 * (Qj[4] - half * rR * (uR * uR + vR * vR + wR * wR));
  S hL = (Qi[4] + PL) / rL, hR = (Qj[4] + PR) / rR;
  S rho = sqrt(rL * rR);
  S sg = rho / (rL + rho);
  S u = uL + sg * (uR - uL), v = vL + sg * (vR - vL), w = wL + sg * (wR - wL), h = hL + sg * (hR - hL);
  S v2h = half * (u * u + v * v + w * w);
  S Qr[NEQN] = {rho, rho * u, rho * v, rho * w, rho / gamma * (h + gm1 * v2h)};
  if (bad_extrap(gamma, Qr)) m |= 4;
  return m;
}

// An FP32 value of x on the integer pipes: sign, exponent and the top 23
// significand bits of the double, truncated (relative error below 2^-23),
// 0 below FP32's normal range, infinity above it, NaN for a non-finite x.
// An FP64 to FP32 conversion instruction would issue on the FP64 pipe, which
// the edge pass is bound by.
__device__ __forceinline__ float f32_of(double x) {
  const int hi = __double2hiint(x);
  const unsigned lo = (unsigned)__double2loint(x);
  const int e = (hi >> 20) & 0x7ff;
  const int fe = e - 1023 + 127;
  unsigned bits;
  if (e == 0x7ff) bits = 0x7fc00000u;
  else if (fe <= 0) bits = 0u;
  else if (fe >= 255) bits = 0x7f800000u;
  else bits = ((unsigned)fe << 23) | ((unsigned)(hi & 0xfffff) << 3) | (lo >> 29);
  return __uint_as_float(bits | ((unsigned)hi & 0x80000000u));
}
__device__ __forceinline__ float f32_of(dfl x) { return x.hi; }

// True when the three tests of clip_check_ext certainly pass (no clip),
// decided in FP32: each tested quantity (density, total energy, pressure of
// both extrapolated states and of their Roe average) must exceed the test's
// threshold by 1e-3 of the magnitudes it is formed from, two orders above
// the FP32 evaluation's own error (below 1e-5 of those magnitudes once each
// density keeps at least a tenth of its parts, which the pass also asks).
// False sends the edge to the exact test.
template <class S>
__device__ bool clip_clear_f32(const S* qL, const S* qR, const S* c, const S* lL, const S* lR, float gamma) {
  const float tiny = 1.0e-10f, mrg = 1.0e-3f, gm1 = gamma - 1.0f;
  float Q[2][NEQN], M[2][NEQN];
  for (int t = 0; t < NEQN; t++) {
    float a = f32_of(qL[t]), d = f32_of(c[t]) * f32_of(lL[t]);
    Q[0][t] = a + d;
    M[0][t] = fabsf(a) + fabsf(d);
    a = f32_of(qR[t]);
    d = f32_of(c[NEQN + t]) * f32_of(lR[t]);
    Q[1][t] = a + d;
    M[1][t] = fabsf(a) + fabsf(d);
  }
  float u[2], v[2], w[2], h[2], hm[2];
  for (int k = 0; k < 2; k++) {
    const float r = Q[k][0];
    if (!(r > 0.1f * M[k][0])) return false;
    const float ir = 1.0f / r;
    u[k] = Q[k][1] * ir;
    v[k] = Q[k][2] * ir;
    w[k] = Q[k][3] * ir;
    const float ke = 0.5f * r * (u[k] * u[k] + v[k] * v[k] + w[k] * w[k]);
    const float sc = M[k][4] + ke;
    const float p = gm1 * (Q[k][4] - ke);
    if (!(Q[k][4] > tiny + mrg * M[k][4]) || !(p > tiny + mrg * gm1 * sc)) return false;
    h[k] = (Q[k][4] + p) * ir;
    hm[k] = (M[k][4] + gm1 * sc) * ir;
  }
  const float rho = sqrtf(Q[0][0] * Q[1][0]);
  const float sg = rho / (Q[0][0] + rho);
  const float ur = u[0] + sg * (u[1] - u[0]), vr = v[0] + sg * (v[1] - v[0]), wr = w[0] + sg * (w[1] - w[0]);
  const float hr = h[0] + sg * (h[1] - h[0]);
  const float v2h = 0.5f * (ur * ur + vr * vr + wr * wr);
  const float e4 = rho / gamma * (hr + gm1 * v2h);
  const float ke = rho * v2h;
  const float sc = rho / gamma * (hm[0] + hm[1] + gm1 * v2h) + ke;
  const float p = gm1 * (e4 - ke);
  return rho > 0.0f && e4 > tiny + mrg * sc && p > tiny + mrg * gm1 * sc;
}

__device__ __forceinline__ int bad_extrap_d(double gamma, const double* Q) {
  double r = Q[0];
  double ir = 1.0 / r;
  double u = Q[1] * ir, v = Q[2] * ir, w = Q[3] * ir;
  double p = (gamma - 1.0) * (Q[4] - r * (0.5 * (u * u + v * v + w * w)));
  return (p < 1.0e-10) || (r < 0.0) || (Q[4] < 1.0e-10);
}

// Kernel_PressureClip (ucs/limiters.tcc:737) evaluated with the post-limiter
// values on both sides of every edge; a node whose own extrapolation, or the
// Roe average with any neighbour's, is non-physical gets a zero limiter.
// (The reference applies the same test edge by edge in sequence; the two
// agree whenever no clip fires, and clips are counted in the health word.)
__global__ void __launch_bounds__(128) k_pressure_clip(int nnode, const int* __restrict__ nptr,
                                                       const int* __restrict__ nnbr, const double* __restrict__ q,
                                                       const double* __restrict__ grad,
                                                       const double* __restrict__ xyz, double chi, double gamma,
                                                       const double* __restrict__ lim_in, double* __restrict__ lim_out,
                                                       unsigned long long* health) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nnode) return;
  double li[NEQN];
  for (int t = 0; t < NEQN; t++) li[t] = lim_in[(size_t)i * NEQN + t];
  int clip = 0;
  const double* qi = &q[(size_t)i * NVARS];
  const double* gi = &grad[(size_t)i * NTERMS * 3];
  for (int k = nptr[i]; k < nptr[i + 1] && !clip; k++) {
    int j = nnbr[k];
    const double* qj = &q[(size_t)j * NVARS];
    const double* gj = &grad[(size_t)j * NTERMS * 3];
    double dx[3], Qi[NEQN], Qj[NEQN];
    for (int c = 0; c < 3; c++) dx[c] = 0.5 * (xyz[3 * j + c] - xyz[3 * i + c]);
    for (int t = 0; t < NEQN; t++) {
      double dQ = qj[t] - qi[t];
      Qi[t] = qi[t] + (0.5 * chi * dQ + (1.0 - chi) * (gi[3 * t] * dx[0] + gi[3 * t + 1] * dx[1] + gi[3 * t + 2] * dx[2])) * li[t];
      double lj = lim_in[(size_t)j * NEQN + t];
      Qj[t] = qj[t] + (0.5 * chi * (-dQ) + (1.0 - chi) * (gj[3 * t] * (-dx[0]) + gj[3 * t + 1] * (-dx[1]) + gj[3 * t + 2] * (-dx[2]))) * lj;
    }
    if (bad_extrap_d(gamma, Qi)) { clip = 1; break; }
    // RoeVariables (ucs/compressible.tcc:533) of the pair, then the same test
    double gm1 = gamma - 1.0;
    double rL = Qi[0], rR = Qj[0];
    double uL = Qi[1] / rL, vL = Qi[2] / rL, wL = Qi[3] / rL;
    double uR = Qj[1] / rR, vR = Qj[2] / rR, wR = Qj[3] / rR;
    double PL = gm1 * (Qi[4] - 0.5 * rL * (uL * uL + vL * vL + wL * wL));
    double PR = gm1 * (Qj[4] - 0.5 * rR * (uR * uR + vR * vR + wR * wR));
    double hL = (Qi[4] + PL) / rL, hR = (Qj[4] + PR) / rR;
    double rho = sqrt(rL * rR);
    double sg = rho / (rL + rho);
    double u = uL + sg * (uR - uL), v = vL + sg * (vR - vL), w = wL + sg * (wR - wL), h = hL + sg * (hR - hL);
    double v2h = 0.5 * (u * u + v * v + w * w);
    double Qr[NEQN] = {rho, rho * u, rho * v, rho * w, rho / gamma * (h + gm1 * v2h)};
    if (bad_extrap_d(gamma, Qr)) { clip = 1; break; }
  }
  if (clip) atomicAdd(&health[H_LIMCLIP], 1ull);
  for (int t = 0; t < NEQN; t++) {
    double v = clip ? 0.0 : li[t];
    lim_out[(size_t)i * NEQN + t] = (v < 0.0) ? 0.0 : v;
  }
}

// -------------------------------------------------------------------------
// residual (SpatialResidual, ucs/residual.tcc:66)
// -------------------------------------------------------------------------

// the flux constants in one scalar type
template <class S>
struct FluxK {
  S gamma, gm1, igamma, igm1, chi, hchi, omc, inv_retilde, Sc_, cp_over_pr;
};

struct FluxConst {
  double gamma, chi;
  int ho, viscous;
  int clip;            // second order with a limiter: the pressure clip applies
  double inv_retilde;  // Mach / Re
  double S;            // Sutherland constant / T_ref
  double cp_over_pr;   // (1/(gamma-1)) / Pr
  FluxK<double> kd;    // derived constants, FP64
  FluxK<dfl> kf;       // the same split into double-float on the host
};

template <class S>
__device__ __forceinline__ const FluxK<S>& flux_k(const FluxConst& k);
template <>
__device__ __forceinline__ const FluxK<double>& flux_k<double>(const FluxConst& k) { return k.kd; }
template <>
__device__ __forceinline__ const FluxK<dfl>& flux_k<dfl>(const FluxConst& k) { return k.kf; }

template <class S>
__device__ __forceinline__ int kneecap5(S* f) {
  int bad = 0;
#pragma unroll
  for (int i = 0; i < NEQN; i++)
    if (isnan(f[i])) { f[i] = Sc<S>::c(0.0); bad = 1; }
  return bad;
}

// Kernel_Inviscid_Flux (:192) for one edge, stored as the flux leaving the
// left node (k_edge_visc adds the viscous part).
// MODE 0: plain evaluation.  MODE 1: also flags the nodes whose extrapolated
// or Roe-averaged states are non-physical - the pressure clip of the limiter
// (ucs/limiters.tcc:737) tests exactly these states, so when nothing is
// flagged the clip is a no-op and the fluxes already stand.  MODE 2:
// re-evaluates only edges touching a flagged node, after their limiters were
// zeroed; it returns at once when nothing was flagged.  CHI0: chi = 0, so
// the MUSCL correction is grad.dx alone (bit-identical to the general form).
// EXT (chi = 0): both ends' corrections come from ext, as the limiter pass
// formed them from the same gradient, instead of the gradient gathers.
template <class S, int MODE, bool CHI0, bool EXT>
__global__ void __launch_bounds__(128) k_edge_flux(int nedge, const int2* __restrict__ en,
                                                   const typename V4<S>::type* __restrict__ ea,
                                                   const S* __restrict__ eh, const S* __restrict__ q,
                                                   const S* __restrict__ grad, const S* __restrict__ lim, FluxConst kd,
                                                   S* __restrict__ ef, unsigned long long* health,
                                                   int* __restrict__ clipflag, int* __restrict__ clipany,
                                                   const S* __restrict__ limraw, const S* __restrict__ ext) {
  if (MODE == 2 && *(volatile int*)clipany == 0) return;
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nedge) return;
  const int2 n = en[e];
  if (MODE == 2 && !((clipflag[n.x] | clipflag[n.y]) & 1)) return;
  const FluxK<S>& k = flux_k<S>(kd);
  const typename V4<S>::type a = ea[e];
  const S* qL = &q[(size_t)n.x * NVARS];
  const S* qR = &q[(size_t)n.y * NVARS];
  S QL[NEQN], QR[NEQN];
#pragma unroll
  for (int t = 0; t < NEQN; t++) { QL[t] = qL[t]; QR[t] = qR[t]; }
  S h0 = Sc<S>::c(0.0), h1 = h0, h2 = h0;
  if (!EXT && (kd.ho || kd.viscous)) { h0 = eh[3 * (size_t)e]; h1 = eh[3 * (size_t)e + 1]; h2 = eh[3 * (size_t)e + 2]; }
  if (EXT) {
    const S* xe = &ext[(size_t)e * (2 * NEQN)];
    const S* lL = &lim[(size_t)n.x * NEQN];
    const S* lR = &lim[(size_t)n.y * NEQN];
#pragma unroll
    for (int t = 0; t < NEQN; t++) {
      QL[t] = qL[t] + xe[t] * lL[t];
      QR[t] = qR[t] + xe[NEQN + t] * lR[t];
    }
  } else if (kd.ho) {
    const S* gL = &grad[(size_t)n.x * NTERMS * 3];
    const S* gR = &grad[(size_t)n.y * NTERMS * 3];
    const S* lL = &lim[(size_t)n.x * NEQN];
    const S* lR = &lim[(size_t)n.y * NEQN];
#pragma unroll
    for (int t = 0; t < NEQN; t++) {
      S gl = gL[3 * t] * h0 + gL[3 * t + 1] * h1 + gL[3 * t + 2] * h2;
      S gr = gR[3 * t] * (-h0) + gR[3 * t + 1] * (-h1) + gR[3 * t + 2] * (-h2);
      S cl, cr;
      if (CHI0) {
        cl = gl;
        cr = gr;
      } else {
        S dQ = qR[t] - qL[t];
        cl = k.hchi * dQ + k.omc * gl;
        cr = k.hchi * (-dQ) + k.omc * gr;
      }
      QL[t] = qL[t] + cl * lL[t];
      QR[t] = qR[t] + cr * lR[t];
    }
  }
  S f[NEQN];
  int bad = roe_flux(QL, QR, a.x, a.y, a.z, a.w, k.gamma, k.gm1, k.igamma, k.igm1, f);
  if (MODE == 1 && kd.clip && ((clipflag[n.x] | clipflag[n.y]) & 2)) {
    // an endpoint had negative raw limiter values, which the clip sees
    // before they are clamped: test the states it would build
    if (EXT) {
      // from the stored corrections; an FP32 pass clears the edge when its
      // states are far from every threshold, the exact test decides the rest
      const S* xe = &ext[(size_t)e * (2 * NEQN)];
      const S* rl = &limraw[(size_t)n.x * NEQN];
      const S* rr = &limraw[(size_t)n.y * NEQN];
      bad = clip_clear_f32(qL, qR, xe, rl, rr, (float)kd.gamma) ? 0 : clip_check_ext(qL, qR, xe, rl, rr, k.gamma);
    } else {
      bad = clip_check(qL, qR, &grad[(size_t)n.x * NTERMS * 3], &grad[(size_t)n.y * NTERMS * 3],
                       &limraw[(size_t)n.x * NEQN], &limraw[(size_t)n.y * NEQN], h0, h1, h2, k.chi, k.gamma);
    }
  }
  if (MODE == 1 && kd.clip && bad) {
    if (bad & 5) atomicOr(&clipflag[n.x], 1);
    if (bad & 6) atomicOr(&clipflag[n.y], 1);
    atomicOr(clipany, 1);
  }
  if (kneecap5(f)) atomicAdd(&health[H_KNEECAP], 1ull);
#pragma unroll
  for (int t = 0; t < NEQN; t++) ef[(size_t)e * NEQN + t] = f[t];
}

// Kernel_Viscous_Flux (:390) for one edge, added to the stored inviscid
// flux.  A separate pass keeps each of the two kernels' code and register
// footprint small (the double-float forms are long).
template <class S>
__global__ void __launch_bounds__(128) k_edge_visc(int nedge, const int2* __restrict__ en,
                                                   const typename V4<S>::type* __restrict__ ea,
                                                   const S* __restrict__ eh, const S* __restrict__ q,
                                                   const S* __restrict__ grad, FluxConst kd, S* __restrict__ ef) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nedge) return;
  const int2 n = en[e];
  const FluxK<S>& k = flux_k<S>(kd);
  const typename V4<S>::type a = ea[e];
  const S* qL = &q[(size_t)n.x * NVARS];
  const S* qR = &q[(size_t)n.y * NVARS];
  const S h0 = eh[3 * (size_t)e], h1 = eh[3 * (size_t)e + 1], h2 = eh[3 * (size_t)e + 2];
  {
    // face state: plain average of the nodal conservative variables
    S Q0 = halve(qL[0] + qR[0]), Q1 = halve(qL[1] + qR[1]), Q2 = halve(qL[2] + qR[2]), Q3 = halve(qL[3] + qR[3]),
      Q4 = halve(qL[4] + qR[4]);
    S iQ0 = Sc<S>::c(1.0) / Q0;
    S u = Q1 * iQ0, v = Q2 * iQ0, w = Q3 * iQ0;
    S P = k.gm1 * (Q4 - halve(Q0) * (u * u + v * v + w * w));
    S T = k.gamma * P * iQ0;
    const S* gL = &grad[(size_t)n.x * NTERMS * 3];
    const S* gR = &grad[(size_t)n.y * NTERMS * 3];
    S g[NTERMS * 3];
#pragma unroll
    for (int t = 0; t < NTERMS * 3; t++) g[t] = halve(gL[t] + gR[t]);
    if (kd.ho) {
      // directional correction along the edge (dx = xR - xL = 2 h)
      S d0 = twice(h0), d1 = twice(h1), d2 = twice(h2);
      S s2 = d0 * d0 + d1 * d1 + d2 * d2;
      S is2 = Sc<S>::c(1.0) / s2;
#pragma unroll
      for (int t = 0; t < NTERMS; t++) {
        S qdots = d0 * g[3 * t] + d1 * g[3 * t + 1] + d2 * g[3 * t + 2];
        int loc = c_gradlist[t];
        S dq = (qR[loc] - qL[loc] - qdots) * is2;
        g[3 * t] += dq * d0;
        g[3 * t + 1] += dq * d1;
        g[3 * t + 2] += dq * d2;
      }
    }
    S fv[NEQN];
    viscous_flux(u, v, w, T, g, a.x, a.y, a.z, a.w * k.inv_retilde, k.Sc_, k.cp_over_pr, fv);
#pragma unroll
    for (int t = 0; t < NEQN; t++) ef[(size_t)e * NEQN + t] += fv[t];
  }
}

// Zeroes the limiter of every flagged node (the pressure clip); returns at
// once when nothing was flagged.
template <class S>
__global__ void k_clip_apply(int nnode, const int* __restrict__ clipflag, const int* __restrict__ clipany,
                             S* __restrict__ lim, unsigned long long* health) {
  if (*(volatile const int*)clipany == 0) return;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnode; i += gridDim.x * blockDim.x) {
    if (clipflag[i] & 1) {
      for (int t = 0; t < NEQN; t++) lim[(size_t)i * NEQN + t] = Sc<S>::c(0.0);
      atomicAdd(&health[H_LIMCLIP], 1ull);
    }
  }
}

// Bkernel_Inviscid_Flux (:299) + Bkernel_Viscous_Flux (:472) for one
// half-edge (boundary node, phantom node).
template <class S>
__global__ void __launch_bounds__(128) k_bedge_flux(int nbedge, const int2* __restrict__ bn,
                                                    const typename V4<S>::type* __restrict__ ba,
                                                    const S* __restrict__ q, const S* __restrict__ grad, FluxConst kd,
                                                    S* __restrict__ bf, unsigned long long* health) {
  int he = blockIdx.x * blockDim.x + threadIdx.x;
  if (he >= nbedge) return;
  const FluxK<S>& k = flux_k<S>(kd);
  const int2 n = bn[he];
  const typename V4<S>::type a = ba[he];
  const S* qL = &q[(size_t)n.x * NVARS];
  const S* qR = &q[(size_t)n.y * NVARS];
  S QL[NEQN], QR[NEQN], f[NEQN];
#pragma unroll
  for (int t = 0; t < NEQN; t++) { QL[t] = qL[t]; QR[t] = qR[t]; }
  roe_flux(QL, QR, a.x, a.y, a.z, a.w, k.gamma, k.gm1, k.igamma, k.igm1, f);
  if (kneecap5(f)) atomicAdd(&health[H_KNEECAP], 1ull);
  if (kd.viscous) {
    S Q0 = halve(qL[0] + qR[0]), Q1 = halve(qL[1] + qR[1]), Q2 = halve(qL[2] + qR[2]), Q3 = halve(qL[3] + qR[3]),
      Q4 = halve(qL[4] + qR[4]);
    S iQ0 = Sc<S>::c(1.0) / Q0;
    S u = Q1 * iQ0, v = Q2 * iQ0, w = Q3 * iQ0;
    S P = k.gm1 * (Q4 - halve(Q0) * (u * u + v * v + w * w));
    S T = k.gamma * P * iQ0;
    S fv[NEQN];
    viscous_flux(u, v, w, T, &grad[(size_t)n.x * NTERMS * 3], a.x, a.y, a.z, a.w * k.inv_retilde, k.Sc_,
                 k.cp_over_pr, fv);
#pragma unroll
    for (int t = 0; t < NEQN; t++) f[t] += fv[t];
  }
#pragma unroll
  for (int t = 0; t < NEQN; t++) bf[(size_t)he * NEQN + t] = f[t];
}

// b_i = sum over incident edges in ascending edge id (-F_e if i is the left
// node, +F_e otherwise) - sum of its half-edge fluxes; then the no-slip
// residual hook (ModifyViscousWallResidual, ucs/compressible.tcc:1612) and
// per-block partial sums of b^2 for the norms.  The sum runs in S and b is
// stored in FP64.
template <class S>
__global__ void __launch_bounds__(kNormThreads) k_gather(int nnode, const int* __restrict__ nptr,
                                                         const int* __restrict__ nedg, const S* __restrict__ ef,
                                                         const int* __restrict__ bptr, const int* __restrict__ bhe,
                                                         const S* __restrict__ bf, const int* __restrict__ bbc,
                                                         const double* __restrict__ btw, double* __restrict__ b,
                                                         double* __restrict__ part, int* __restrict__ clipflag,
                                                         const int* __restrict__ clipany,
                                                         const double* __restrict__ q,
                                                         const double* __restrict__ qold,
                                                         const double* __restrict__ vol, double timestep) {
  __shared__ double red[kNormThreads / 32][6];
  double acc[6] = {0, 0, 0, 0, 0, 0};
  const int any = *(volatile const int*)clipany;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnode; i += gridDim.x * blockDim.x) {
    if (any && (clipflag[i] & 1)) clipflag[i] &= ~1;
    S r[NEQN];
#pragma unroll
    for (int t = 0; t < NEQN; t++) r[t] = Sc<S>::c(0.0);
    for (int k = nptr[i]; k < nptr[i + 1]; k++) {
      int se = nedg[k];
      if (se < 0) {
        const S* f = &ef[(size_t)(~se) * NEQN];
#pragma unroll
        for (int t = 0; t < NEQN; t++) r[t] += -f[t];
      } else {
        const S* f = &ef[(size_t)se * NEQN];
#pragma unroll
        for (int t = 0; t < NEQN; t++) r[t] += f[t];
      }
    }
    for (int p = bptr[i]; p < bptr[i + 1]; p++) {
      int he = bhe[p];
      const S* f = &bf[(size_t)he * NEQN];
#pragma unroll
      for (int t = 0; t < NEQN; t++) r[t] += -f[t];
    }
    double rd[NEQN];
#pragma unroll
    for (int t = 0; t < NEQN; t++) rd[t] = Sc<S>::to(r[t]);
    if (qold) {
      // TemporalResidual (ucs/residual.tcc:150-175), first order: b -= (vol/dt) (q - q_old),
      // in the reference's rounding (no contraction)
      const double c = vol[i] / timestep;
#pragma unroll
      for (int t = 0; t < NEQN; t++)
        rd[t] = __dsub_rn(rd[t], __dmul_rn(c, __dsub_rn(q[(size_t)i * NVARS + t], qold[(size_t)i * NEQN + t])));
    }
    for (int p = bptr[i]; p < bptr[i + 1]; p++) {
      int he = bhe[p];
      if (bbc[he] != PCFD_BC_NOSLIP) continue;
      rd[1] = 0.0; rd[2] = 0.0; rd[3] = 0.0; rd[4] = 0.0;
      if (btw[he] < 0.0) rd[0] = 0.0;
    }
#pragma unroll
    for (int t = 0; t < NEQN; t++) {
      b[(size_t)i * NEQN + t] = rd[t];
      acc[1 + t] += rd[t] * rd[t];
    }
  }
  acc[0] = acc[1] + acc[2] + acc[3] + acc[4] + acc[5];
  // deterministic block reduction: warp shuffles then a fixed-order sum
  for (int c = 0; c < 6; c++) {
    double v = acc[c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][c] = v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double v = 0.0;
    for (int w = 0; w < kNormThreads / 32; w++) v += red[w][threadIdx.x];
    part[(size_t)blockIdx.x * 6 + threadIdx.x] = v;
  }
}

// Sum of column k of nb per-block partials (row stride st) by one warp in a
// fixed order: lane l adds rows l, l+32, ... in turn, then a butterfly;
// lane 0's value is the result.  Reads bypass L1 (the partials come from
// other blocks of the same launch in k_mdot).
__device__ __forceinline__ double warp_col_sum(const double* part, int nb, int st, int k, int lane) {
  double v = 0.0;
#pragma unroll 8
  for (int b = lane; b < nb; b += 32) v += __ldcg(&part[(size_t)b * st + k]);
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// a warp per norm, each summing the per-block partials in a fixed order
__global__ void k_norm_final(int nblocks, int nnode, const double* __restrict__ part, double* __restrict__ norms,
                             int* __restrict__ clipany) {
  const int lane = threadIdx.x & 31, c = threadIdx.x >> 5;
  if (threadIdx.x == 0) *clipany = 0;
  if (c >= 6) return;
  const double v = warp_col_sum(part, nblocks, 6, c, lane);
  if (lane == 0) norms[c] = c == 0 ? sqrt(v) / ((double)nnode * NEQN) : sqrt(v) / (double)nnode;
}

// FP64 -> double-float copies (state each evaluation; static geometry once)
__global__ void k_df_to_f64(long long n, const dfl* __restrict__ in, double* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = to_dbl(in[i]);
}
__global__ void k_to_df(long long n, const double* __restrict__ in, dfl* __restrict__ out) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = to_df(in[i]);
}
#include "implicit.cuh"
#include "learned.cuh"

// -------------------------------------------------------------------------
// host helpers
// -------------------------------------------------------------------------

template <class T>
int dalloc(T** p, size_t n) {
  if (n == 0) n = 1;
  cudaError_t e = cudaMalloc((void**)p, n * sizeof(T));
  if (e != cudaSuccess) return set_err(PCFD_ERR_NOMEM, std::string("cudaMalloc: ") + cudaGetErrorString(e));
  return PCFD_OK;
}

template <class T>
int dput(T** p, const T* h, size_t n) {
  int rc = dalloc(p, n);
  if (rc) return rc;
  if (n) CUDA_TRY(cudaMemcpy(*p, h, n * sizeof(T), cudaMemcpyHostToDevice));
  return PCFD_OK;
}

void free_learned(Learned* lp);

void free_solver(Solver* s) {
  if (!s) return;
  free_learned(s->lp);
  void* ptrs[] = {s->d_en, s->d_ea, s->d_eh, s->d_bn, s->d_ba, s->d_bbc, s->d_btw, s->d_bfactag, s->d_bnrm, s->d_xyz,
                  s->d_vol, s->d_nptr, s->d_nedg, s->d_nnbr, s->d_lsq, s->d_bptr, s->d_bhe, s->d_bgnode,
                  s->d_bgptr, s->d_bghe, s->d_bgslot, s->d_bgqr, s->d_q, s->d_grad, s->d_lim, s->d_b, s->d_qold, s->d_qpre, s->d_ef, s->d_bf, s->d_part,
                  s->d_norms, s->d_health, s->d_clipflag, s->d_clipany, s->d_bind, s->d_limraw,
                  s->d_ia, s->d_ja, s->d_pos_lr, s->d_pos_rl, s->d_M, s->d_diag, s->d_dlu, s->d_dinv, s->d_piv,
                  s->d_bblk, s->d_dt, s->d_x, s->d_xf, s->d_diagf, s->d_dinvf, s->d_wd, s->d_dotsf, s->d_mdot_done, s->d_scal, s->d_color_rows, s->d_cptr, s->d_rowdesc, s->d_mv, s->d_gbar, s->d_sgs_err, s->d_V, s->d_Z, s->d_w, s->d_dots,
                  s->f_q, s->f_grad, s->f_lim, s->f_limraw, s->f_eh, s->f_lsq, s->f_ef, s->f_bf, s->f_ea, s->f_ba,
                  s->d_ext, s->f_ext};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  if (s->ev0) cudaEventDestroy(s->ev0);
  if (s->ev1) cudaEventDestroy(s->ev1);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
}

// Most-normal neighbour of a no-slip wall node (ucs/bc.tcc:1184-1207); a
// mesh constant, found once here instead of on every call.
int normal_node(const pcfd_mesh_view* m, int node, const double* avec) {
  int normalNode = -1;
  double dotmax = 0.0;
  const double* wx = &m->xyz[3 * node];
  for (int k = m->ipsp[node]; k < m->ipsp[node + 1]; k++) {
    int pt = m->psp[k];
    const double* px = &m->xyz[3 * pt];
    double dx[3] = {px[0] - wx[0], px[1] - wx[1], px[2] - wx[2]};
    double mg = std::sqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2]);
    dx[0] = dx[0] / mg; dx[1] = dx[1] / mg; dx[2] = dx[2] / mg;
    double dot = 0.0;
    for (int i = 0; i < 3; i++) dot -= dx[i] * avec[i];
    if (dot >= dotmax) { normalNode = pt; dotmax = dot; }
  }
  return normalNode;
}

BcConst make_bc_const(const Solver* s) {
  BcConst k;
  k.gamma = s->prm.gamma;
  k.no_cvbc = s->prm.no_cvbc;
  for (int j = 0; j < NVARS; j++) k.qinf[j] = s->qinf[j];
  return k;
}

FluxConst make_flux_const(const Solver* s) {
  FluxConst k;
  k.gamma = s->prm.gamma;
  k.chi = s->prm.chi;
  k.ho = s->prm.sorder > 1;
  k.viscous = s->prm.viscous;
  k.clip = k.ho && s->prm.limiter != 0;
  k.inv_retilde = s->prm.Re != 0.0 ? s->prm.mach / s->prm.Re : 0.0;
  k.S = 110.4 / s->prm.ref_temperature;
  k.cp_over_pr = (1.0 / (s->prm.gamma - 1.0)) / s->prm.Pr;
  const double g = k.gamma;
  const double vals[10] = {g, g - 1.0, 1.0 / g, 1.0 / (g - 1.0), k.chi, 0.5 * k.chi, 1.0 - k.chi,
                           k.inv_retilde, k.S, k.cp_over_pr};
  double* dd = &k.kd.gamma;
  dfl* ff = &k.kf.gamma;
  for (int i = 0; i < 10; i++) {
    dd[i] = vals[i];
    float hi = (float)vals[i];
    ff[i].hi = hi;
    ff[i].lo = (float)(vals[i] - (double)hi);
  }
  return k;
}

// Param::dt as the temporal residual reads it: <= 0 is steady, 0 stands for
// the reference's default -1.0
double param_time_step(const pcfd_params& p) { return p.time_step == 0.0 ? -1.0 : p.time_step; }

// SolutionField::EvolveInTime for the state (ucs/solutionField.tcc:203): the
// conservative state of the interior nodes becomes the step's q_old
__global__ void k_save_qold(int nnode, const double* __restrict__ q, double* __restrict__ qold) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nnode; i += gridDim.x * blockDim.x)
#pragma unroll
    for (int t = 0; t < NEQN; t++) qold[(size_t)i * NEQN + t] = q[(size_t)i * NVARS + t];
}

int save_qold(Solver* s) {
  return launch(s, T_SETUP, [&] {
    k_save_qold<<<nblk(s->nnode, 256), 256, 0, s->stream>>>(s->nnode, s->d_q, s->d_qold);
  });
}

void host_qinf(const pcfd_params& p, double* Q) {
  // UpdateQinf (ucs/compressible.tcc:827-864): rho = gamma p / T with the
  // non-dimensional freestream T and p (1 up to the rounding of the
  // reference's scaling)
  double gamma = p.gamma, gm1 = gamma - 1.0;
  const double T = p.tinf == 0.0 ? 1.0 : p.tinf;
  const double pr = p.pinf == 0.0 ? 1.0 : p.pinf;
  double rho = pr * gamma / T;
  double u = p.flowdir[0] * p.mach, v = p.flowdir[1] * p.mach, w = p.flowdir[2] * p.mach;
  double E = pr / gm1 + 0.5 * rho * (u * u + v * v + w * w);
  Q[0] = rho; Q[1] = rho * u; Q[2] = rho * v; Q[3] = rho * w; Q[4] = E;
  double ir = 1.0 / Q[0];
  double uu = Q[1] * ir, vv = Q[2] * ir, ww = Q[3] * ir;
  double P = gm1 * (Q[4] - 0.5 * Q[0] * (uu * uu + vv * vv + ww * ww));
  Q[6] = P; Q[5] = gamma * P * ir; Q[7] = uu; Q[8] = vv; Q[9] = ww;
}

int run_bcs(Solver* s, int arith = 0) {
  // a valid double-float copy of q is updated with the rows the conditions
  // write (the sequential walk invalidates it instead)
  dfl* fq = (s->f_q_valid && !s->bc_sequential) ? s->f_q : nullptr;
  if (!fq) s->f_q_valid = 0;
  BcConst k = make_bc_const(s);
  if (s->bc_sequential) {
    return launch(s, T_BC, [&] {
      k_bc_sequential<<<1, 1, 0, s->stream>>>(s->nbedge, s->d_bn, s->d_ba, s->d_bbc, s->d_btw, s->d_bnrm, k, s->d_q,
                                              s->d_health);
    });
  }
  int rc = PCFD_OK;
  if (s->nbind > 0) {
    rc = launch(s, T_BC, [&] {
      if (arith)
        k_bc_halfedges_df<<<nblk(s->nbind, 128), 128, 0, s->stream>>>(s->nbind, s->d_bind, s->d_bn, s->d_ba,
                                                                      s->d_bbc, k, s->d_q, fq, s->d_health);
      else
        k_bc_halfedges<<<nblk(s->nbind, 128), 128, 0, s->stream>>>(s->nbind, s->d_bind, s->d_bn, s->d_ba, s->d_bbc,
                                                                   s->d_btw, k, s->d_q, fq, s->d_health);
    });
    if (rc) return rc;
  }
  if (s->nbgroup == 0) return PCFD_OK;
  rc = launch(s, T_BC, [&] {
    if (arith)
      k_bc_group_halfedges<true><<<nblk(s->nbgslot, 128), 128, 0, s->stream>>>(
          s->nbgslot, s->d_bgslot, s->d_bgnode, s->d_bgptr, s->d_bghe, s->d_bn, s->d_ba, s->d_bbc, s->d_btw,
          s->d_bnrm, k, s->d_q, s->d_bgqr, s->d_health);
    else
      k_bc_group_halfedges<false><<<nblk(s->nbgslot, 128), 128, 0, s->stream>>>(
          s->nbgslot, s->d_bgslot, s->d_bgnode, s->d_bgptr, s->d_bghe, s->d_bn, s->d_ba, s->d_bbc, s->d_btw,
          s->d_bnrm, k, s->d_q, s->d_bgqr, s->d_health);
  });
  if (rc) return rc;
  return launch(s, T_BC, [&] {
    k_bc_group_nodes<<<nblk(s->nbgroup, 128), 128, 0, s->stream>>>(s->nbgroup, s->d_bgnode, s->d_bgptr, s->d_bghe,
                                                                   s->d_bn, s->d_bbc, s->d_btw, s->d_bnrm, k,
                                                                   s->d_bgqr, s->d_q, fq);
  });
}


// The residual-path buffers in the working scalar type: the FP64 arrays,
// or their double-float copies (allocated on first use).
template <class S>
struct RBuf {
  S *q, *grad, *lim, *limraw, *eh, *lsq, *ef, *bf;
  typename V4<S>::type *ea, *ba;
};
RBuf<double> rbuf_d(Solver* s) {
  return {s->d_q, s->d_grad, s->d_lim, s->d_limraw, s->d_eh, s->d_lsq, s->d_ef, s->d_bf, s->d_ea, s->d_ba};
}
RBuf<dfl> rbuf_f(Solver* s) {
  return {s->f_q, s->f_grad, s->f_lim, s->f_limraw, s->f_eh, s->f_lsq, s->f_ef, s->f_bf, s->f_ea, s->f_ba};
}

int to_df_launch(Solver* s, const double* in, dfl* out, long long n) {
  return launch(s, T_SETUP, [&] { k_to_df<<<kNormBlocks, 256, 0, s->stream>>>(n, in, out); });
}

// double-float copies of the static geometry and buffers for the state
int ensure_df(Solver* s) {
  if (s->f_q) return PCFD_OK;
  int rc;
  const long long nn = s->nnode, ne = s->nedge, nb = s->nbedge;
  if ((rc = dalloc(&s->f_q, (size_t)s->ntot * NVARS))) return rc;
  if ((rc = dalloc(&s->f_grad, (size_t)nn * NTERMS * 3))) return rc;
  if ((rc = dalloc(&s->f_lim, (size_t)nn * NEQN))) return rc;
  if ((rc = dalloc(&s->f_limraw, (size_t)nn * NEQN))) return rc;
  if ((rc = dalloc(&s->f_eh, (size_t)ne * 3))) return rc;
  if ((rc = dalloc(&s->f_lsq, (size_t)ne * 6))) return rc;
  if ((rc = dalloc(&s->f_ef, (size_t)ne * NEQN))) return rc;
  if ((rc = dalloc(&s->f_bf, (size_t)std::max<long long>(nb, 1) * NEQN))) return rc;
  if ((rc = dalloc(&s->f_ea, (size_t)ne))) return rc;
  if ((rc = dalloc(&s->f_ba, (size_t)std::max<long long>(nb, 1)))) return rc;
  if ((rc = to_df_launch(s, s->d_eh, s->f_eh, ne * 3))) return rc;
  if ((rc = to_df_launch(s, s->d_lsq, s->f_lsq, ne * 6))) return rc;
  if ((rc = to_df_launch(s, (const double*)s->d_ea, (dfl*)s->f_ea, ne * 4))) return rc;
  if (nb > 0 && (rc = to_df_launch(s, (const double*)s->d_ba, (dfl*)s->f_ba, nb * 4))) return rc;
  return PCFD_OK;
}

// the state in the working scalar type (converted once per change of q)
int prep_state(Solver* s, int arith) {
  if (arith == 0) return PCFD_OK;
  int rc = ensure_df(s);
  if (rc) return rc;
  if (s->f_q_valid) return PCFD_OK;
  rc = to_df_launch(s, s->d_q, s->f_q, (long long)s->ntot * NVARS);
  if (rc == PCFD_OK) s->f_q_valid = 1;
  return rc;
}

template <class S>
int run_gradient_t(Solver* s, RBuf<S> r) {
  return launch(s, T_GRAD, [&] {
    k_gradient<S><<<nblk(s->nnode, 128), 128, 0, s->stream>>>(s->nnode, s->d_nptr, s->d_nnbr, r.lsq, r.q, s->d_bptr,
                                                             s->d_bhe, s->d_bbc, r.ba, r.grad);
  });
}

int run_gradient(Solver* s, int arith = 0) {
  int rc = prep_state(s, arith);
  if (rc) return rc;
  s->ext_ready = 0;  // formed from the previous gradient
  rc = arith ? run_gradient_t(s, rbuf_f(s)) : run_gradient_t(s, rbuf_d(s));
  if (rc == PCFD_OK) {
    s->have_grad = 1;
    s->grad_arith = arith;
  }
  return rc;
}

template <class S>
S*& ext_buf(Solver* s);
template <>
double*& ext_buf<double>(Solver* s) { return s->d_ext; }
template <>
dfl*& ext_buf<dfl>(Solver* s) { return s->f_ext; }

template <class S>
int run_venkat_t(Solver* s, RBuf<S> r, bool clip) {
  double K = s->prm.venkat_K;
  const bool c0 = s->prm.chi == 0.0;
  auto kern = s->prm.limiter == 1 ? (c0 ? k_venkat<S, 1, true> : k_venkat<S, 1, false>)
              : s->prm.limiter == 2 ? (c0 ? k_venkat<S, 2, true> : k_venkat<S, 2, false>)
                                    : (c0 ? k_venkat<S, 3, true> : k_venkat<S, 3, false>);
  // the MUSCL corrections of every edge end, for the residual's edge pass
  // (chi = 0, and not for the explicit-clip form)
  S* ext = nullptr;
  if (c0 && !clip) {
    S*& buf = ext_buf<S>(s);
    if (!buf) {
      int rc = dalloc(&buf, (size_t)s->nedge * 2 * NEQN);
      if (rc) return rc;
    }
    ext = buf;
  }
  return launch(s, T_LIMITER, [&] {
    kern<<<nblk(s->nnode, 128), 128, 0, s->stream>>>(s->nnode, s->d_nptr, s->d_nedg, s->d_nnbr, r.q, r.grad, r.eh,
                                                     s->d_vol, s->prm.chi, K * K * K, r.limraw,
                                                     clip ? nullptr : r.lim, s->d_clipflag, ext);
  });
}

// Limiter<T>::Compute.  clip = true runs the explicit pressure-clip kernel
// (FP64 only); clip = false folds the clip into the residual's edge pass.
int run_limiter(Solver* s, bool clip, int arith = 0) {
  if (clip) arith = 0;
  if (s->prm.limiter == 0) {
    // limiters stay 1.0 (OFF), Limiter ctor (ucs/limiters.tcc:36-41)
    std::vector<double> ones((size_t)s->nnode * NEQN, 1.0);
    CUDA_TRY(cudaMemcpyAsync(s->d_lim, ones.data(), ones.size() * sizeof(double), cudaMemcpyHostToDevice, s->stream));
    if (arith) {
      int rc = ensure_df(s);
      if (rc) return rc;
      rc = to_df_launch(s, s->d_lim, s->f_lim, (long long)s->nnode * NEQN);
      if (rc) return rc;
    }
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    s->have_lim = 1;
    s->lim_arith = arith;
    s->lim_clipped = 0;
    return PCFD_OK;
  }
  if (!s->have_grad || s->grad_arith != arith) return set_err(PCFD_ERR_STATE, "limiter: gradient not computed");
  s->ext_ready = 0;
  int rc = arith ? run_venkat_t(s, rbuf_f(s), clip) : run_venkat_t(s, rbuf_d(s), clip);
  if (rc) return rc;
  if (!clip) {
    // the clip is folded into the residual's edge pass (k_edge_flux<S, 1>)
    s->have_lim = 1;
    s->lim_arith = arith;
    s->lim_clipped = 0;
    s->lim_fresh = 1;
    s->ext_ready = s->prm.chi == 0.0;
    s->ext_arith = arith;
    return PCFD_OK;
  }
  rc = launch(s, T_LIMITER, [&] {
    k_pressure_clip<<<nblk(s->nnode, 128), 128, 0, s->stream>>>(s->nnode, s->d_nptr, s->d_nnbr, s->d_q, s->d_grad,
                                                               s->d_xyz, s->prm.chi, s->prm.gamma, s->d_limraw,
                                                               s->d_lim, s->d_health);
  });
  if (rc == PCFD_OK) {
    s->have_lim = 1;
    s->lim_arith = 0;
    s->lim_clipped = 1;
  }
  return rc;
}

template <class S>
int run_residual_t(Solver* s, RBuf<S> r, FluxConst k, const S* ext) {
  const bool c0 = s->prm.chi == 0.0;
  // with the limiter pass's stored corrections (ext) the edge pass reads
  // them instead of gathering both ends' gradients
  auto flux1 = ext  ? k_edge_flux<S, 1, true, true>
               : c0 ? k_edge_flux<S, 1, true, false>
                    : k_edge_flux<S, 1, false, false>;
  auto flux2 = ext  ? k_edge_flux<S, 2, true, true>
               : c0 ? k_edge_flux<S, 2, true, false>
                    : k_edge_flux<S, 2, false, false>;
  int rc = launch(s, T_EDGEFLUX, [&] {
    flux1<<<nblk(s->nedge, 128), 128, 0, s->stream>>>(s->nedge, s->d_en, r.ea, r.eh, r.q, r.grad, r.lim, k, r.ef,
                                                      s->d_health, s->d_clipflag, s->d_clipany, r.limraw, ext);
  });
  if (rc) return rc;
  if (k.clip) {
    rc = launch(s, T_CLIP, [&] {
      k_clip_apply<S><<<kNormBlocks, 256, 0, s->stream>>>(s->nnode, s->d_clipflag, s->d_clipany, r.lim, s->d_health);
    });
    if (rc) return rc;
    rc = launch(s, T_CLIP, [&] {
      flux2<<<nblk(s->nedge, 128), 128, 0, s->stream>>>(s->nedge, s->d_en, r.ea, r.eh, r.q, r.grad, r.lim, k, r.ef,
                                                        s->d_health, s->d_clipflag, s->d_clipany, r.limraw, ext);
    });
    if (rc) return rc;
  }
  if (k.viscous) {
    rc = launch(s, T_EDGEVISC, [&] {
      k_edge_visc<S><<<nblk(s->nedge, 128), 128, 0, s->stream>>>(s->nedge, s->d_en, r.ea, r.eh, r.q, r.grad, k, r.ef);
    });
    if (rc) return rc;
  }
  if (s->nbedge > 0) {
    rc = launch(s, T_BEDGEFLUX, [&] {
      k_bedge_flux<S><<<nblk(s->nbedge, 128), 128, 0, s->stream>>>(s->nbedge, s->d_bn, r.ba, r.q, r.grad, k, r.bf,
                                                                  s->d_health);
    });
    if (rc) return rc;
  }
  rc = launch(s, T_GATHER, [&] {
    k_gather<S><<<kNormBlocks, kNormThreads, 0, s->stream>>>(s->nnode, s->d_nptr, s->d_nedg, r.ef, s->d_bptr, s->d_bhe,
                                                            r.bf, s->d_bbc, s->d_btw, s->d_b, s->d_part, s->d_clipflag,
                                                            s->d_clipany, s->d_q, s->prm.torder ? s->d_qold : nullptr,
                                                            s->d_vol, param_time_step(s->prm));
  });
  if (rc) return rc;
  return launch(s, T_NORM, [&] {
    k_norm_final<<<1, 192, 0, s->stream>>>(kNormBlocks, s->nnode, s->d_part, s->d_norms, s->d_clipany);
  });
}

int run_residual(Solver* s, int arith = 0, bool first_order = false) {
  FluxConst k = make_flux_const(s);
  if (first_order) k.ho = 0;
  k.clip = k.ho && s->prm.limiter != 0 && s->lim_fresh;
  if ((k.ho || k.viscous) && (!s->have_grad || s->grad_arith != arith))
    return set_err(PCFD_ERR_STATE, "residual: gradient not computed");
  if (k.ho && (!s->have_lim || s->lim_arith != arith)) return set_err(PCFD_ERR_STATE, "residual: limiter not computed");
  if (s->lim_clipped) k.clip = 0;  // the explicit clip already ran
  int rc = prep_state(s, arith);
  if (rc) return rc;
  const bool ext = k.ho && s->ext_ready && s->ext_arith == arith;
  rc = arith ? run_residual_t(s, rbuf_f(s), k, ext ? s->f_ext : nullptr)
             : run_residual_t(s, rbuf_d(s), k, ext ? s->d_ext : nullptr);
  s->lim_fresh = 0;  // the pressure clip belongs to the limiter evaluation it follows
  s->ext_ready = 0;
  return rc;
}


// ---- implicit system runners ---------------------------------------------

size_t prec_bytes(int prec) { return prec == 0 ? 8 : (prec == 1 ? 4 : 2); }

int ensure_matrix(Solver* s, int prec) {
  if (prec < 0 || prec > 2) return set_err(PCFD_ERR_ARG, "Jacobian precision must be 0 (FP64), 1 (FP32) or 2 (BF16)");
  if (s->d_M && s->jac_prec == prec) return PCFD_OK;
  if (s->d_M) { cudaFree(s->d_M); s->d_M = nullptr; }
  if (!s->d_xf) {
    int rc = dalloc(&s->d_xf, (size_t)s->nnode * NEQN);
    if (!rc) rc = dalloc(&s->d_diagf, (size_t)s->nnode * 25);
    if (!rc) rc = dalloc(&s->d_dinvf, (size_t)s->nnode * 25 + 4);  // tail padding for staged windows
    if (rc) return rc;
  }
  // 16 bytes of tail padding for the aligned windows of the staged row kernels
  size_t bytes = (size_t)s->nblocks * 25 * prec_bytes(prec) + 16;
  cudaError_t e = cudaMalloc(&s->d_M, bytes);
  if (e != cudaSuccess) return set_err(PCFD_ERR_NOMEM, std::string("matrix: ") + cudaGetErrorString(e));
  CUDA_TRY(cudaMemsetAsync(s->d_M, 0, bytes, s->stream));
  s->jac_prec = prec;
  s->have_jac = 0;
  return PCFD_OK;
}

// Param::UpdateCFL (ucs/param.tcc:696), prescribed ramp
double ramp_cfl(int iter, double cfl_start, double cfl, int ramp_steps) {
  if (ramp_steps > 0 && iter < ramp_steps) return (cfl - cfl_start) / (double)ramp_steps * (double)iter + cfl_start;
  return cfl;
}

// local time steps in the residual's arithmetic (the pseudo-time step does
// not enter the converged answer)
int run_timestep(Solver* s, double cfl) {
  int rc = prep_state(s, s->arith);
  if (rc) return rc;
  rc = launch(s, T_TIMESTEP, [&] {
    if (s->arith) {
      RBuf<dfl> r = rbuf_f(s);
      k_timestep<dfl><<<nblk(s->nnode, 128), 128, 0, s->stream>>>(s->nnode, s->d_nptr, s->d_nedg, s->d_nnbr, r.ea,
                                                                 s->d_bptr, s->d_bhe, s->d_bn, r.ba, r.q, s->d_vol,
                                                                 s->prm.gamma, cfl, s->d_dt);
    } else {
      k_timestep<double><<<nblk(s->nnode, 128), 128, 0, s->stream>>>(s->nnode, s->d_nptr, s->d_nedg, s->d_nnbr,
                                                                    s->d_ea, s->d_bptr, s->d_bhe, s->d_bn, s->d_ba,
                                                                    s->d_q, s->d_vol, s->prm.gamma, cfl, s->d_dt);
    }
  });
  if (rc) return rc;
  rc = launch(s, T_TIMESTEP, [&] { k_min_part<<<kNormBlocks, kNormThreads, 0, s->stream>>>(s->nnode, s->d_dt, s->d_part); });
  if (rc) return rc;
  rc = launch(s, T_TIMESTEP, [&] { k_min_final<<<1, 32, 0, s->stream>>>(kNormBlocks, s->d_part, s->d_scal + 0); });
  if (rc == PCFD_OK) s->have_dt = 1;
  return rc;
}

JacConst make_jac_const(const Solver* s) {
  JacConst k;
  k.gamma = s->prm.gamma;
  k.Pr = s->prm.Pr;
  k.inv_retilde = s->prm.Re != 0.0 ? s->prm.mach / s->prm.Re : 0.0;
  k.S = 110.4 / s->prm.ref_temperature;
  k.viscous = s->prm.viscous;
  return k;
}

template <class T>
int run_jacobian_t(Solver* s) {
  T* M = (T*)s->d_M;
  JacConst jk = make_jac_const(s);
  BcConst bk = make_bc_const(s);
  // inviscid differences on the state before the conditions, viscous blocks
  // on the state after them (ComputeSpatialJacobian's order).  The flux
  // differences run in double-float when the residual does, and whenever
  // the matrix is stored in FP32 or BF16: their ~48-bit significand carries
  // the difference quotient (step 1e-8) to about 3e-7, the order of FP32
  // storage's own rounding, at the FP32 pipes' rate.
  const bool dfj = s->arith || !std::is_same<T, double>::value;
  int rc = launch(s, T_JAC_EDGE, [&] {
    if (dfj)
      k_jac_edge_df<T><<<nblk(s->nedge, 128), 128, 0, s->stream>>>(s->nedge, s->d_en, s->d_ea, s->d_eh, s->d_qpre,
                                                                  s->d_q, s->d_pos_lr, s->d_pos_rl, jk, M,
                                                                  s->d_health);
    else
      k_jac_edge<T><<<nblk(s->nedge, 128), 128, 0, s->stream>>>(s->nedge, s->d_en, s->d_ea, s->d_eh, s->d_qpre,
                                                               s->d_q, s->d_pos_lr, s->d_pos_rl, jk, M, s->d_health);
  });
  if (rc) return rc;
  if (s->nbedge > 0) {
    const BedgeSlots sl{s->nbind, s->d_bind, s->d_bgslot, s->d_bgnode, s->d_bgptr, s->d_bghe};
    const int nth = s->nbind + s->nbgslot;
    rc = launch(s, T_JAC_BEDGE, [&] {
      if (s->bc_sequential)
        k_jac_bedge_sequential<<<1, 1, 0, s->stream>>>(s->nbedge, s->d_bn, s->d_ba, s->d_bbc, s->d_btw, s->d_bnrm, bk,
                                                       s->prm.jac_boundary_eval, s->d_qpre, s->d_bblk, s->d_health);
      else if (dfj)
        k_jac_bedge_df<<<nblk(nth, 128), 128, 0, s->stream>>>(nth, sl, s->d_bn, s->d_ba, s->d_bbc, s->d_btw,
                                                             s->d_bnrm, bk, s->prm.jac_boundary_eval, s->d_qpre,
                                                             s->d_bblk, s->d_health);
      else
        k_jac_bedge<<<nblk(nth, 128), 128, 0, s->stream>>>(nth, sl, s->d_bn, s->d_ba, s->d_bbc, s->d_btw, s->d_bnrm,
                                                          bk, s->prm.jac_boundary_eval, s->d_qpre, s->d_bblk,
                                                          s->d_health);
    });
    if (rc) return rc;
  }
  rc = launch(s, T_JAC_DIAG, [&] {
    k_jac_diag<T><<<nblk(s->nnode, 128), 128, 0, s->stream>>>(s->nnode, s->d_nptr, s->d_nedg, s->d_pos_lr,
                                                             s->d_pos_rl, s->d_bptr, s->d_bhe, s->d_bblk, M,
                                                             s->d_vol, s->d_dt, s->d_diag);
  });
  if (rc) return rc;
  rc = launch(s, T_JAC_FINISH, [&] {
    k_jac_finish<T><<<nblk(s->nnode, 128), 128, 0, s->stream>>>(s->nnode, s->d_ia, s->d_ja, s->d_bptr, s->d_bhe,
                                                               s->d_bbc, s->d_btw, s->d_bnrm, s->prm.gamma, M,
                                                               s->d_diag, s->d_dlu, s->d_piv, s->d_health);
  });
  if (rc) return rc;
  rc = launch(s, T_JAC_FINISH, [&] {
    k_diag_inverse<<<nblk(s->nnode, 128), 128, 0, s->stream>>>(s->nnode, s->d_dlu, s->d_piv, s->d_dinv);
  });
  if (rc == PCFD_OK && !std::is_same<T, double>::value)
    rc = launch(s, T_JAC_FINISH, [&] {
      k_diag_f32<<<kNormBlocks, 256, 0, s->stream>>>((long long)s->nnode * 25, s->d_diag, s->d_dinv, s->d_diagf,
                                                     s->d_dinvf);
    });
  if (rc == PCFD_OK) s->have_jac = 1;
  return rc;
}

// ComputeJacobians (ucs/jacobian.tcc:13) including the boundary-condition
// application its boundary kernel performs on the stored state.
int run_jacobian(Solver* s) {
  if (!s->have_dt) return set_err(PCFD_ERR_STATE, "jacobian: no time step computed yet (pcfd_timestep)");
  if (!s->d_M) {
    int rc = ensure_matrix(s, 0);
    if (rc) return rc;
  }
  // ComputeSpatialJacobian (ucs/jacobian.tcc:130) reads the state before the
  // boundary conditions for its inviscid differences, and its boundary pass
  // applies the conditions to the stored state (what UpdateBCs does) before
  // the viscous blocks: keep a copy of the state before, then update it
  if (!s->d_qpre) {
    int rc = dalloc(&s->d_qpre, (size_t)s->ntot * NVARS);
    if (rc) return rc;
  }
  CUDA_TRY(cudaMemcpyAsync(s->d_qpre, s->d_q, (size_t)s->ntot * NVARS * sizeof(double), cudaMemcpyDeviceToDevice,
                           s->stream));
  int rc = run_bcs(s, s->arith);
  if (rc) return rc;
  // the gradient no longer matches the state; the limiter field keeps its
  // values, as the reference's does between evaluations
  s->have_grad = 0;
  switch (s->jac_prec) {
    case 0: return run_jacobian_t<double>(s);
    case 1: return run_jacobian_t<float>(s);
    default: return run_jacobian_t<__nv_bfloat16>(s);
  }
}

int run_sumsq(Solver* s, const double* v, long long n, double* out_dev) {
  int rc = launch(s, T_KRYLOV, [&] { k_sumsq<<<kNormBlocks, kNormThreads, 0, s->stream>>>(n, v, s->d_part); });
  if (rc) return rc;
  return launch(s, T_KRYLOV, [&] { k_sum_final<<<1, 32, 0, s->stream>>>(kNormBlocks, s->d_part, out_dev); });
}

// nsweeps of multicolour block symmetric Gauss-Seidel on A x = b from the
// current x (CRS::SGS, ucs/crs.tcc:62).  The reference sweeps rows in index
// order; here rows of one colour (no two adjacent) update together and the
// colours are swept forward then backward, the GPU form of the same
// smoother.  Returns |norm(x_last) - norm(x_previous)| as the reference does.
// nsweeps symmetric block-SGS sweeps (CRS::SGS, ucs/crs.tcc:62) as one
// cooperative launch of k_sgs_sweep: as many blocks as can be resident (at
// most three per multiprocessor), none beyond what the largest colour needs.
template <class T, class K>
int run_sweeps(Solver* s, int nsweeps, const K* dinv, const K* b, K* x, typename OffAcc<T>::type* xa) {
  if (nsweeps <= 0) return PCFD_OK;
  auto kern = k_sgs_sweep<T, K>;
  int per_sm = 0;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, 0));
  if (per_sm < 1) return set_err(PCFD_ERR_CUDA, "sgs: sweep kernel cannot be resident");
  int maxrows = 1;
  for (int c = 0; c < s->ncolor; c++) maxrows = std::max(maxrows, s->color_ptr[c + 1] - s->color_ptr[c]);
  int grid = std::max(1, std::min(std::min(per_sm, 3) * s->nsm, nblk(maxrows, 8)));
  const T* M = (const T*)s->d_M;
  int ncolor = s->ncolor;
  void* args[] = {&ncolor, &s->d_cptr, &s->d_rowdesc, &s->d_ja, &M,         &dinv,         &b,
                  &x,      &xa,        &nsweeps,       &s->d_gbar, &s->d_sgs_err};
  cudaError_t ce = cudaSuccess;
  int rc = launch(s, T_SGS, [&] { ce = cudaLaunchCooperativeKernel((void*)kern, grid, 256, args, 0, s->stream); });
  if (rc) return rc;
  if (ce != cudaSuccess) return set_err(PCFD_ERR_CUDA, std::string("sgs sweep launch: ") + cudaGetErrorString(ce));
  return PCFD_OK;
}

// a timed-out grid barrier in an earlier sweep (read at the call's
// synchronisation point)
int check_sweeps(Solver* s) {
  int e = 0;
  CUDA_TRY(cudaMemcpy(&e, s->d_sgs_err, sizeof(int), cudaMemcpyDeviceToHost));
  if (e) {
    CUDA_TRY(cudaMemset(s->d_sgs_err, 0, sizeof(int)));
    CUDA_TRY(cudaMemset(s->d_gbar, 0, 2 * sizeof(unsigned int)));
    return set_err(PCFD_ERR_CUDA, "sgs: a sweep's grid barrier timed out");
  }
  return PCFD_OK;
}

template <class E>
int run_sweeps_staged(Solver* s, int nsweeps, const E* dinv, const E* b, E* x);

template <class T>
int run_sgs_t(Solver* s, int nsweeps, const double* b, double* x, double* dnorm) {
  const double cnt = (double)s->nnode * NEQN;
  double prev = 0.0, cur = 0.0;
  typedef typename OffAcc<T>::type A;
  A* xa = (A*)x;
  if (!std::is_same<T, double>::value) {
    int rc = launch(s, T_SGS, [&] {
      k_to_f32<<<kNormBlocks, 256, 0, s->stream>>>((long long)s->nnode * NEQN, x, s->d_xf);
    });
    if (rc) return rc;
    xa = (A*)s->d_xf;
  }
  auto norm = [&](double& out) -> int {
    int rc = run_sumsq(s, x, (long long)s->nnode * NEQN, s->d_scal + 2);
    if (rc) return rc;
    double v;
    CUDA_TRY(cudaMemcpyAsync(&v, s->d_scal + 2, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    out = std::sqrt(v) / cnt;
    return PCFD_OK;
  };
  // FP64 blocks and vectors run the staged kernel, mixed types the
  // register-staged one
  auto sweeps = [&](int k) -> int {
    if (std::is_same<T, double>::value) return run_sweeps_staged<double>(s, k, s->d_dinv, b, x);
    return run_sweeps<T, double>(s, k, s->d_dinv, b, x, xa);
  };
  int rc;
  if (dnorm && nsweeps >= 2) {
    // the reference returns the norm change of the last sweep
    if ((rc = sweeps(nsweeps - 1))) return rc;
    if ((rc = norm(prev))) return rc;
    if ((rc = sweeps(1))) return rc;
    if ((rc = norm(cur))) return rc;
  } else {
    if ((rc = sweeps(nsweeps))) return rc;
    if (dnorm && nsweeps == 1 && (rc = norm(cur))) return rc;
  }
  if (dnorm) *dnorm = std::fabs(prev - cur);
  return PCFD_OK;
}

int run_sgs(Solver* s, int nsweeps, const double* b, double* x, double* dnorm) {
  if (!s->have_jac) return set_err(PCFD_ERR_STATE, "sgs: no Jacobian assembled");
  switch (s->jac_prec) {
    case 0: return run_sgs_t<double>(s, nsweeps, b, x, dnorm);
    case 1: return run_sgs_t<float>(s, nsweeps, b, x, dnorm);
    default: return run_sgs_t<__nv_bfloat16>(s, nsweeps, b, x, dnorm);
  }
}

// nsweeps of the same sweep on FP32 vectors (the FP32 Krylov solver's
// preconditioner; FP32 or BF16 matrix storage)
template <class T>
int run_sgs_f_t(Solver* s, int nsweeps, const float* b, float* x) {
  return run_sweeps<T, float>(s, nsweeps, s->d_dinvf, b, x, x);
}

// nsweeps sweeps through the staged kernel (cooperative; as many blocks as
// fit, at most four per multiprocessor), blocks and vectors of type E
template <class E>
int run_sweeps_staged(Solver* s, int nsweeps, const E* dinv, const E* b, E* x) {
  if (nsweeps <= 0) return PCFD_OK;
  auto kern = k_sgs_sweep_staged<E>;
  constexpr int smem = 8 * kRowStages * (int)sizeof(RowStage<E>);
  static bool attr = false;
  if (!attr) {
    CUDA_TRY(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    attr = true;
  }
  int per_sm = 0;
  CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, 256, smem));
  if (per_sm < 1) return set_err(PCFD_ERR_CUDA, "sgs: staged sweep kernel cannot be resident");
  int maxrows = 1;
  for (int c = 0; c < s->ncolor; c++) maxrows = std::max(maxrows, s->color_ptr[c + 1] - s->color_ptr[c]);
  int grid = std::max(1, std::min(std::min(per_sm, 4) * s->nsm, nblk(maxrows, 8)));
  const E* M = (const E*)s->d_M;
  int ncolor = s->ncolor;
  void* args[] = {&ncolor, &s->d_cptr, &s->d_rowdesc, &s->d_ja, &M, &dinv, &b, &x, &nsweeps, &s->d_gbar, &s->d_sgs_err};
  cudaError_t ce = cudaSuccess;
  int rc = launch(s, T_SGS, [&] { ce = cudaLaunchCooperativeKernel((void*)kern, grid, 256, args, smem, s->stream); });
  if (rc) return rc;
  if (ce != cudaSuccess) return set_err(PCFD_ERR_CUDA, std::string("sgs sweep launch: ") + cudaGetErrorString(ce));
  return PCFD_OK;
}

// FP32 blocks and vectors: the staged kernel
template <>
int run_sgs_f_t<float>(Solver* s, int nsweeps, const float* b, float* x) {
  return run_sweeps_staged<float>(s, nsweeps, s->d_dinvf, b, x);
}

int run_sgs_f(Solver* s, int nsweeps, const float* b, float* x) {
  if (!s->have_jac) return set_err(PCFD_ERR_STATE, "sgs: no Jacobian assembled");
  if (s->jac_prec == 1) return run_sgs_f_t<float>(s, nsweeps, b, x);
  if (s->jac_prec == 2) return run_sgs_f_t<__nv_bfloat16>(s, nsweeps, b, x);
  return set_err(PCFD_ERR_STATE, "FP32 sweep needs FP32 or BF16 matrix storage");
}

int run_apply_dq(Solver* s, double* dqnorm) {
  // a valid double-float copy of q is updated row by row
  dfl* fq = s->f_q_valid ? s->f_q : nullptr;
  int rc = launch(s, T_UPDATE, [&] {
    k_apply_dq<<<kNormBlocks, kNormThreads, 0, s->stream>>>(s->nnode, s->prm.gamma, s->d_x, s->d_q, fq, s->d_part,
                                                           s->d_health);
  });
  if (rc) return rc;
  rc = launch(s, T_UPDATE, [&] { k_sum_final<<<1, 32, 0, s->stream>>>(kNormBlocks, s->d_part, s->d_scal + 3); });
  if (rc) return rc;
  s->have_grad = 0;
  if (dqnorm) {
    double v;
    CUDA_TRY(cudaMemcpyAsync(&v, s->d_scal + 3, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    *dqnorm = std::sqrt(v) / ((double)s->nnode * NEQN);
  }
  return PCFD_OK;
}


// ---- FGMRES -----------------------------------------------------------------

template <class T>
int run_spmv_t(Solver* s, const double* x, double* y) {
  typedef typename OffAcc<T>::type A;
  const A* xa = (const A*)x;
  if (!std::is_same<T, double>::value) {
    int rc = launch(s, T_SPMV, [&] {
      k_to_f32<<<kNormBlocks, 256, 0, s->stream>>>((long long)s->nnode * NEQN, x, s->d_xf);
    });
    if (rc) return rc;
    xa = (const A*)s->d_xf;
  }
  return launch(s, T_SPMV, [&] {
    k_spmv<T, double><<<row_grid(s->nnode), 256, 0, s->stream>>>(s->nnode, s->d_ia, s->d_ja, (const T*)s->d_M,
                                                                s->d_diag, x, xa, y);
  });
}

template <class T>
int run_spmv_f_t(Solver* s, const float* x, float* y) {
  return launch(s, T_SPMV, [&] {
    k_spmv<T, float><<<row_grid(s->nnode), 256, 0, s->stream>>>(s->nnode, s->d_ia, s->d_ja, (const T*)s->d_M,
                                                               s->d_diagf, x, x, y);
  });
}

// FP32 blocks: the staged pipeline (k_spmv_staged), four blocks per
// multiprocessor
template <>
int run_spmv_f_t<float>(Solver* s, const float* x, float* y) {
  constexpr int smem = 8 * kRowStages * (int)sizeof(RowStage<float>);
  static bool attr = false;
  if (!attr) {
    CUDA_TRY(cudaFuncSetAttribute(k_spmv_staged, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    attr = true;
  }
  const int grid = std::max(1, std::min(nblk(s->nnode, 8), 4 * s->nsm));
  return launch(s, T_SPMV, [&] {
    k_spmv_staged<<<grid, 256, smem, s->stream>>>(s->nnode, s->d_ia, s->d_ja, (const float*)s->d_M, s->d_diagf, x, y);
  });
}

int run_spmv_f(Solver* s, const float* x, float* y) {
  if (s->jac_prec == 1) return run_spmv_f_t<float>(s, x, y);
  return run_spmv_f_t<__nv_bfloat16>(s, x, y);
}

int run_spmv(Solver* s, const double* x, double* y) {
  switch (s->jac_prec) {
    case 0: return run_spmv_t<double>(s, x, y);
    case 1: return run_spmv_t<float>(s, x, y);
    default: return run_spmv_t<__nv_bfloat16>(s, x, y);
  }
}

int ensure_krylov(Solver* s, int m) {
  if (s->fg_m >= m && s->d_V) return PCFD_OK;
  if (s->d_V) cudaFree(s->d_V);
  if (s->d_Z) cudaFree(s->d_Z);
  if (s->d_w) cudaFree(s->d_w);
  if (s->d_dots) cudaFree(s->d_dots);
  s->d_V = s->d_Z = s->d_w = s->d_dots = nullptr;
  const size_t n = (size_t)s->nnode * NEQN;
  int rc;
  // (with tail padding for the staged row kernels' aligned windows)
  if ((rc = dalloc(&s->d_V, n * (m + 1) + 4))) return rc;
  if ((rc = dalloc(&s->d_Z, n * m + 4))) return rc;
  if ((rc = dalloc(&s->d_w, n))) return rc;
  // partials [kKrylovBlocks][m+2], then four result slots of m+2 each
  if ((rc = dalloc(&s->d_dots, (size_t)kKrylovBlocks * (m + 2) + 4 * (m + 2)))) return rc;
  if (s->d_dotsf) cudaFree(s->d_dotsf);
  s->d_dotsf = nullptr;
  if ((rc = dalloc(&s->d_dotsf, 4 * (size_t)(m + 2)))) return rc;
  if (!s->d_wd && (rc = dalloc(&s->d_wd, n))) return rc;
  if (!s->d_mdot_done) {
    if ((rc = dalloc(&s->d_mdot_done, 1))) return rc;
    CUDA_TRY(cudaMemsetAsync(s->d_mdot_done, 0, sizeof(unsigned int), s->stream));
  }
  s->fg_m = m;
  return PCFD_OK;
}

// result slot `slot` (0..3) of the Krylov dot buffer, m+2 doubles
double* krylov_slot(Solver* s, int slot) {
  return s->d_dots + (size_t)kKrylovBlocks * (s->fg_m + 2) + (size_t)slot * (s->fg_m + 2);
}

float* krylov_slot_f(Solver* s, int slot) { return s->d_dotsf + (size_t)slot * (s->fg_m + 2); }
template <class K>
K* krylov_coef(Solver* s, int slot);
template <>
double* krylov_coef<double>(Solver* s, int slot) { return krylov_slot(s, slot); }
template <>
float* krylov_coef<float>(Solver* s, int slot) { return krylov_slot_f(s, slot); }

// dots[k] = (w, V_k), k < nv, into result slot `slot` on the device (FP64,
// with an FP32 copy)
template <class K>
int run_mdot_dev(Solver* s, const K* V, int nv, const K* w, int slot) {
  const long long n = (long long)s->nnode * NEQN;
  double* part = s->d_dots;
  double* res = krylov_slot(s, slot);
  float* resf = krylov_slot_f(s, slot);
  return launch(s, T_KRYLOV, [&] {
    k_mdot<K><<<kKrylovBlocks, kNormThreads, 0, s->stream>>>(n, nv, V, w, part, s->d_mdot_done, res, resf);
  });
}

// One wave of a Gram-Schmidt kernel: its resident blocks per multiprocessor
// times the multiprocessors (they hold the element's vectors in registers,
// so fewer blocks fit than the fixed Krylov grid); each kernel reduces its
// own partials, so the grid only has to be fixed per device.
template <class F>
int orth_grid(Solver* s, int slot, F kernel) {
  if (!s->orth_grid[slot]) {
    int per_sm = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kNormThreads, 0);
    s->orth_grid[slot] = std::max(1, std::min(kKrylovBlocks, std::max(1, per_sm) * s->nsm));
  }
  return s->orth_grid[slot];
}

// The Gram-Schmidt kernels hold up to NV vectors in registers; each call
// takes the smallest of 4, 8, 16, 32 that holds nv (larger nv: 32, where
// k_orth_norm falls back to its sequential loop).
template <class K, template <class, int> class KER, class F4, class F8, class F16, class F32>
int orth_launch(Solver* s, int base, int nv, F4 f4, F8 f8, F16 f16, F32 f32) {
  const int t = std::is_same<K, double>::value ? 4 : 0;
  if (nv <= 4) return f4(orth_grid(s, base + t + 0, KER<K, 4>::fn()));
  if (nv <= 8) return f8(orth_grid(s, base + t + 1, KER<K, 8>::fn()));
  if (nv <= 16) return f16(orth_grid(s, base + t + 2, KER<K, 16>::fn()));
  return f32(orth_grid(s, base + t + 3, KER<K, 32>::fn()));
}
template <class K, int NV>
struct OrthNormK {
  static auto fn() { return k_orth_norm<K, NV>; }
};
template <class K, int NV>
struct OrthMdotK {
  static auto fn() { return k_orth_mdot<K, NV>; }
};

// w -= sum_k h[k] V_k with (w, w) of the result into result slot 0
template <class K>
int run_orth_norm(Solver* s, const K* V, int nv, const K* h, K* w) {
  const long long n = (long long)s->nnode * NEQN;
  auto go = [&](auto kernel, int grid) {
    return launch(s, T_KRYLOV, [&] {
      kernel<<<grid, kNormThreads, 0, s->stream>>>(n, nv, V, h, w, s->d_dots, s->d_mdot_done, krylov_slot(s, 0));
    });
  };
  return orth_launch<K, OrthNormK>(
      s, 0, nv, [&](int g) { return go(k_orth_norm<K, 4>, g); }, [&](int g) { return go(k_orth_norm<K, 8>, g); },
      [&](int g) { return go(k_orth_norm<K, 16>, g); }, [&](int g) { return go(k_orth_norm<K, 32>, g); });
}

// w -= sum_k h[k] V_k, then its dot products with V_0..V_{nv-1} into result
// slot `slot` (nv <= 32)
template <class K>
int run_orth_mdot(Solver* s, const K* V, int nv, const K* h, K* w, int slot) {
  const long long n = (long long)s->nnode * NEQN;
  auto go = [&](auto kernel, int grid) {
    return launch(s, T_KRYLOV, [&] {
      kernel<<<grid, kNormThreads, 0, s->stream>>>(n, nv, V, h, w, s->d_dots, s->d_mdot_done, krylov_slot(s, slot),
                                                    krylov_slot_f(s, slot));
    });
  };
  return orth_launch<K, OrthMdotK>(
      s, 8, nv, [&](int g) { return go(k_orth_mdot<K, 4>, g); }, [&](int g) { return go(k_orth_mdot<K, 8>, g); },
      [&](int g) { return go(k_orth_mdot<K, 16>, g); }, [&](int g) { return go(k_orth_mdot<K, 32>, g); });
}


// learned preconditioner (defined with the network's host code below)
int lp_precondition(Solver* s, int nsgs, const double* v, double* z);

// Restarted right-preconditioned flexible GMRES (Saad 1993) with classical
// Gram-Schmidt applied twice; the reference's GMRES (ucs/crs.tcc:176) is the
// non-flexible form.  Preconditioner: nsgs block-SGS sweeps, or with use_lp
// the learned correction on top of them; a cycle in which the learned
// preconditioner reduces the residual by less than 10 % switches the rest of
// the solve to plain SGS and adds one cycle (counted in *fallbacks).
int lp_precondition_f(Solver* s, int nsgs, const float* v, float* z);

// preconditioner and product in the Krylov vector type
int krylov_prec(Solver* s, int nsgs, bool use_lp, const double* v, double* z) {
  return use_lp ? lp_precondition(s, nsgs, v, z) : run_sgs(s, nsgs, v, z, nullptr);
}
int krylov_prec(Solver* s, int nsgs, bool use_lp, const float* v, float* z) {
  return use_lp ? lp_precondition_f(s, nsgs, v, z) : run_sgs_f(s, nsgs, v, z);
}
int krylov_spmv(Solver* s, const double* x, double* y) { return run_spmv(s, x, y); }
int krylov_spmv(Solver* s, const float* x, float* y) { return run_spmv_f(s, x, y); }

// r0 = b - A x into the Krylov vector w (x = 0 on the first cycle)
int krylov_residual(Solver* s, bool first, double* w) {
  const long long n = (long long)s->nnode * NEQN;
  if (first) {
    CUDA_TRY(cudaMemcpyAsync(w, s->d_b, n * sizeof(double), cudaMemcpyDeviceToDevice, s->stream));
    return PCFD_OK;
  }
  int rc = run_spmv(s, s->d_x, w);
  if (rc) return rc;
  return launch(s, T_KRYLOV, [&] { k_residual_vec<<<kNormBlocks, 256, 0, s->stream>>>(n, s->d_b, w); });
}
int krylov_residual(Solver* s, bool first, float* w) {
  const long long n = (long long)s->nnode * NEQN;
  if (!first) {
    int rc = run_spmv(s, s->d_x, s->d_wd);
    if (rc) return rc;
  }
  const double* r = first ? nullptr : s->d_wd;
  return launch(s, T_KRYLOV, [&] { k_residual_vec_f32<<<kNormBlocks, 256, 0, s->stream>>>(n, s->d_b, r, w); });
}

// Restarted right-preconditioned flexible GMRES (Saad 1993) with classical
// Gram-Schmidt applied twice; the reference's GMRES (ucs/crs.tcc:176) is the
// non-flexible form.  K is the Krylov vector type: FP64 with the FP64
// matrix, FP32 with FP32 or BF16 storage - the linear solve is then a
// defect correction whose rounding the FP64 residual of each restart and of
// the next Newton step wins back; the update x stays FP64.  Preconditioner:
// nsgs block-SGS sweeps, or with use_lp the learned correction on top of
// them; a cycle in which the learned preconditioner reduces the residual by
// less than 10 % switches the rest of the solve to plain SGS and adds one
// cycle (counted in *fallbacks).
// aug: instead, every cycle's second direction is the learned vector of the
// cycle's first Krylov vector (the residual direction), after plain SGS of
// it as the first: the space then holds both, so the correction cannot make
// a cycle worse per direction, and no fallback is needed.
template <class K>
int run_fgmres_t(Solver* s, const pcfd_newton_opts* o, double* relres, int* iters, bool use_lp, int* fallbacks,
                 bool aug) {
  const int m = std::max(1, std::min(o->fgmres_m > 0 ? o->fgmres_m : 30, 60));
  int restarts = std::max(1, o->fgmres_restarts);
  if (fallbacks) *fallbacks = 0;
  const double rtol = o->fgmres_rtol > 0.0 ? o->fgmres_rtol : 1e-3;
  int rc = ensure_krylov(s, m);
  if (rc) return rc;
  const long long n = (long long)s->nnode * NEQN;
  K* V = (K*)s->d_V;
  K* Z = (K*)s->d_Z;
  K* w = (K*)s->d_w;
  K* hdev = krylov_coef<K>(s, 3);
  std::vector<double> H((size_t)(m + 1) * m, 0.0), cs(m), sn(m), g(m + 1), hcol(m + 2), y(m);
  std::vector<K> yk(m);
  double beta0 = -1.0;
  int total = 0;
  double rel = 1.0;
  const size_t st = s->fg_m + 2;
  std::vector<double> dd(3 * st);
  for (int rs = 0; rs < restarts; rs++) {
    if ((rc = krylov_residual(s, rs == 0, w))) return rc;
    if ((rc = run_mdot_dev<K>(s, w, 1, w, 0))) return rc;
    double bb;
    CUDA_TRY(cudaMemcpyAsync(&bb, krylov_slot(s, 0), sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    double beta = std::sqrt(bb);
    if (beta0 < 0.0) beta0 = beta;
    if (beta == 0.0 || beta0 == 0.0) { rel = 0.0; break; }
    if ((rc = launch(s, T_KRYLOV, [&] { k_scale_copy<K><<<kKrylovBlocks, 256, 0, s->stream>>>(n, K(1.0 / beta), w, V); })))
      return rc;
    std::fill(g.begin(), g.end(), 0.0);
    g[0] = beta;
    int j = 0;
    for (; j < m; j++) {
      K* zj = Z + (size_t)j * n;
      CUDA_TRY(cudaMemsetAsync(zj, 0, n * sizeof(K), s->stream));
      const bool lp_here = use_lp && (aug ? j == 1 : (o->lp_directions <= 0 || j < o->lp_directions));
      const K* vin = (aug && j == 1) ? V : V + (size_t)j * n;
      if ((rc = krylov_prec(s, std::max(1, o->nsgs), lp_here, vin, zj))) return rc;
      if ((rc = krylov_spmv(s, zj, w))) return rc;
      // CGS2 with the coefficients kept on the device (slots 1, 2) and the
      // norm of the result (slot 0, formed by the second update); one host
      // synchronisation per iteration
      if ((rc = run_mdot_dev<K>(s, V, j + 1, w, 1))) return rc;
      if (j + 1 <= 32) {
        if ((rc = run_orth_mdot<K>(s, V, j + 1, krylov_coef<K>(s, 1), w, 2))) return rc;
      } else {
        K* dv = krylov_coef<K>(s, 1);
        if ((rc = launch(s, T_KRYLOV, [&] { k_orth_update<K><<<kKrylovBlocks, 256, 0, s->stream>>>(n, j + 1, V, dv, w); })))
          return rc;
        if ((rc = run_mdot_dev<K>(s, V, j + 1, w, 2))) return rc;
      }
      if ((rc = run_orth_norm<K>(s, V, j + 1, krylov_coef<K>(s, 2), w))) return rc;
      CUDA_TRY(cudaMemcpyAsync(dd.data(), krylov_slot(s, 0), dd.size() * sizeof(double), cudaMemcpyDeviceToHost,
                               s->stream));
      CUDA_TRY(cudaStreamSynchronize(s->stream));
      for (int k = 0; k <= j + 1; k++) hcol[k] = 0.0;
      for (int k = 0; k <= j; k++) hcol[k] = dd[st + k] + dd[2 * st + k];
      double hn = std::sqrt(dd[0]);
      hcol[j + 1] = hn;
      if (hn > 0.0) {
        K* vn = V + (size_t)(j + 1) * n;
        if ((rc = launch(s, T_KRYLOV, [&] { k_scale_copy<K><<<kKrylovBlocks, 256, 0, s->stream>>>(n, K(1.0 / hn), w, vn); })))
          return rc;
      }
      // apply previous rotations, then a new one
      for (int k = 0; k < j; k++) {
        double t = cs[k] * hcol[k] + sn[k] * hcol[k + 1];
        hcol[k + 1] = -sn[k] * hcol[k] + cs[k] * hcol[k + 1];
        hcol[k] = t;
      }
      double den = std::sqrt(hcol[j] * hcol[j] + hcol[j + 1] * hcol[j + 1]);
      cs[j] = den > 0.0 ? hcol[j] / den : 1.0;
      sn[j] = den > 0.0 ? hcol[j + 1] / den : 0.0;
      hcol[j] = den;
      hcol[j + 1] = 0.0;
      g[j + 1] = -sn[j] * g[j];
      g[j] = cs[j] * g[j];
      for (int k = 0; k <= j; k++) H[(size_t)k * m + j] = hcol[k];
      total++;
      rel = std::fabs(g[j + 1]) / beta0;
      if (rel < rtol || hn == 0.0) { j++; break; }
    }
    // back substitution and x += Z y
    for (int k = j - 1; k >= 0; k--) {
      double t = g[k];
      for (int q = k + 1; q < j; q++) t -= H[(size_t)k * m + q] * y[q];
      y[k] = t / H[(size_t)k * m + k];
    }
    for (int k = 0; k < j; k++) yk[k] = (K)y[k];
    CUDA_TRY(cudaMemcpyAsync(hdev, yk.data(), j * sizeof(K), cudaMemcpyHostToDevice, s->stream));
    if ((rc = launch(s, T_KRYLOV, [&] { k_combine<K><<<kKrylovBlocks, 256, 0, s->stream>>>(n, j, Z, hdev, s->d_x); })))
      return rc;
    if (rel < rtol) break;
    if (use_lp && !aug && rel > 0.9 * beta / beta0) {
      use_lp = false;
      restarts++;
      if (fallbacks) (*fallbacks)++;
    }
  }
  // the host copy of y must outlive the asynchronous copy above
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  if (relres) *relres = rel;
  if (iters) *iters = total;
  return PCFD_OK;
}

int run_fgmres(Solver* s, const pcfd_newton_opts* o, double* relres, int* iters, bool use_lp = false,
               int* fallbacks = nullptr, bool aug = false) {
  if (s->jac_prec == 0) return run_fgmres_t<double>(s, o, relres, iters, use_lp, fallbacks, aug);
  return run_fgmres_t<float>(s, o, relres, iters, use_lp, fallbacks, aug);
}

// -------------------------------------------------------------------------
// learned right preconditioner (kernels in learned.cuh)
// -------------------------------------------------------------------------

struct Learned {
  int n = 0;
  long long nnz = 0;
  float4* ef = nullptr;           // [nnz] oriented edge features
  float* invdeg = nullptr;        // [n]
  float* w = nullptr;             // [NPARAM] FP32 master parameters
  float* g = nullptr;             // [NPARAM + 1] gradient, then the loss sum
  float *m1 = nullptr, *m2 = nullptr;  // Adam moments
  int adam_t = 0;
  __nv_bfloat16 *img_fwd = nullptr, *img_bwd = nullptr;  // [NL][LP_IMG]
  float* x = nullptr;             // [n][NIN]
  __nv_bfloat16* h = nullptr;     // [NL+1][n][H]
  __nv_bfloat16* m = nullptr;     // [NL][n][H]
  float *out = nullptr, *t = nullptr;        // [n][NOUT]
  float *dh = nullptr, *dhs = nullptr, *dm = nullptr;  // [n][H]
  __nv_bfloat16* dz = nullptr;    // [n][H]
  float* part = nullptr;          // per-block gradient partials
  size_t part_len = 0;
  double *y = nullptr, *sigma = nullptr, *vbuf = nullptr;  // [n][5], [1], [n][5]
  int* err = nullptr;
  int grid_red = 0;               // blocks of the grid-stride backward kernels
  int npb = 0;                    // nodes per block of the weight-gradient kernels
  std::vector<float*> sx, st;     // stored training pairs
};

void free_learned(Learned* lp) {
  if (!lp) return;
  void* ptrs[] = {lp->ef, lp->invdeg, lp->w, lp->g, lp->m1, lp->m2, lp->img_fwd, lp->img_bwd, lp->x, lp->h, lp->m,
                  lp->out, lp->t, lp->dh, lp->dhs, lp->dm, lp->dz, lp->part, lp->y, lp->sigma, lp->vbuf, lp->err};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (float* p : lp->sx) cudaFree(p);
  for (float* p : lp->st) cudaFree(p);
  delete lp;
}

// seeded initial parameters: Kaiming-uniform matrices, unit gates, zero
// decoder (the preconditioner starts as its SGS base)
void lp_initial_params(unsigned long long seed, std::vector<float>& w) {
  w.assign(LP_NPARAM, 0.f);
  unsigned long long st = seed;
  auto uni = [&](double a) {
    st += 0x9E3779B97F4A7C15ull;
    unsigned long long z = st;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (float)(a * (2.0 * ((double)(z >> 11) * (1.0 / 9007199254740992.0)) - 1.0));
  };
  for (int i = 0; i < LP_H * LP_NIN; i++) w[LP_OFF_WIN + i] = uni(std::sqrt(6.0 / LP_NIN));
  for (int l = 0; l < LP_NL; l++) {
    float* wl = &w[LP_OFF_L0 + l * LP_L_SIZE];
    for (int i = 0; i < LP_H * LP_NE; i++) wl[LP_L_WE + i] = uni(0.1);
    for (int i = 0; i < LP_H; i++) wl[LP_L_CE + i] = 1.f;
    for (int i = 0; i < LP_H * LP_H; i++) wl[LP_L_WS + i] = uni(std::sqrt(6.0 / (2 * LP_H)));
    for (int i = 0; i < LP_H * LP_H; i++) wl[LP_L_WM + i] = uni(std::sqrt(6.0 / (2 * LP_H)));
  }
}

int lp_pack(Solver* s) {
  Learned* lp = s->lp;
  return launch(s, T_LP_BWD, [&] {
    k_lp_pack<<<nblk(LP_NL * LP_IMG, 256), 256, 0, s->stream>>>(lp->w, lp->img_fwd, lp->img_bwd);
  });
}

int lp_check_err(Solver* s) {
  int e = 0;
  CUDA_TRY(cudaMemcpyAsync(&e, s->lp->err, sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  if (e) {
    CUDA_TRY(cudaMemsetAsync(s->lp->err, 0, sizeof(int), s->stream));
    return set_err(PCFD_ERR_NUMERIC, "learned preconditioner: tensor-core wait expired");
  }
  return PCFD_OK;
}

// Forward pass from the features in lp->x.  train: store h, m and out for
// the backward pass; otherwise write z = y + sigma * out.
int lp_forward(Solver* s, bool train, double* z) {
  Learned* lp = s->lp;
  const int n = lp->n;
  const size_t nh = (size_t)n * LP_H;
  int rc = launch(s, T_LP_FWD, [&] {
    k_lp_encode<<<nblk((long long)n * (LP_H / 2), 256), 256, 0, s->stream>>>(n, lp->x, lp->w, lp->h);
  });
  if (rc) return rc;
  const int tiles = nblk(n, LP_TILE);
  for (int l = 0; l < LP_NL; l++) {
    const float* wl = lp->w + LP_OFF_L0 + l * LP_L_SIZE;
    const __nv_bfloat16* hin = lp->h + (train ? l : (l & 1)) * nh;
    __nv_bfloat16* hout = lp->h + (train ? l + 1 : ((l + 1) & 1)) * nh;
    __nv_bfloat16* mout = train ? lp->m + l * nh : nullptr;
    const __nv_bfloat16* img = lp->img_fwd + (size_t)l * LP_IMG;
    rc = launch(s, T_LP_FWD, [&] {
      if (l < LP_NL - 1)
        k_lp_layer<false><<<tiles, LP_THREADS, LP_SMEM, s->stream>>>(
            n, s->d_nptr, s->d_nnbr, lp->ef, lp->invdeg, hin, wl, img, hout, mout, lp->w, nullptr, nullptr, nullptr,
            nullptr, lp->err);
      else
        k_lp_layer<true><<<tiles, LP_THREADS, LP_SMEM, s->stream>>>(
            n, s->d_nptr, s->d_nnbr, lp->ef, lp->invdeg, hin, wl, img, train ? hout : nullptr, mout, lp->w,
            train ? lp->out : nullptr, lp->y, lp->sigma, train ? nullptr : z, lp->err);
    });
    if (rc) return rc;
  }
  return PCFD_OK;
}

// gradient of the loss against lp->t into lp->g (after lp_forward(train))
int lp_backward(Solver* s) {
  Learned* lp = s->lp;
  const int n = lp->n;
  const size_t nh = (size_t)n * LP_H;
  const int tiles = nblk(n, LP_TILE);
  const int gr = lp->grid_red;
  const int nwb = nblk(n, lp->npb);
  auto reduce = [&](int nb, int len, float* dst) {
    return launch(s, T_LP_BWD, [&] { k_lp_reduce<<<nblk(len, 256), 256, 0, s->stream>>>(nb, len, lp->part, dst); });
  };
  int rc = launch(s, T_LP_BWD, [&] {
    k_lp_dec_bwd<<<gr, 256, 0, s->stream>>>(n, lp->out, lp->t, lp->h + LP_NL * nh, lp->w, lp->dh, lp->part);
  });
  if (rc || (rc = reduce(gr, LP_DEC_LEN, lp->g + LP_OFF_WOUT))) return rc;
  for (int l = LP_NL - 1; l >= 0; l--) {
    const float* wl = lp->w + LP_OFF_L0 + l * LP_L_SIZE;
    float* gl = lp->g + LP_OFF_L0 + l * LP_L_SIZE;
    rc = launch(s, T_LP_BWD, [&] {
      k_lp_layer_bwd<<<tiles, LP_THREADS, LP_SMEM, s->stream>>>(n, lp->dh, lp->h + (l + 1) * nh,
                                                               lp->img_bwd + (size_t)l * LP_IMG, lp->dz, lp->dhs,
                                                               lp->dm, lp->err);
    });
    if (rc) return rc;
    rc = launch(s, T_LP_BWD, [&] {
      k_lp_wgrad<<<nwb, 256, 0, s->stream>>>(n, lp->npb, lp->dz, lp->h + l * nh, lp->m + l * nh, lp->part);
    });
    if (rc || (rc = reduce(nwb, LP_WG_LEN, gl + LP_L_WS))) return rc;
    rc = launch(s, T_LP_BWD, [&] {
      k_lp_gather_bwd<<<gr, 256, 0, s->stream>>>(n, s->d_nptr, s->d_nnbr, lp->ef, lp->invdeg, lp->h + l * nh, wl,
                                                lp->dhs, lp->dm, lp->dh, lp->part);
    });
    if (rc || (rc = reduce(gr, LP_GB_LEN, gl + LP_L_WE))) return rc;
  }
  rc = launch(s, T_LP_BWD, [&] {
    k_lp_enc_bwd<<<nwb, 256, 0, s->stream>>>(n, lp->npb, lp->dh, lp->h, lp->x, lp->part);
  });
  if (rc || (rc = reduce(nwb, LP_EB_LEN, lp->g + LP_OFF_WIN))) return rc;
  return PCFD_OK;
}

// sigma of lp->y, then the node features into lp->x
int lp_features(Solver* s) {
  Learned* lp = s->lp;
  int rc = launch(s, T_LP_FWD, [&] {
    k_sumsq<<<kNormBlocks, kNormThreads, 0, s->stream>>>((long long)lp->n * NEQN, lp->y, s->d_part);
  });
  if (rc) return rc;
  rc = launch(s, T_LP_FWD, [&] {
    k_lp_sigma<<<1, 256, 0, s->stream>>>(kNormBlocks, s->d_part, (double)lp->n * NEQN, lp->sigma);
  });
  if (rc) return rc;
  double qinf[NVARS];
  host_qinf(s->prm, qinf);
  const double cinf = std::sqrt(s->prm.gamma * qinf[6] / qinf[0]);
  return launch(s, T_LP_FWD, [&] {
    k_lp_features<<<nblk(lp->n, 256), 256, 0, s->stream>>>(lp->n, lp->y, lp->sigma, s->d_q, s->d_vol, qinf[0],
                                                          qinf[6], cinf, s->lp_vmean, lp->x);
  });
}

// z = y + sigma N(x(y)),  y = nsgs SGS sweeps on v
int lp_precondition(Solver* s, int nsgs, const double* v, double* z) {
  Learned* lp = s->lp;
  if (!lp) return set_err(PCFD_ERR_STATE, "learned preconditioner: pcfd_lp_init not called");
  CUDA_TRY(cudaMemsetAsync(lp->y, 0, (size_t)lp->n * NEQN * sizeof(double), s->stream));
  int rc = run_sgs(s, nsgs, v, lp->y, nullptr);
  if (rc || (rc = lp_features(s))) return rc;
  return lp_forward(s, false, z);
}

// the same on FP32 Krylov vectors: the sweep in the FP32 solver's own
// kernel (into z, which is padded like every Krylov vector), the network on
// an FP64 copy of its result
int lp_precondition_f(Solver* s, int nsgs, const float* v, float* z) {
  Learned* lp = s->lp;
  if (!lp) return set_err(PCFD_ERR_STATE, "learned preconditioner: pcfd_lp_init not called");
  const long long n = (long long)lp->n * NEQN;
  CUDA_TRY(cudaMemsetAsync(z, 0, n * sizeof(float), s->stream));
  int rc = run_sgs_f(s, nsgs, v, z);
  if (rc) return rc;
  rc = launch(s, T_KRYLOV, [&] { k_f32_to_f64<<<kNormBlocks, 256, 0, s->stream>>>(n, z, lp->y); });
  if (rc || (rc = lp_features(s)) || (rc = lp_forward(s, false, s->d_wd))) return rc;
  return launch(s, T_KRYLOV, [&] { k_to_f32<<<kNormBlocks, 256, 0, s->stream>>>(n, s->d_wd, z); });
}

int lp_adam_step(Solver* s, double lr) {
  Learned* lp = s->lp;
  lp->adam_t++;
  const float b1 = 0.9f, b2 = 0.999f;
  const float bc1 = 1.f - std::pow(b1, (float)lp->adam_t), bc2 = 1.f - std::pow(b2, (float)lp->adam_t);
  int rc = launch(s, T_LP_BWD, [&] {
    k_lp_adam<<<nblk(LP_NPARAM, 256), 256, 0, s->stream>>>(LP_NPARAM, lp->w, lp->g, lp->m1, lp->m2, (float)lr,
                                                          b1, b2, 1e-8f, bc1, bc2);
  });
  if (rc) return rc;
  return lp_pack(s);
}

int lp_alloc(Solver* s) {
  Learned* lp = new Learned();
  s->lp = lp;
  const int n = s->nnode;
  lp->n = n;
  lp->nnz = 2LL * s->nedge;
  lp->grid_red = std::min(nblk(n, 8), 4 * 152);
  lp->npb = std::max(256, nblk(n, 1216));
  const int nwb = nblk(n, lp->npb);
  lp->part_len = std::max({(size_t)lp->grid_red * LP_DEC_LEN, (size_t)lp->grid_red * LP_GB_LEN,
                           (size_t)nwb * LP_WG_LEN, (size_t)nwb * LP_EB_LEN});
  const size_t nh = (size_t)n * LP_H;
  int rc;
  if ((rc = dalloc(&lp->ef, std::max<long long>(lp->nnz, 1)))) return rc;
  if ((rc = dalloc(&lp->invdeg, n))) return rc;
  if ((rc = dalloc(&lp->w, LP_NPARAM))) return rc;
  if ((rc = dalloc(&lp->g, LP_NPARAM + 1))) return rc;
  if ((rc = dalloc(&lp->m1, LP_NPARAM))) return rc;
  if ((rc = dalloc(&lp->m2, LP_NPARAM))) return rc;
  if ((rc = dalloc(&lp->img_fwd, (size_t)LP_NL * LP_IMG))) return rc;
  if ((rc = dalloc(&lp->img_bwd, (size_t)LP_NL * LP_IMG))) return rc;
  if ((rc = dalloc(&lp->x, (size_t)n * LP_NIN))) return rc;
  if ((rc = dalloc(&lp->h, (LP_NL + 1) * nh))) return rc;
  if ((rc = dalloc(&lp->m, LP_NL * nh))) return rc;
  if ((rc = dalloc(&lp->out, (size_t)n * LP_NOUT))) return rc;
  if ((rc = dalloc(&lp->t, (size_t)n * LP_NOUT))) return rc;
  if ((rc = dalloc(&lp->dh, nh))) return rc;
  if ((rc = dalloc(&lp->dhs, nh))) return rc;
  if ((rc = dalloc(&lp->dm, nh))) return rc;
  if ((rc = dalloc(&lp->dz, nh))) return rc;
  if ((rc = dalloc(&lp->part, lp->part_len))) return rc;
  if ((rc = dalloc(&lp->y, (size_t)n * NEQN + 4))) return rc;  // tail padding: staged sweep windows
  if ((rc = dalloc(&lp->vbuf, (size_t)n * NEQN + 4))) return rc;
  if ((rc = dalloc(&lp->sigma, 1))) return rc;
  if ((rc = dalloc(&lp->err, 1))) return rc;
  CUDA_TRY(cudaMemsetAsync(lp->err, 0, sizeof(int), s->stream));
  CUDA_TRY(cudaMemsetAsync(lp->h, 0, (LP_NL + 1) * nh * sizeof(__nv_bfloat16), s->stream));
  CUDA_TRY(cudaFuncSetAttribute(k_lp_layer<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LP_SMEM));
  CUDA_TRY(cudaFuncSetAttribute(k_lp_layer<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LP_SMEM));
  // three layer CTAs (3 x 51 KB) share a multiprocessor
  CUDA_TRY(cudaFuncSetAttribute(k_lp_layer<false>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                (int)cudaSharedmemCarveoutMaxShared));
  CUDA_TRY(cudaFuncSetAttribute(k_lp_layer<true>, cudaFuncAttributePreferredSharedMemoryCarveout,
                                (int)cudaSharedmemCarveoutMaxShared));
  CUDA_TRY(cudaFuncSetAttribute(k_lp_layer_bwd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)LP_SMEM));
  return launch(s, T_SETUP, [&] {
    k_lp_graph<<<nblk(n, 256), 256, 0, s->stream>>>(n, s->d_nptr, s->d_nedg, s->d_en, s->d_ea, s->d_xyz,
                                                    s->lp_lmean, lp->ef, lp->invdeg);
  });
}

int lp_set_params(Solver* s, const float* w) {
  Learned* lp = s->lp;
  CUDA_TRY(cudaMemcpyAsync(lp->w, w, LP_NPARAM * sizeof(float), cudaMemcpyHostToDevice, s->stream));
  CUDA_TRY(cudaMemsetAsync(lp->m1, 0, LP_NPARAM * sizeof(float), s->stream));
  CUDA_TRY(cudaMemsetAsync(lp->m2, 0, LP_NPARAM * sizeof(float), s->stream));
  lp->adam_t = 0;
  int rc = lp_pack(s);
  if (rc) return rc;
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PCFD_OK;
}

}  // namespace

// -------------------------------------------------------------------------
// C ABI
// -------------------------------------------------------------------------

// lets the library's other translation units report through pcfd_last_error
void pcfd_set_last_error(const std::string& msg) { g_err = msg; }

extern "C" {

PCFD_API const char* pcfd_last_error(void) { return g_err.c_str(); }

PCFD_API const char* pcfd_build_info(void) {
  static std::string info;
  if (info.empty()) {
    char buf[256];
    std::snprintf(buf, sizeof(buf), "pcfd sm_103a; CUDA runtime %d; edge-flux + node-gather residual (FP64)",
                  CUDART_VERSION);
    info = buf;
  }
  return info.c_str();
}

PCFD_API int pcfd_create(const pcfd_mesh_view* m, const pcfd_params* prm, pcfd_solver_t* out) {
  if (!m || !prm || !out) return set_err(PCFD_ERR_ARG, "pcfd_create: null argument");
  *out = nullptr;
  if (m->nnode <= 0 || m->nedge <= 0 || m->nbedge < 0 || m->nbnode != m->nbedge)
    return set_err(PCFD_ERR_ARG, "pcfd_create: bad mesh sizes");
  if (!m->edges || !m->edge_area || !m->xyz || !m->vol || !m->sw || !m->ipsp || !m->psp ||
      (m->nbedge > 0 && (!m->bedges || !m->bedge_area || !m->bfactag)))
    return set_err(PCFD_ERR_ARG, "pcfd_create: null mesh array");
  if (prm->gamma <= 1.0 || prm->sorder < 1 || prm->sorder > 2 || prm->ntags <= 0 || !prm->bc_type || !prm->bc_twall)
    return set_err(PCFD_ERR_ARG, "pcfd_create: bad parameters");
  if (prm->jac_boundary_eval < 0 || prm->jac_boundary_eval > 3)
    return set_err(PCFD_ERR_ARG, "pcfd_create: jac_boundary_eval must be 0, 1, 2 or 3");
  if (prm->limiter < 0 || prm->limiter > 3)
    return set_err(PCFD_ERR_UNSUPPORTED, "pcfd_create: limiter must be 0 (off), 1 (Barth), 2 (Venkatakrishnan) or 3 "
                                         "(modified Venkatakrishnan)");
  if (prm->torder < 0 || prm->torder > 1 || prm->time_step > 0.0)
    return set_err(PCFD_ERR_UNSUPPORTED, "pcfd_create: steady runs only (torder 0 or 1, time_step <= 0); the "
                                         "second-order time-accurate residual is not built");
  if (prm->tinf < 0.0 || prm->pinf < 0.0) return set_err(PCFD_ERR_ARG, "pcfd_create: tinf and pinf must be >= 0");
  if (prm->viscous && (prm->Re <= 0.0 || prm->Pr <= 0.0 || prm->ref_temperature <= 0.0))
    return set_err(PCFD_ERR_ARG, "pcfd_create: viscous run needs Re, Pr and ref_temperature > 0");
  const long long nn = m->nnode, ne = m->nedge, nb = m->nbedge;
  // validate integer maps before they reach a kernel
  for (long long e = 0; e < ne; e++) {
    int a = m->edges[2 * e], b = m->edges[2 * e + 1];
    if (a < 0 || a >= nn || b < 0 || b >= nn || a == b) return set_err(PCFD_ERR_ARG, "pcfd_create: edge node out of range");
  }
  for (long long k = 0; k < nb; k++) {
    int a = m->bedges[2 * k], b = m->bedges[2 * k + 1];
    if (a < 0 || a >= nn || b != nn + k) return set_err(PCFD_ERR_ARG, "pcfd_create: half-edge ids out of range");
    int tag = m->bfactag[k];
    if (tag < 0 || tag >= prm->ntags) return set_err(PCFD_ERR_ARG, "pcfd_create: half-edge tag without a BC");
  }
  if (m->ipsp[0] != 0) return set_err(PCFD_ERR_ARG, "pcfd_create: ipsp[0] != 0");
  for (long long i = 0; i < nn; i++)
    if (m->ipsp[i + 1] < m->ipsp[i]) return set_err(PCFD_ERR_ARG, "pcfd_create: ipsp not monotone");
  for (long long k = 0; k < m->ipsp[nn]; k++)
    if (m->psp[k] < 0 || m->psp[k] >= nn) return set_err(PCFD_ERR_ARG, "pcfd_create: psp out of range");

  Solver* s = new Solver();
  s->nnode = m->nnode;
  s->nbnode = m->nbnode;
  s->nedge = m->nedge;
  s->nbedge = m->nbedge;
  s->ntot = m->nnode + m->nbnode;
  s->prm = *prm;
  s->bc_type.assign(prm->bc_type, prm->bc_type + prm->ntags);
  s->bc_twall.assign(prm->bc_twall, prm->bc_twall + prm->ntags);
  s->prm.bc_type = s->bc_type.data();
  s->prm.bc_twall = s->bc_twall.data();
  if (s->prm.venkat_K <= 0.0) s->prm.venkat_K = 1.0;
  host_qinf(s->prm, s->qinf);

  int rc = PCFD_OK;
#define TRY(x)                \
  do {                        \
    rc = (x);                 \
    if (rc) {                 \
      free_solver(s);         \
      return rc;              \
    }                         \
  } while (0)
  cudaError_t ce = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking);
  if (ce != cudaSuccess) { free_solver(s); return set_err(PCFD_ERR_CUDA, std::string("stream: ") + cudaGetErrorString(ce)); }
  cudaEventCreate(&s->ev0);
  cudaEventCreate(&s->ev1);
  {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&s->nsm, cudaDevAttrMultiProcessorCount, dev);
    if (s->nsm <= 0) s->nsm = 1;
  }

  // --- host-side integer preprocessing of the GPU maps ---
  // node -> incident edges, ascending edge id
  std::vector<int> nptr(nn + 1, 0);
  for (long long e = 0; e < ne; e++) {
    nptr[m->edges[2 * e] + 1]++;
    nptr[m->edges[2 * e + 1] + 1]++;
  }
  for (long long i = 0; i < nn; i++) nptr[i + 1] += nptr[i];
  std::vector<int> nedg(2 * ne), nnbr(2 * ne);
  {
    std::vector<int> fill(nptr.begin(), nptr.end() - 1);
    for (long long e = 0; e < ne; e++) {
      int a = m->edges[2 * e], b = m->edges[2 * e + 1];
      nedg[fill[a]] = ~(int)e; nnbr[fill[a]++] = b;
      nedg[fill[b]] = (int)e; nnbr[fill[b]++] = a;
    }
  }
  // node -> boundary half-edges (bedge order) and boundary node groups
  std::vector<int> bptr(nn + 1, 0), bhe(nb);
  for (long long k = 0; k < nb; k++) bptr[m->bedges[2 * k] + 1]++;
  for (long long i = 0; i < nn; i++) bptr[i + 1] += bptr[i];
  {
    std::vector<int> fill(bptr.begin(), bptr.end() - 1);
    for (long long k = 0; k < nb; k++) bhe[fill[m->bedges[2 * k]]++] = (int)k;
  }
  std::vector<int> gnode, gptr(1, 0), bghe_list;
  for (long long i = 0; i < nn; i++)
    if (bptr[i + 1] > bptr[i]) {
      gnode.push_back((int)i);
      gptr.push_back(bptr[i + 1]);
    }
  s->nbgroup = (int)gnode.size();
  // per-half-edge BC data; no-slip normal nodes
  std::vector<int> bbc(nb), bnrm(nb, -1);
  std::vector<double> btw(nb, 0.0);
  std::vector<char> hardset(nn, 0);
  for (long long k = 0; k < nb; k++) {
    int tag = m->bfactag[k];
    bbc[k] = s->bc_type[tag];
    btw[k] = s->bc_twall[tag] / s->prm.ref_temperature;
    if (bbc[k] == PCFD_BC_NOSLIP) bnrm[k] = normal_node(m, m->bedges[2 * k], &m->bedge_area[4 * k]);
    if (bbc[k] == PCFD_BC_NOSLIP || bbc[k] == PCFD_BC_SONIC_INFLOW || bbc[k] == PCFD_BC_DIRICHLET)
      hardset[m->bedges[2 * k]] = 1;
  }
  s->bc_sequential = 0;
  for (long long k = 0; k < nb; k++)
    if (bnrm[k] >= 0 && hardset[bnrm[k]]) s->bc_sequential = 1;
  // nodes no condition hard-sets get one thread per half-edge; the rest keep
  // their half-edges in order on one thread
  std::vector<int> bind;
  {
    std::vector<int> gnode2, gptr2(1, 0), ghe2;
    for (size_t g = 0; g < gnode.size(); g++) {
      int node = gnode[g];
      if (!hardset[node]) {
        for (int p = gptr[g]; p < gptr[g + 1]; p++) bind.push_back(bhe[p]);
      } else {
        gnode2.push_back(node);
        for (int p = gptr[g]; p < gptr[g + 1]; p++) ghe2.push_back(bhe[p]);
        gptr2.push_back((int)ghe2.size());
      }
    }
    gnode.swap(gnode2);
    gptr.swap(gptr2);
    bghe_list.swap(ghe2);
  }
  s->nbgroup = (int)gnode.size();
  s->nbind = (int)bind.size();

  std::vector<int2> en(ne), bn(nb);
  std::vector<D4> ea(ne), ba(nb);
  for (long long e = 0; e < ne; e++) {
    en[e] = make_int2(m->edges[2 * e], m->edges[2 * e + 1]);
    const double* a = &m->edge_area[4 * e];
    ea[e] = D4{a[0], a[1], a[2], a[3]};
  }
  for (long long k = 0; k < nb; k++) {
    bn[k] = make_int2(m->bedges[2 * k], m->bedges[2 * k + 1]);
    const double* a = &m->bedge_area[4 * k];
    ba[k] = D4{a[0], a[1], a[2], a[3]};
  }

  TRY(dput(&s->d_en, en.data(), ne));
  TRY(dput(&s->d_ea, ea.data(), ne));
  TRY(dput(&s->d_bn, bn.data(), nb));
  TRY(dput(&s->d_ba, ba.data(), nb));
  TRY(dput(&s->d_bbc, bbc.data(), nb));
  TRY(dput(&s->d_btw, btw.data(), nb));
  TRY(dput(&s->d_bfactag, m->bfactag, nb));
  TRY(dput(&s->d_bnrm, bnrm.data(), nb));
  TRY(dput(&s->d_xyz, m->xyz, 3 * nn));
  TRY(dput(&s->d_vol, m->vol, nn));
  {
    // mean edge length and mean dual volume, summed in index order (the
    // learned preconditioner's feature scales)
    double ls = 0.0, vs = 0.0;
    for (long long e = 0; e < ne; e++) {
      const double* a = &m->xyz[3 * m->edges[2 * e]];
      const double* b = &m->xyz[3 * m->edges[2 * e + 1]];
      const double dx = b[0] - a[0], dy = b[1] - a[1], dz = b[2] - a[2];
      ls += std::sqrt(dx * dx + dy * dy + dz * dz);
    }
    for (long long i = 0; i < nn; i++) vs += m->vol[i];
    s->lp_lmean = ne > 0 ? ls / ne : 1.0;
    s->lp_vmean = nn > 0 ? vs / nn : 1.0;
  }
  TRY(dput(&s->d_nptr, nptr.data(), nn + 1));
  TRY(dput(&s->d_nedg, nedg.data(), 2 * ne));
  TRY(dput(&s->d_nnbr, nnbr.data(), 2 * ne));
  TRY(dput(&s->d_bptr, bptr.data(), nn + 1));
  TRY(dput(&s->d_bhe, bhe.data(), nb));
  TRY(dput(&s->d_bgnode, gnode.data(), gnode.size()));
  TRY(dput(&s->d_bgptr, gptr.data(), gptr.size()));
  TRY(dput(&s->d_bghe, bghe_list.data(), bghe_list.size()));
  {
    std::vector<int> slot(bghe_list.size());
    for (size_t g = 0; g < gnode.size(); g++)
      for (int p = gptr[g]; p < gptr[g + 1]; p++) slot[p] = (int)g;
    s->nbgslot = (int)slot.size();
    TRY(dput(&s->d_bgslot, slot.data(), slot.size()));
    TRY(dalloc(&s->d_bgqr, std::max<size_t>(slot.size(), 1) * NVARS));
  }
  TRY(dput(&s->d_bind, bind.data(), bind.size()));
  TRY(dalloc(&s->d_clipflag, (size_t)nn));
  TRY(dalloc(&s->d_limraw, (size_t)nn * NEQN));
  TRY(dalloc(&s->d_clipany, 1));
  if (cudaMemsetAsync(s->d_clipflag, 0, sizeof(int) * (size_t)nn, s->stream) != cudaSuccess ||
      cudaMemsetAsync(s->d_clipany, 0, sizeof(int), s->stream) != cudaSuccess) {
    free_solver(s);
    return set_err(PCFD_ERR_CUDA, "memset clip flags");
  }
  TRY(dalloc(&s->d_eh, 3 * ne));
  TRY(dalloc(&s->d_lsq, 3 * 2 * ne));
  TRY(dalloc(&s->d_q, (size_t)s->ntot * NVARS));
  TRY(dalloc(&s->d_grad, (size_t)nn * NTERMS * 3));
  TRY(dalloc(&s->d_lim, (size_t)nn * NEQN));
  TRY(dalloc(&s->d_b, (size_t)nn * NEQN + 4));  // tail padding: staged sweep windows
  TRY(dalloc(&s->d_qold, (size_t)nn * NEQN));
  TRY(dalloc(&s->d_ef, (size_t)ne * NEQN));
  TRY(dalloc(&s->d_bf, (size_t)nb * NEQN));
  TRY(dalloc(&s->d_part, (size_t)kNormBlocks * 6));
  TRY(dalloc(&s->d_norms, 6));
  TRY(dalloc(&s->d_health, 8));
  if (cudaMemsetAsync(s->d_health, 0, 8 * sizeof(unsigned long long), s->stream) != cudaSuccess) {
    free_solver(s);
    return set_err(PCFD_ERR_CUDA, "memset health");
  }
  double* d_sw = nullptr;
  double* d_qinf = nullptr;
  TRY(dput(&d_sw, m->sw, 6 * nn));
  TRY(dput(&d_qinf, s->qinf, NVARS));
  TRY(launch(s, T_SETUP, [&] {
    k_lsq_weights<<<nblk(nn, 128), 128, 0, s->stream>>>(s->nnode, s->d_nptr, s->d_nnbr, s->d_xyz, d_sw, s->d_lsq);
  }));
  TRY(launch(s, T_SETUP, [&] {
    k_edge_half<<<nblk(ne, 256), 256, 0, s->stream>>>(s->nedge, s->d_en, s->d_xyz, s->d_eh);
  }));
  TRY(launch(s, T_SETUP, [&] {
    k_fill_state<<<nblk(s->ntot, 256), 256, 0, s->stream>>>(s->ntot, d_qinf, s->d_q);
  }));
  TRY(save_qold(s));
  ce = cudaStreamSynchronize(s->stream);
  cudaFree(d_sw);
  cudaFree(d_qinf);
  if (ce != cudaSuccess) {
    free_solver(s);
    return set_err(PCFD_ERR_CUDA, std::string("pcfd_create setup: ") + cudaGetErrorString(ce));
  }
  // the limiter starts at 1.0 (OFF), as the Limiter constructor leaves it
  {
    std::vector<double> ones((size_t)nn * NEQN, 1.0);
    if (cudaMemcpy(s->d_lim, ones.data(), ones.size() * sizeof(double), cudaMemcpyHostToDevice) != cudaSuccess) {
      free_solver(s);
      return set_err(PCFD_ERR_CUDA, "limiter init");
    }
  }
  // --- implicit system structure: block CRS exactly as CRSMatrix::Init
  // (ucs/crsmatrix.tcc:48), the block of each edge located once here instead
  // of by GetPointer's row search on every access (:740), and a greedy
  // colouring of the node graph for the Gauss-Seidel sweeps
  {
    std::vector<int> ia(nn + 1), ja;
    ia[0] = 0;
    for (long long i = 0; i < nn; i++) ia[i + 1] = ia[i] + (m->ipsp[i + 1] - m->ipsp[i]) + 1;
    s->nblocks = ia[nn];
    ja.resize(s->nblocks);
    for (long long i = 0; i < nn; i++) {
      int c = ia[i];
      ja[c++] = (int)i;
      for (int k = m->ipsp[i]; k < m->ipsp[i + 1]; k++) ja[c++] = m->psp[k];
    }
    std::vector<int> pos_lr(ne), pos_rl(ne);
    auto find = [&](int row, int col) {
      for (int b = ia[row] + 1; b < ia[row + 1]; b++)
        if (ja[b] == col) return b;
      return -1;
    };
    for (long long e = 0; e < ne; e++) {
      int a = m->edges[2 * e], b = m->edges[2 * e + 1];
      pos_lr[e] = find(a, b);
      pos_rl[e] = find(b, a);
      if (pos_lr[e] < 0 || pos_rl[e] < 0) {
        free_solver(s);
        return set_err(PCFD_ERR_ARG, "pcfd_create: edge missing from psp (maps inconsistent)");
      }
    }
    // colouring: smallest colour not used by an already coloured neighbour
    std::vector<int> color(nn, -1);
    int ncol = 0;
    std::vector<int> mark(64, -1);
    for (long long i = 0; i < nn; i++) {
      for (int k = m->ipsp[i]; k < m->ipsp[i + 1]; k++) {
        int c = color[m->psp[k]];
        if (c >= 0) {
          if (c >= (int)mark.size()) mark.resize(c + 1, -1);
          mark[c] = (int)i;
        }
      }
      int c = 0;
      while (c < (int)mark.size() && mark[c] == (int)i) c++;
      if (c >= (int)mark.size()) mark.resize(c + 1, -1);
      color[i] = c;
      ncol = std::max(ncol, c + 1);
    }
    s->ncolor = ncol;
    s->color_ptr.assign(ncol + 1, 0);
    for (long long i = 0; i < nn; i++) s->color_ptr[color[i] + 1]++;
    for (int c = 0; c < ncol; c++) s->color_ptr[c + 1] += s->color_ptr[c];
    std::vector<int> rows(nn), fill(s->color_ptr.begin(), s->color_ptr.end() - 1);
    for (long long i = 0; i < nn; i++) rows[fill[color[i]]++] = (int)i;
    TRY(dput(&s->d_ia, ia.data(), ia.size()));
    TRY(dput(&s->d_ja, ja.data(), ja.size()));
    TRY(dput(&s->d_pos_lr, pos_lr.data(), pos_lr.size()));
    TRY(dput(&s->d_pos_rl, pos_rl.data(), pos_rl.size()));
    TRY(dput(&s->d_color_rows, rows.data(), rows.size()));
    TRY(dput(&s->d_cptr, s->color_ptr.data(), s->color_ptr.size()));
    {
      std::vector<int4> desc(nn);
      for (long long g = 0; g < nn; g++) {
        const int i = rows[g];
        desc[g] = make_int4(i, ia[i] + 1, ia[i + 1] - ia[i] - 1, 0);
      }
      TRY(dput(&s->d_rowdesc, desc.data(), desc.size()));
    }
    TRY(dalloc(&s->d_gbar, 2));
    TRY(dalloc(&s->d_sgs_err, 1));
    CUDA_TRY(cudaMemset(s->d_gbar, 0, 2 * sizeof(unsigned int)));
    CUDA_TRY(cudaMemset(s->d_sgs_err, 0, sizeof(int)));
    TRY(dalloc(&s->d_diag, (size_t)nn * 25));
    TRY(dalloc(&s->d_dlu, (size_t)nn * 25));
    TRY(dalloc(&s->d_dinv, (size_t)nn * 25 + 4));
    TRY(dalloc(&s->d_piv, (size_t)nn * 5));
    TRY(dalloc(&s->d_bblk, (size_t)std::max<long long>(nb, 1) * 25));
    TRY(dalloc(&s->d_dt, (size_t)nn));
    TRY(dalloc(&s->d_x, (size_t)nn * NEQN + 4));
    TRY(dalloc(&s->d_scal, 16));
  }
#undef TRY
  *out = (pcfd_solver_t)s;
  return PCFD_OK;
}

PCFD_API int pcfd_destroy(pcfd_solver_t h) {
  if (!h) return set_err(PCFD_ERR_ARG, "pcfd_destroy: null handle");
  Solver* s = (Solver*)h;
  cudaStreamSynchronize(s->stream);
  free_solver(s);
  return PCFD_OK;
}

PCFD_API int pcfd_set_state(pcfd_solver_t h, const double* q, int nvars, int nrows) {
  Solver* s = (Solver*)h;
  if (!s || !q || nvars != NVARS || nrows != s->ntot) return set_err(PCFD_ERR_ARG, "pcfd_set_state: bad arguments");
  CUDA_TRY(cudaMemcpyAsync(s->d_q, q, (size_t)nrows * NVARS * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  int rc = save_qold(s);
  if (rc) return rc;
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  s->have_grad = s->have_lim = 0;
  s->f_q_valid = 0;
  return PCFD_OK;
}

PCFD_API int pcfd_set_qold(pcfd_solver_t h, const double* q, int nvars, int nrows) {
  Solver* s = (Solver*)h;
  if (!s || !q || (nvars != NVARS && nvars != NEQN) || nrows < s->nnode)
    return set_err(PCFD_ERR_ARG, "pcfd_set_qold: bad arguments");
  CUDA_TRY(cudaMemcpy2DAsync(s->d_qold, NEQN * sizeof(double), q, (size_t)nvars * sizeof(double),
                             NEQN * sizeof(double), (size_t)s->nnode, cudaMemcpyHostToDevice, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PCFD_OK;
}

PCFD_API int pcfd_get_state(pcfd_solver_t h, double* q, int nvars, int nrows) {
  Solver* s = (Solver*)h;
  if (!s || !q || nvars != NVARS || nrows != s->ntot) return set_err(PCFD_ERR_ARG, "pcfd_get_state: bad arguments");
  CUDA_TRY(cudaMemcpyAsync(q, s->d_q, (size_t)nrows * NVARS * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PCFD_OK;
}

PCFD_API int pcfd_get_qinf(pcfd_solver_t h, double* qinf10) {
  Solver* s = (Solver*)h;
  if (!s || !qinf10) return set_err(PCFD_ERR_ARG, "pcfd_get_qinf: bad arguments");
  std::memcpy(qinf10, s->qinf, sizeof(s->qinf));
  return PCFD_OK;
}

PCFD_API int pcfd_update_bcs(pcfd_solver_t h) {
  Solver* s = (Solver*)h;
  if (!s) return set_err(PCFD_ERR_ARG, "pcfd_update_bcs: null handle");
  int rc = run_bcs(s);
  if (rc) return rc;
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  s->have_grad = s->have_lim = 0;
  return PCFD_OK;
}

PCFD_API int pcfd_gradient(pcfd_solver_t h, double* qgrad_out) {
  Solver* s = (Solver*)h;
  if (!s) return set_err(PCFD_ERR_ARG, "pcfd_gradient: null handle");
  int rc = run_gradient(s);
  if (rc) return rc;
  if (qgrad_out)
    CUDA_TRY(cudaMemcpyAsync(qgrad_out, s->d_grad, (size_t)s->nnode * NTERMS * 3 * sizeof(double),
                             cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PCFD_OK;
}

// FORCE_Kernel (ucs/forces.tcc:124-197) over the boundary half-edges: a
// half-edge whose tag belongs to the body adds p |a| n to the pressure force
// and, on a no-slip wall of a viscous run, the wall stress times |a| to the
// viscous force.  The stress is ComputeStressVector's
// (ucs/compressible.tcc:1113), which reads gradient entries 3..11 (those of
// the momentum components); Sutherland's law as in the viscous flux.
// Per-block sums in a fixed order, then one warp per component.
__global__ void __launch_bounds__(kNormThreads) k_forces(int nbedge, const int2* __restrict__ bn,
                                                         const D4* __restrict__ ba, const int* __restrict__ bfactag,
                                                         const int* __restrict__ bbc, const int* __restrict__ in_body,
                                                         const double* __restrict__ q, const double* __restrict__ grad,
                                                         int viscous, double Sconst, double inv_retilde,
                                                         double* __restrict__ part) {
  __shared__ double red[kNormThreads / 32][6];
  double acc[6] = {0, 0, 0, 0, 0, 0};
  for (int he = blockIdx.x * blockDim.x + threadIdx.x; he < nbedge; he += gridDim.x * blockDim.x) {
    if (!in_body[bfactag[he]]) continue;
    const int a = bn[he].x;
    const D4 av = ba[he];
    const double* Q = &q[(size_t)a * NVARS];
    const double p = Q[6];
    acc[0] += p * av.x * av.w;
    acc[1] += p * av.y * av.w;
    acc[2] += p * av.z * av.w;
    if (viscous && bbc[he] == PCFD_BC_NOSLIP) {
      const double T = Q[5];
      const double mu = sutherland(T, Sconst);
      const double* g = &grad[(size_t)a * NTERMS * 3];
      const double ux = g[3], uy = g[4], uz = g[5], vx = g[6], vy = g[7], vz = g[8], wx = g[9], wy = g[10],
                   wz = g[11];
      const double div = -2.0 / 3.0 * (ux + vy + wz);
      const double txx = 2.0 * ux + div, tyy = 2.0 * vy + div, tzz = 2.0 * wz + div;
      const double txy = uy + vx, txz = uz + wx, tyz = vz + wy;
      const double c = -(mu * inv_retilde) * av.w;
      acc[3] += c * (txx * av.x + txy * av.y + txz * av.z);
      acc[4] += c * (txy * av.x + tyy * av.y + tyz * av.z);
      acc[5] += c * (txz * av.x + tyz * av.y + tzz * av.z);
    }
  }
  for (int c = 0; c < 6; c++) {
    double v = acc[c];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][c] = v;
  }
  __syncthreads();
  if (threadIdx.x < 6) {
    double v = 0.0;
    for (int w = 0; w < kNormThreads / 32; w++) v += red[w][threadIdx.x];
    part[(size_t)blockIdx.x * 6 + threadIdx.x] = v;
  }
}

__global__ void k_forces_final(int nblocks, const double* __restrict__ part, double* __restrict__ out) {
  const int lane = threadIdx.x & 31, c = threadIdx.x >> 5;
  if (c >= 6) return;
  const double v = warp_col_sum(part, nblocks, 6, c, lane);
  if (lane == 0) out[c] = v;
}

PCFD_API int pcfd_forces(pcfd_solver_t h, const int* tags, int ntags, double* out6) {
  Solver* s = (Solver*)h;
  if (!s || !tags || ntags <= 0 || !out6) return set_err(PCFD_ERR_ARG, "pcfd_forces: bad arguments");
  std::vector<int> mask(s->prm.ntags, 0);
  for (int i = 0; i < ntags; i++) {
    if (tags[i] < 0 || tags[i] >= s->prm.ntags) return set_err(PCFD_ERR_ARG, "pcfd_forces: tag without a BC");
    mask[tags[i]] = 1;
  }
  int rc;
  if (s->prm.viscous && (!s->have_grad || s->grad_arith != 0) && (rc = run_gradient(s, 0))) return rc;
  int* d_mask = nullptr;
  double* d_out = nullptr;
  if ((rc = dput(&d_mask, mask.data(), mask.size()))) return rc;
  if ((rc = dalloc(&d_out, 6))) { cudaFree(d_mask); return rc; }
  const double Sconst = 110.4 / s->prm.ref_temperature;
  const double inv_retilde = s->prm.Re != 0.0 ? s->prm.mach / s->prm.Re : 0.0;
  rc = launch(s, T_SETUP, [&] {
    k_forces<<<kNormBlocks, kNormThreads, 0, s->stream>>>(s->nbedge, s->d_bn, s->d_ba, s->d_bfactag, s->d_bbc, d_mask,
                                                          s->d_q, s->d_grad, s->prm.viscous, Sconst, inv_retilde,
                                                          s->d_part);
  });
  if (!rc) rc = launch(s, T_SETUP, [&] { k_forces_final<<<1, 192, 0, s->stream>>>(kNormBlocks, s->d_part, d_out); });
  if (!rc && cudaMemcpyAsync(out6, d_out, 6 * sizeof(double), cudaMemcpyDeviceToHost, s->stream) != cudaSuccess)
    rc = set_err(PCFD_ERR_CUDA, "pcfd_forces: copy");
  if (!rc && cudaStreamSynchronize(s->stream) != cudaSuccess) rc = set_err(PCFD_ERR_CUDA, "pcfd_forces: sync");
  cudaFree(d_mask);
  cudaFree(d_out);
  return rc;
}

PCFD_API int pcfd_limiter(pcfd_solver_t h, double* l_out) {
  Solver* s = (Solver*)h;
  if (!s) return set_err(PCFD_ERR_ARG, "pcfd_limiter: null handle");
  if (s->prm.limiter != 0 && !s->have_grad) return set_err(PCFD_ERR_STATE, "pcfd_limiter: gradient not computed");
  int rc = run_limiter(s, true);
  if (rc) return rc;
  if (l_out)
    CUDA_TRY(cudaMemcpyAsync(l_out, s->d_lim, (size_t)s->nnode * NEQN * sizeof(double), cudaMemcpyDeviceToHost,
                             s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PCFD_OK;
}

PCFD_API int pcfd_get_limiter(pcfd_solver_t h, double* l_out) {
  Solver* s = (Solver*)h;
  if (!s || !l_out) return set_err(PCFD_ERR_ARG, "pcfd_get_limiter: bad arguments");
  if (!s->have_lim) return set_err(PCFD_ERR_STATE, "pcfd_get_limiter: no limiter computed");
  const long long n = (long long)s->nnode * NEQN;
  if (s->lim_arith) {
    int rc = launch(s, T_SETUP, [&] { k_df_to_f64<<<kNormBlocks, 256, 0, s->stream>>>(n, s->f_lim, s->d_lim); });
    if (rc) return rc;
  }
  CUDA_TRY(cudaMemcpyAsync(l_out, s->d_lim, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PCFD_OK;
}

PCFD_API int pcfd_set_limiter(pcfd_solver_t h, const double* l) {
  Solver* s = (Solver*)h;
  if (!s || !l) return set_err(PCFD_ERR_ARG, "pcfd_set_limiter: bad arguments");
  const long long n = (long long)s->nnode * NEQN;
  CUDA_TRY(cudaMemcpyAsync(s->d_lim, l, n * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  if (s->arith) {
    int rc = ensure_df(s);
    if (rc || (rc = to_df_launch(s, s->d_lim, s->f_lim, n))) return rc;
  }
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  s->have_lim = 1;
  s->lim_arith = s->arith;
  s->lim_clipped = 1;  // final values: no pressure-clip pass follows
  s->lim_fresh = 0;
  return PCFD_OK;
}

PCFD_API int pcfd_residual(pcfd_solver_t h, double* b_out, double* norms_out) {
  Solver* s = (Solver*)h;
  if (!s) return set_err(PCFD_ERR_ARG, "pcfd_residual: null handle");
  int rc = run_residual(s);
  if (rc) return rc;
  if (b_out)
    CUDA_TRY(cudaMemcpyAsync(b_out, s->d_b, (size_t)s->nnode * NEQN * sizeof(double), cudaMemcpyDeviceToHost,
                             s->stream));
  if (norms_out)
    CUDA_TRY(cudaMemcpyAsync(norms_out, s->d_norms, 6 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PCFD_OK;
}

PCFD_API int pcfd_get_residual(pcfd_solver_t h, double* b_out) {
  Solver* s = (Solver*)h;
  if (!s || !b_out) return set_err(PCFD_ERR_ARG, "pcfd_get_residual: bad arguments");
  CUDA_TRY(cudaMemcpyAsync(b_out, s->d_b, (size_t)s->nnode * NEQN * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PCFD_OK;
}

PCFD_API int pcfd_residual_full(pcfd_solver_t h, double* norms_out) {
  Solver* s = (Solver*)h;
  if (!s) return set_err(PCFD_ERR_ARG, "pcfd_residual_full: null handle");
  const bool need_grad = s->prm.sorder > 1 || s->prm.viscous;
  int rc;
  if ((rc = run_bcs(s, s->arith))) return rc;
  if (need_grad) {
    if ((rc = run_gradient(s, s->arith))) return rc;
    if (s->prm.sorder > 1 && (rc = run_limiter(s, false, s->arith))) return rc;
  }
  if ((rc = run_residual(s, s->arith))) return rc;
  if (norms_out)
    CUDA_TRY(cudaMemcpyAsync(norms_out, s->d_norms, 6 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PCFD_OK;
}

PCFD_API int pcfd_bench_residual_full(pcfd_solver_t h, int nsteps, double* ms_out, double* norms_out) {
  Solver* s = (Solver*)h;
  if (!s || nsteps <= 0 || !ms_out) return set_err(PCFD_ERR_ARG, "pcfd_bench_residual_full: bad arguments");
  const bool need_grad = s->prm.sorder > 1 || s->prm.viscous;
  int saved = s->profile;
  s->profile = 0;
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  CUDA_TRY(cudaEventRecord(e0, s->stream));
  int rc = PCFD_OK;
  for (int it = 0; it < nsteps && rc == PCFD_OK; it++) {
    rc = run_bcs(s, s->arith);
    if (!rc && need_grad) rc = run_gradient(s, s->arith);
    if (!rc && need_grad && s->prm.sorder > 1) rc = run_limiter(s, false, s->arith);
    if (!rc) rc = run_residual(s, s->arith);
  }
  cudaEventRecord(e1, s->stream);
  cudaError_t ce = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  s->profile = saved;
  if (rc) return rc;
  if (ce != cudaSuccess) return set_err(PCFD_ERR_CUDA, std::string("bench: ") + cudaGetErrorString(ce));
  *ms_out = ms;
  if (norms_out) {
    CUDA_TRY(cudaMemcpyAsync(norms_out, s->d_norms, 6 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
  }
  return PCFD_OK;
}

PCFD_API int pcfd_set_residual_arithmetic(pcfd_solver_t h, int mode) {
  Solver* s = (Solver*)h;
  if (!s || (mode != 0 && mode != 1)) return set_err(PCFD_ERR_ARG, "pcfd_set_residual_arithmetic: mode must be 0 or 1");
  if (mode == 1) {
    int rc = ensure_df(s);
    if (rc) return rc;
    CUDA_TRY(cudaStreamSynchronize(s->stream));
  }
  s->arith = mode;
  s->have_grad = s->have_lim = 0;
  return PCFD_OK;
}

PCFD_API int pcfd_set_device(int device) {
  int n = 0;
  CUDA_TRY(cudaGetDeviceCount(&n));
  if (device < 0 || device >= n) return set_err(PCFD_ERR_ARG, "pcfd_set_device: no such device");
  CUDA_TRY(cudaSetDevice(device));
  return PCFD_OK;
}

PCFD_API int pcfd_device_sync(void) {
  CUDA_TRY(cudaDeviceSynchronize());
  return PCFD_OK;
}

PCFD_API int pcfd_timestep(pcfd_solver_t h, double cfl, double* dt_out, double* dtmin) {
  Solver* s = (Solver*)h;
  if (!s || !(cfl > 0.0)) return set_err(PCFD_ERR_ARG, "pcfd_timestep: bad arguments");
  int rc = run_timestep(s, cfl);
  if (rc) return rc;
  if (dt_out)
    CUDA_TRY(cudaMemcpyAsync(dt_out, s->d_dt, (size_t)s->nnode * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  if (dtmin) CUDA_TRY(cudaMemcpyAsync(dtmin, s->d_scal + 0, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PCFD_OK;
}

PCFD_API int pcfd_set_jacobian_precision(pcfd_solver_t h, int precision) {
  Solver* s = (Solver*)h;
  if (!s) return set_err(PCFD_ERR_ARG, "pcfd_set_jacobian_precision: null handle");
  int rc = ensure_matrix(s, precision);
  if (rc) return rc;
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PCFD_OK;
}

PCFD_API int pcfd_jacobian(pcfd_solver_t h) {
  Solver* s = (Solver*)h;
  if (!s) return set_err(PCFD_ERR_ARG, "pcfd_jacobian: null handle");
  int rc = run_jacobian(s);
  if (rc) return rc;
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PCFD_OK;
}

PCFD_API int pcfd_get_jacobian(pcfd_solver_t h, double* blocks, long long nblocks) {
  Solver* s = (Solver*)h;
  if (!s || !blocks || nblocks != s->nblocks) return set_err(PCFD_ERR_ARG, "pcfd_get_jacobian: bad arguments");
  if (!s->have_jac) return set_err(PCFD_ERR_STATE, "pcfd_get_jacobian: no Jacobian assembled");
  const size_t nv = (size_t)s->nblocks * 25;
  std::vector<double> out(nv);
  std::vector<char> raw(nv * prec_bytes(s->jac_prec));
  CUDA_TRY(cudaMemcpyAsync(raw.data(), s->d_M, raw.size(), cudaMemcpyDeviceToHost, s->stream));
  std::vector<double> diag((size_t)s->nnode * 25);
  std::vector<int> ia(s->nnode + 1);
  CUDA_TRY(cudaMemcpyAsync(diag.data(), s->d_diag, diag.size() * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaMemcpyAsync(ia.data(), s->d_ia, ia.size() * sizeof(int), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  for (size_t i = 0; i < nv; i++) {
    if (s->jac_prec == 0) out[i] = ((double*)raw.data())[i];
    else if (s->jac_prec == 1) out[i] = ((float*)raw.data())[i];
    else {
      uint16_t b = ((uint16_t*)raw.data())[i];
      uint32_t u = (uint32_t)b << 16;
      float f;
      std::memcpy(&f, &u, 4);
      out[i] = f;
    }
  }
  for (int i = 0; i < s->nnode; i++)
    for (int t = 0; t < 25; t++) out[(size_t)ia[i] * 25 + t] = diag[(size_t)i * 25 + t];
  std::memcpy(blocks, out.data(), nv * sizeof(double));
  return PCFD_OK;
}

PCFD_API int pcfd_crs_structure(pcfd_solver_t h, int* ia, int* ja, int* ncolor) {
  Solver* s = (Solver*)h;
  if (!s) return set_err(PCFD_ERR_ARG, "pcfd_crs_structure: null handle");
  if (ia) CUDA_TRY(cudaMemcpy(ia, s->d_ia, (size_t)(s->nnode + 1) * sizeof(int), cudaMemcpyDeviceToHost));
  if (ja) CUDA_TRY(cudaMemcpy(ja, s->d_ja, (size_t)s->nblocks * sizeof(int), cudaMemcpyDeviceToHost));
  if (ncolor) *ncolor = s->ncolor;
  return PCFD_OK;
}

PCFD_API int pcfd_coloring(pcfd_solver_t h, int* color_ptr, int* rows) {
  Solver* s = (Solver*)h;
  if (!s) return set_err(PCFD_ERR_ARG, "pcfd_coloring: null handle");
  if (color_ptr) std::memcpy(color_ptr, s->color_ptr.data(), s->color_ptr.size() * sizeof(int));
  if (rows) CUDA_TRY(cudaMemcpy(rows, s->d_color_rows, (size_t)s->nnode * sizeof(int), cudaMemcpyDeviceToHost));
  return PCFD_OK;
}

PCFD_API long long pcfd_nblocks(pcfd_solver_t h) {
  Solver* s = (Solver*)h;
  return s ? s->nblocks : -1;
}

PCFD_API int pcfd_sgs(pcfd_solver_t h, int nsweeps, double* x_out, double* dnorm) {
  Solver* s = (Solver*)h;
  if (!s || nsweeps < 0) return set_err(PCFD_ERR_ARG, "pcfd_sgs: bad arguments");
  CUDA_TRY(cudaMemsetAsync(s->d_x, 0, (size_t)s->nnode * NEQN * sizeof(double), s->stream));
  int rc = run_sgs(s, nsweeps, s->d_b, s->d_x, dnorm);
  if (rc) return rc;
  if (x_out)
    CUDA_TRY(cudaMemcpyAsync(x_out, s->d_x, (size_t)s->nnode * NEQN * sizeof(double), cudaMemcpyDeviceToHost,
                             s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return check_sweeps(s);
}

PCFD_API int pcfd_fgmres(pcfd_solver_t h, int m, int restarts, double rtol, int nsgs, double* x_out, double* relres,
                         int* iters) {
  Solver* s = (Solver*)h;
  if (!s || m < 1 || m > 60 || restarts < 1 || !(rtol > 0.0) || nsgs < 1)
    return set_err(PCFD_ERR_ARG, "pcfd_fgmres: bad arguments");
  if (!s->have_jac) return set_err(PCFD_ERR_STATE, "pcfd_fgmres: no Jacobian assembled");
  pcfd_newton_opts o = {};
  o.nsgs = nsgs;
  o.fgmres_m = m;
  o.fgmres_restarts = restarts;
  o.fgmres_rtol = rtol;
  CUDA_TRY(cudaMemsetAsync(s->d_x, 0, (size_t)s->nnode * NEQN * sizeof(double), s->stream));
  double rel = 1.0;
  int it = 0;
  int rc = run_fgmres(s, &o, &rel, &it);
  if (rc) return rc;
  if (x_out)
    CUDA_TRY(cudaMemcpyAsync(x_out, s->d_x, (size_t)s->nnode * NEQN * sizeof(double), cudaMemcpyDeviceToHost,
                             s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  if (relres) *relres = rel;
  if (iters) *iters = it;
  return check_sweeps(s);
}

PCFD_API int pcfd_matvec(pcfd_solver_t h, const double* x, double* y, int vec_precision) {
  Solver* s = (Solver*)h;
  if (!s || !x || !y || vec_precision < 0 || vec_precision > 1) return set_err(PCFD_ERR_ARG, "pcfd_matvec: bad arguments");
  if (!s->have_jac) return set_err(PCFD_ERR_STATE, "pcfd_matvec: no Jacobian assembled");
  if (vec_precision == 1 && s->jac_prec == 0)
    return set_err(PCFD_ERR_STATE, "pcfd_matvec: FP32 vectors need FP32 or BF16 matrix storage");
  const long long n = (long long)s->nnode * NEQN;
  // scratch: two FP64 vectors, then two FP32 vectors with tail padding
  if (!s->d_mv) {
    int rc = dalloc(&s->d_mv, (size_t)2 * n + (size_t)n + 4);
    if (rc) return rc;
  }
  double* xd = s->d_mv;
  double* yd = s->d_mv + n;
  float* xf = (float*)(s->d_mv + 2 * n);
  float* yf = xf + n + 4;
  CUDA_TRY(cudaMemcpyAsync(xd, x, n * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  int rc;
  if (vec_precision == 0) {
    rc = run_spmv(s, xd, yd);
  } else {
    rc = launch(s, T_SPMV, [&] { k_to_f32<<<kNormBlocks, 256, 0, s->stream>>>(n, xd, xf); });
    if (!rc) rc = run_spmv_f(s, xf, yf);
    if (!rc) rc = launch(s, T_SPMV, [&] { k_f32_to_f64<<<kNormBlocks, 256, 0, s->stream>>>(n, yf, yd); });
  }
  if (rc) return rc;
  CUDA_TRY(cudaMemcpyAsync(y, yd, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PCFD_OK;
}

PCFD_API int pcfd_bench_spmv(pcfd_solver_t h, int nrep, int vec_precision, double* ms_out) {
  Solver* s = (Solver*)h;
  if (!s || nrep <= 0 || !ms_out || vec_precision < 0 || vec_precision > 1)
    return set_err(PCFD_ERR_ARG, "pcfd_bench_spmv: bad arguments");
  if (!s->have_jac) return set_err(PCFD_ERR_STATE, "pcfd_bench_spmv: no Jacobian assembled");
  if (vec_precision == 1 && s->jac_prec == 0)
    return set_err(PCFD_ERR_STATE, "pcfd_bench_spmv: FP32 vectors need FP32 or BF16 matrix storage");
  const long long n = (long long)s->nnode * NEQN;
  if (!s->d_mv) {
    int rc = dalloc(&s->d_mv, (size_t)2 * n + (size_t)n + 4);
    if (rc) return rc;
  }
  double* xd = s->d_mv;
  double* yd = s->d_mv + n;
  float* xf = (float*)(s->d_mv + 2 * n);
  float* yf = xf + n + 4;
  // x = 0 (the products' cost does not depend on the values)
  CUDA_TRY(cudaMemsetAsync(s->d_mv, 0, ((size_t)2 * n + (size_t)n + 4) * sizeof(double), s->stream));
  int saved = s->profile;
  s->profile = 0;
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  CUDA_TRY(cudaEventRecord(e0, s->stream));
  int rc = PCFD_OK;
  for (int it = 0; it < nrep && rc == PCFD_OK; it++) rc = vec_precision ? run_spmv_f(s, xf, yf) : run_spmv(s, xd, yd);
  cudaEventRecord(e1, s->stream);
  cudaError_t ce = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  s->profile = saved;
  if (rc) return rc;
  if (ce != cudaSuccess) return set_err(PCFD_ERR_CUDA, std::string("bench spmv: ") + cudaGetErrorString(ce));
  *ms_out = ms;
  return PCFD_OK;
}

PCFD_API int pcfd_bench_sgs(pcfd_solver_t h, int nrep, int nsweeps, int vec_precision, double* ms_out) {
  Solver* s = (Solver*)h;
  if (!s || nrep <= 0 || nsweeps <= 0 || !ms_out || vec_precision < 0 || vec_precision > 1)
    return set_err(PCFD_ERR_ARG, "pcfd_bench_sgs: bad arguments");
  if (!s->have_jac) return set_err(PCFD_ERR_STATE, "pcfd_bench_sgs: no Jacobian assembled");
  if (vec_precision == 1 && s->jac_prec == 0)
    return set_err(PCFD_ERR_STATE, "pcfd_bench_sgs: FP32 vectors need FP32 or BF16 matrix storage");
  const long long n = (long long)s->nnode * NEQN;
  if (!s->d_mv) {
    int rc = dalloc(&s->d_mv, (size_t)2 * n + (size_t)n + 4);
    if (rc) return rc;
  }
  double* xd = s->d_mv + n;
  float* bf = (float*)(s->d_mv + 2 * n);
  float* xf = bf + n + 4;
  // the right-hand side is the last residual (its values do not change the
  // sweeps' work)
  int rc = PCFD_OK;
  if (vec_precision == 1) rc = launch(s, T_SGS, [&] { k_to_f32<<<kNormBlocks, 256, 0, s->stream>>>(n, s->d_b, bf); });
  if (rc) return rc;
  CUDA_TRY(cudaMemsetAsync(xd, 0, n * sizeof(double), s->stream));
  CUDA_TRY(cudaMemsetAsync(xf, 0, n * sizeof(float), s->stream));
  int saved = s->profile;
  s->profile = 0;
  cudaEvent_t e0, e1;
  CUDA_TRY(cudaEventCreate(&e0));
  CUDA_TRY(cudaEventCreate(&e1));
  CUDA_TRY(cudaEventRecord(e0, s->stream));
  for (int it = 0; it < nrep && rc == PCFD_OK; it++)
    rc = vec_precision ? run_sgs_f(s, nsweeps, bf, xf) : run_sgs(s, nsweeps, s->d_b, xd, nullptr);
  cudaEventRecord(e1, s->stream);
  cudaError_t ce = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  s->profile = saved;
  if (rc) return rc;
  if (ce != cudaSuccess) return set_err(PCFD_ERR_CUDA, std::string("bench sgs: ") + cudaGetErrorString(ce));
  *ms_out = ms;
  return check_sweeps(s);
}

PCFD_API int pcfd_sgs_rhs(pcfd_solver_t h, int nsweeps, const double* b, double* x_out, int vec_precision) {
  Solver* s = (Solver*)h;
  if (!s || !b || !x_out || nsweeps < 0 || vec_precision < 0 || vec_precision > 1)
    return set_err(PCFD_ERR_ARG, "pcfd_sgs_rhs: bad arguments");
  if (!s->have_jac) return set_err(PCFD_ERR_STATE, "pcfd_sgs_rhs: no Jacobian assembled");
  if (vec_precision == 1 && s->jac_prec == 0)
    return set_err(PCFD_ERR_STATE, "pcfd_sgs_rhs: FP32 vectors need FP32 or BF16 matrix storage");
  const long long n = (long long)s->nnode * NEQN;
  if (!s->d_mv) {
    int rc = dalloc(&s->d_mv, (size_t)2 * n + (size_t)n + 4);
    if (rc) return rc;
  }
  double* bd = s->d_mv;
  double* xd = s->d_mv + n;
  float* bf = (float*)(s->d_mv + 2 * n);
  float* xf = bf + n + 4;
  CUDA_TRY(cudaMemcpyAsync(bd, b, n * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  int rc;
  if (vec_precision == 0) {
    CUDA_TRY(cudaMemsetAsync(xd, 0, n * sizeof(double), s->stream));
    rc = run_sgs(s, nsweeps, bd, xd, nullptr);
  } else {
    CUDA_TRY(cudaMemsetAsync(xf, 0, n * sizeof(float), s->stream));
    rc = launch(s, T_SGS, [&] { k_to_f32<<<kNormBlocks, 256, 0, s->stream>>>(n, bd, bf); });
    if (!rc) rc = run_sgs_f(s, nsweeps, bf, xf);
    if (!rc) rc = launch(s, T_SGS, [&] { k_f32_to_f64<<<kNormBlocks, 256, 0, s->stream>>>(n, xf, xd); });
  }
  if (rc) return rc;
  CUDA_TRY(cudaMemcpyAsync(x_out, xd, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return check_sweeps(s);
}

PCFD_API int pcfd_apply_dq(pcfd_solver_t h, const double* x_in, double* dqnorm) {
  Solver* s = (Solver*)h;
  if (!s) return set_err(PCFD_ERR_ARG, "pcfd_apply_dq: null handle");
  if (x_in)
    CUDA_TRY(cudaMemcpyAsync(s->d_x, x_in, (size_t)s->nnode * NEQN * sizeof(double), cudaMemcpyHostToDevice,
                             s->stream));
  int rc = run_apply_dq(s, dqnorm);
  if (rc) return rc;
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PCFD_OK;
}

PCFD_API int pcfd_newton_step(pcfd_solver_t h, const pcfd_newton_opts* o, pcfd_newton_report* rep) {
  Solver* s = (Solver*)h;
  if (!s || !o || o->iter < 0 || o->nsgs < 0 || !(o->cfl > 0.0))
    return set_err(PCFD_ERR_ARG, "pcfd_newton_step: bad arguments");
  if (o->linear_solver < 0 || o->linear_solver > 3)
    return set_err(PCFD_ERR_ARG,
                   "pcfd_newton_step: linear_solver must be 0 (SGS), 1 (FGMRES), 2 or 3 (learned)");
  if (o->linear_solver >= 2 && !s->lp)
    return set_err(PCFD_ERR_STATE, "pcfd_newton_step: linear_solver 2 and 3 need pcfd_lp_init");
  int rc;
  if (o->jac_precision != s->jac_prec && (rc = ensure_matrix(s, o->jac_precision))) return rc;
  const double cfl = ramp_cfl(o->iter, o->cfl_start > 0.0 ? o->cfl_start : o->cfl, o->cfl, o->cfl_ramp_steps);
  // SolutionSpace::PreIterate (ucs/solutionSpace.tcc:510): a time step exists
  // before the first Jacobian
  if (!s->have_dt && (rc = run_timestep(s, cfl))) return rc;
  // PreTimeAdvance (:573): the state becomes the step's q_old (EvolveInTime),
  // the Jacobian uses the time step of the previous iteration, then this
  // iteration's CFL and time steps
  if (s->prm.torder && (rc = save_qold(s))) return rc;
  const int jf = o->jac_update_freq > 0 ? o->jac_update_freq : 1;
  if (o->nsgs > 0 && (o->iter % jf == 0 || o->iter == 1 || !s->have_jac) && (rc = run_jacobian(s))) return rc;
  if ((rc = run_timestep(s, cfl))) return rc;
  // NewtonIterate (:640): gradient when second order is active or viscous;
  // the limiter every limiter_refresh iterations until limiter_freeze, the
  // frozen values otherwise (:671-690)
  if ((rc = run_bcs(s, s->arith))) return rc;
  const bool ho_now = s->prm.sorder > 1 && o->iter > o->first_order_steps;
  const int refresh = o->limiter_refresh > 0 ? o->limiter_refresh : 1;
  const bool frozen = o->limiter_freeze > 0 && o->iter >= o->limiter_freeze;
  const bool recompute = (o->iter % refresh == 0 && !frozen) || !s->have_lim || s->lim_arith != s->arith;
  if ((ho_now || s->prm.viscous) && (rc = run_gradient(s, s->arith))) return rc;
  if (ho_now && (s->prm.limiter == 0 || recompute) && (rc = run_limiter(s, false, s->arith))) return rc;
  if ((rc = run_residual(s, s->arith, !ho_now))) return rc;
  double lin = 0.0;
  int lin_it = 0, fallbacks = 0;
  CUDA_TRY(cudaMemsetAsync(s->d_x, 0, (size_t)s->nnode * NEQN * sizeof(double), s->stream));
  if (o->nsgs > 0) {
    if (o->linear_solver == 0) {
      if ((rc = run_sgs(s, o->nsgs, s->d_b, s->d_x, &lin))) return rc;
      lin_it = o->nsgs;
    } else {
      if ((rc = run_fgmres(s, o, &lin, &lin_it, o->linear_solver >= 2, &fallbacks, o->linear_solver == 3)))
        return rc;
      if (o->linear_solver >= 2 && (rc = lp_check_err(s))) return rc;
    }
  }
  double dqn = 0.0;
  if ((rc = run_apply_dq(s, &dqn))) return rc;
  if (rep) {
    std::memset(rep, 0, sizeof(*rep));
    CUDA_TRY(cudaMemcpyAsync(rep->res, s->d_norms, 6 * sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaMemcpyAsync(&rep->dtmin, s->d_scal + 0, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
    CUDA_TRY(cudaStreamSynchronize(s->stream));
    rep->dqnorm = dqn;
    rep->lin_res = lin;
    rep->lin_iters = lin_it;
    rep->cfl = cfl;
    rep->lp_fallbacks = fallbacks;
  } else {
    CUDA_TRY(cudaStreamSynchronize(s->stream));
  }
  return check_sweeps(s);
}

// ---- learned right preconditioner --------------------------------------

PCFD_API int pcfd_lp_init(pcfd_solver_t h, unsigned long long seed) {
  Solver* s = (Solver*)h;
  if (!s) return set_err(PCFD_ERR_ARG, "null handle");
  free_learned(s->lp);
  s->lp = nullptr;
  int rc = lp_alloc(s);
  if (rc) {
    free_learned(s->lp);
    s->lp = nullptr;
    return rc;
  }
  std::vector<float> w;
  lp_initial_params(seed, w);
  return lp_set_params(s, w.data());
}

static Learned* lp_of(pcfd_solver_t h, const char* fn) {
  Solver* s = (Solver*)h;
  if (!s) {
    set_err(PCFD_ERR_ARG, std::string(fn) + ": null handle");
    return nullptr;
  }
  if (!s->lp) set_err(PCFD_ERR_STATE, std::string(fn) + ": pcfd_lp_init not called");
  return s->lp;
}

PCFD_API int pcfd_lp_get_params(pcfd_solver_t h, float* w) {
  Learned* lp = lp_of(h, "pcfd_lp_get_params");
  if (!lp) return h ? PCFD_ERR_STATE : PCFD_ERR_ARG;
  if (!w) return set_err(PCFD_ERR_ARG, "pcfd_lp_get_params: null pointer");
  Solver* s = (Solver*)h;
  CUDA_TRY(cudaMemcpyAsync(w, lp->w, LP_NPARAM * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  return PCFD_OK;
}

PCFD_API int pcfd_lp_set_params(pcfd_solver_t h, const float* w) {
  Learned* lp = lp_of(h, "pcfd_lp_set_params");
  if (!lp) return h ? PCFD_ERR_STATE : PCFD_ERR_ARG;
  if (!w) return set_err(PCFD_ERR_ARG, "pcfd_lp_set_params: null pointer");
  return lp_set_params((Solver*)h, w);
}

PCFD_API int pcfd_lp_forward(pcfd_solver_t h, const float* x, float* out) {
  Learned* lp = lp_of(h, "pcfd_lp_forward");
  if (!lp) return h ? PCFD_ERR_STATE : PCFD_ERR_ARG;
  if (!x || !out) return set_err(PCFD_ERR_ARG, "pcfd_lp_forward: null pointer");
  Solver* s = (Solver*)h;
  CUDA_TRY(cudaMemcpyAsync(lp->x, x, (size_t)lp->n * LP_NIN * sizeof(float), cudaMemcpyHostToDevice, s->stream));
  int rc = lp_forward(s, true, nullptr);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpyAsync(out, lp->out, (size_t)lp->n * LP_NOUT * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
  return lp_check_err(s);
}

PCFD_API int pcfd_lp_loss_grad(pcfd_solver_t h, const float* x, const float* t, float* grad, double* loss) {
  Learned* lp = lp_of(h, "pcfd_lp_loss_grad");
  if (!lp) return h ? PCFD_ERR_STATE : PCFD_ERR_ARG;
  if (!x || !t) return set_err(PCFD_ERR_ARG, "pcfd_lp_loss_grad: null pointer");
  Solver* s = (Solver*)h;
  CUDA_TRY(cudaMemcpyAsync(lp->x, x, (size_t)lp->n * LP_NIN * sizeof(float), cudaMemcpyHostToDevice, s->stream));
  CUDA_TRY(cudaMemcpyAsync(lp->t, t, (size_t)lp->n * LP_NOUT * sizeof(float), cudaMemcpyHostToDevice, s->stream));
  int rc = lp_forward(s, true, nullptr);
  if (rc || (rc = lp_backward(s))) return rc;
  std::vector<float> g(LP_NPARAM + 1);
  CUDA_TRY(cudaMemcpyAsync(g.data(), lp->g, (LP_NPARAM + 1) * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
  if ((rc = lp_check_err(s))) return rc;
  if (grad) std::memcpy(grad, g.data(), LP_NPARAM * sizeof(float));
  if (loss) *loss = (double)g[LP_NPARAM] / (5.0 * lp->n);
  return PCFD_OK;
}

PCFD_API int pcfd_lp_features(pcfd_solver_t h, const double* y, float* x, double* sigma_out) {
  Learned* lp = lp_of(h, "pcfd_lp_features");
  if (!lp) return h ? PCFD_ERR_STATE : PCFD_ERR_ARG;
  if (!y || !x) return set_err(PCFD_ERR_ARG, "pcfd_lp_features: null pointer");
  Solver* s = (Solver*)h;
  CUDA_TRY(cudaMemcpyAsync(lp->y, y, (size_t)lp->n * NEQN * sizeof(double), cudaMemcpyHostToDevice, s->stream));
  int rc = lp_features(s);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpyAsync(x, lp->x, (size_t)lp->n * LP_NIN * sizeof(float), cudaMemcpyDeviceToHost, s->stream));
  double sg = 0.0;
  CUDA_TRY(cudaMemcpyAsync(&sg, lp->sigma, sizeof(double), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  if (sigma_out) *sigma_out = sg;
  return PCFD_OK;
}

PCFD_API int pcfd_lp_apply(pcfd_solver_t h, int nsgs, const double* v, double* z) {
  Learned* lp = lp_of(h, "pcfd_lp_apply");
  if (!lp) return h ? PCFD_ERR_STATE : PCFD_ERR_ARG;
  if (!v || !z || nsgs < 1) return set_err(PCFD_ERR_ARG, "pcfd_lp_apply: bad arguments");
  Solver* s = (Solver*)h;
  const size_t bytes = (size_t)lp->n * NEQN * sizeof(double);
  CUDA_TRY(cudaMemcpyAsync(lp->vbuf, v, bytes, cudaMemcpyHostToDevice, s->stream));
  int rc = lp_precondition(s, nsgs, lp->vbuf, s->d_x);
  if (rc) return rc;
  CUDA_TRY(cudaMemcpyAsync(z, s->d_x, bytes, cudaMemcpyDeviceToHost, s->stream));
  return lp_check_err(s);
}

// store the features of lp->y and the target (xt - y)/sigma as a new pair
int lp_store_pair(Solver* s, const double* xt) {
  Learned* lp = s->lp;
  const size_t n5 = (size_t)lp->n * NEQN;
  int rc = lp_features(s);
  if (rc) return rc;
  float *sx = nullptr, *st = nullptr;
  if ((rc = dalloc(&sx, (size_t)lp->n * LP_NIN))) return rc;
  if ((rc = dalloc(&st, n5))) {
    cudaFree(sx);
    return rc;
  }
  lp->sx.push_back(sx);
  lp->st.push_back(st);
  CUDA_TRY(cudaMemcpyAsync(sx, lp->x, (size_t)lp->n * LP_NIN * sizeof(float), cudaMemcpyDeviceToDevice, s->stream));
  return launch(s, T_LP_BWD, [&] {
    k_lp_target<<<kNormBlocks, 256, 0, s->stream>>>((long long)n5, xt, lp->y, lp->sigma, st);
  });
}

PCFD_API int pcfd_lp_collect(pcfd_solver_t h, int nsgs, double rtol, int krylov_pairs, int* nsamples_out) {
  Learned* lp = lp_of(h, "pcfd_lp_collect");
  if (!lp) return h ? PCFD_ERR_STATE : PCFD_ERR_ARG;
  Solver* s = (Solver*)h;
  if (nsgs < 1 || !(rtol > 0.0) || krylov_pairs < 0)
    return set_err(PCFD_ERR_ARG, "pcfd_lp_collect: bad arguments");
  if (!s->have_jac) return set_err(PCFD_ERR_STATE, "pcfd_lp_collect: no linear system (run pcfd_newton_step first)");
  const size_t n5 = (size_t)lp->n * NEQN;
  // dq: A dq = b to rtol by SGS-preconditioned FGMRES(30)
  pcfd_newton_opts o = {};
  o.nsgs = 1;
  o.fgmres_m = 30;
  o.fgmres_restarts = 50;
  o.fgmres_rtol = rtol;
  CUDA_TRY(cudaMemsetAsync(s->d_x, 0, n5 * sizeof(double), s->stream));
  double rel = 1.0;
  int it = 0;
  int rc = run_fgmres(s, &o, &rel, &it);
  if (rc) return rc;
  CUDA_TRY(cudaMemsetAsync(lp->y, 0, n5 * sizeof(double), s->stream));
  if ((rc = run_sgs(s, nsgs, s->d_b, lp->y, nullptr)) || (rc = lp_store_pair(s, s->d_x))) return rc;
  // (A z_j, z_j) for the directions of the last FGMRES cycle
  const int nk = std::min(std::min(krylov_pairs, it), s->fg_m);
  for (int j = 0; j < nk; j++) {
    const double* zj = s->d_Z + (size_t)j * n5;
    if (s->jac_prec != 0) {
      // FP32 Krylov directions: an FP64 copy
      const float* zf = (const float*)s->d_Z + (size_t)j * n5;
      rc = launch(s, T_KRYLOV, [&] { k_f32_to_f64<<<kNormBlocks, 256, 0, s->stream>>>((long long)n5, zf, s->d_wd); });
      if (rc) return rc;
      zj = s->d_wd;
    }
    if ((rc = run_spmv(s, zj, lp->vbuf))) return rc;
    CUDA_TRY(cudaMemsetAsync(lp->y, 0, n5 * sizeof(double), s->stream));
    if ((rc = run_sgs(s, nsgs, lp->vbuf, lp->y, nullptr)) || (rc = lp_store_pair(s, zj))) return rc;
  }
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  if (nsamples_out) *nsamples_out = (int)lp->sx.size();
  return PCFD_OK;
}

PCFD_API int pcfd_lp_clear_samples(pcfd_solver_t h) {
  Learned* lp = lp_of(h, "pcfd_lp_clear_samples");
  if (!lp) return h ? PCFD_ERR_STATE : PCFD_ERR_ARG;
  CUDA_TRY(cudaStreamSynchronize(((Solver*)h)->stream));
  for (float* p : lp->sx) cudaFree(p);
  for (float* p : lp->st) cudaFree(p);
  lp->sx.clear();
  lp->st.clear();
  return PCFD_OK;
}

PCFD_API int pcfd_lp_train(pcfd_solver_t h, int epochs, double lr, double* loss_first, double* loss_last) {
  Learned* lp = lp_of(h, "pcfd_lp_train");
  if (!lp) return h ? PCFD_ERR_STATE : PCFD_ERR_ARG;
  Solver* s = (Solver*)h;
  if (epochs < 1 || !(lr > 0.0)) return set_err(PCFD_ERR_ARG, "pcfd_lp_train: bad arguments");
  if (lp->sx.empty()) return set_err(PCFD_ERR_STATE, "pcfd_lp_train: no training pairs (pcfd_lp_collect)");
  const int ns = (int)lp->sx.size();
  std::vector<float> lsum(ns);
  for (int e = 0; e < epochs; e++) {
    double tot = 0.0;
    for (int k = 0; k < ns; k++) {
      CUDA_TRY(cudaMemcpyAsync(lp->x, lp->sx[k], (size_t)lp->n * LP_NIN * sizeof(float), cudaMemcpyDeviceToDevice,
                               s->stream));
      CUDA_TRY(cudaMemcpyAsync(lp->t, lp->st[k], (size_t)lp->n * LP_NOUT * sizeof(float), cudaMemcpyDeviceToDevice,
                               s->stream));
      int rc = lp_forward(s, true, nullptr);
      if (rc || (rc = lp_backward(s))) return rc;
      CUDA_TRY(cudaMemcpyAsync(&lsum[k], lp->g + LP_NPARAM, sizeof(float), cudaMemcpyDeviceToHost, s->stream));
      if ((rc = lp_adam_step(s, lr))) return rc;
    }
    int rc = lp_check_err(s);
    if (rc) return rc;
    for (int k = 0; k < ns; k++) tot += (double)lsum[k] / (5.0 * lp->n);
    if (e == 0 && loss_first) *loss_first = tot / ns;
    if (e == epochs - 1 && loss_last) *loss_last = tot / ns;
  }
  return PCFD_OK;
}

PCFD_API int pcfd_profile_enable(pcfd_solver_t h, int on) {
  Solver* s = (Solver*)h;
  if (!s) return set_err(PCFD_ERR_ARG, "null handle");
  s->profile = on ? 1 : 0;
  return PCFD_OK;
}

PCFD_API int pcfd_profile_reset(pcfd_solver_t h) {
  Solver* s = (Solver*)h;
  if (!s) return set_err(PCFD_ERR_ARG, "null handle");
  for (int i = 0; i < T_COUNT; i++) { s->t_ms[i] = 0.0; s->t_n[i] = 0; }
  return PCFD_OK;
}

PCFD_API int pcfd_profile_get(pcfd_solver_t h, int i, char* name_buf, int name_len, double* ms_total,
                              long long* launches) {
  Solver* s = (Solver*)h;
  if (!s || i < 0 || i >= T_COUNT) return PCFD_ERR_ARG;
  if (name_buf && name_len > 0) {
    std::strncpy(name_buf, kTimerNames[i], name_len - 1);
    name_buf[name_len - 1] = 0;
  }
  if (ms_total) *ms_total = s->t_ms[i];
  if (launches) *launches = s->t_n[i];
  return PCFD_OK;
}

PCFD_API long long pcfd_launch_count(pcfd_solver_t h) {
  Solver* s = (Solver*)h;
  return s ? s->launches : -1;
}

PCFD_API int pcfd_get_health(pcfd_solver_t h, long long* c8) {
  Solver* s = (Solver*)h;
  if (!s || !c8) return set_err(PCFD_ERR_ARG, "pcfd_get_health: bad arguments");
  unsigned long long tmp[8];
  CUDA_TRY(cudaMemcpyAsync(tmp, s->d_health, sizeof(tmp), cudaMemcpyDeviceToHost, s->stream));
  CUDA_TRY(cudaStreamSynchronize(s->stream));
  for (int i = 0; i < 8; i++) c8[i] = (long long)tmp[i];
  return PCFD_OK;
}

}  // extern "C"
