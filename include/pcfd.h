/*
 * pcfd.h - C ABI of the GB300 (sm_103a) implementation of ProteusCFD's
 * implicit edge-based finite-volume hot path.
 *
 * Every entry point is extern "C", takes plain pointers and sizes, returns an
 * int status (PCFD_OK = 0) and never exits the process; pcfd_last_error()
 * gives the text of the last failure on the calling thread.  All device
 * entry points are synchronous at return and run on the handle's own CUDA
 * stream.  Caller buffers are borrowed only for the duration of a call; the
 * library owns its device mirrors and never frees caller memory.
 *
 * Each entry point names the reference interface it stands in for
 * (file:line within ngcurrier/ProteusCFD).
 */
#ifndef PCFD_H_
#define PCFD_H_

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define PCFD_API __attribute__((visibility("default")))
#else
#define PCFD_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ------------------------------------------------------ */
#define PCFD_OK 0
#define PCFD_ERR_ARG 1         /* bad argument (null pointer, size out of range) */
#define PCFD_ERR_STATE 2       /* call made in the wrong order */
#define PCFD_ERR_CUDA 3        /* CUDA runtime error */
#define PCFD_ERR_MESH 4        /* mesh preprocessing failed */
#define PCFD_ERR_NOMEM 5       /* allocation failed */
#define PCFD_ERR_UNSUPPORTED 6 /* option the library does not support */
#define PCFD_ERR_NUMERIC 7     /* device reported a numerical failure (see pcfd_get_health) */

/* ---- boundary condition types -------------------------------------------
 * Same integer values as the reference's BCTypes enum (ucs/bc_defines.h:4),
 * so a .bc table read by the reference can be passed through unchanged.    */
enum pcfd_bc_type {
  PCFD_BC_PARALLEL = 0,
  PCFD_BC_DIRICHLET = 1,
  PCFD_BC_NEUMANN = 2,
  PCFD_BC_IMPERMEABLE_WALL = 3,
  PCFD_BC_NOSLIP = 4,
  PCFD_BC_FARFIELD_VISCOUS = 5,
  PCFD_BC_FARFIELD = 6,
  PCFD_BC_SONIC_INFLOW = 7,
  PCFD_BC_SONIC_OUTFLOW = 8,
  PCFD_BC_SYMMETRY = 9
};

/* ---- host mesh preprocessing -------------------------------------------- */

/* Synthetic workload: an nx*ny*nz node box split into 6 Kuhn tets per hex.
 * tags[f] is the boundary tag of face f (x=0, x=max, y=0, y=max, z=0, z=max). */
typedef struct pcfd_box_params {
  int nx, ny, nz;
  double lx, ly, lz;  /* box extents */
  double jitter;      /* interior-node jitter as a fraction of the local spacing */
  uint64_t seed;      /* jitter seed */
  double ramp_deg;    /* shear ramp angle of the y=0 wall for x > ramp_x0 (0 = none) */
  double ramp_x0;
  double y_ratio;     /* geometric clustering ratio toward y=0 (<= 1: uniform) */
  int tags[6];
  int jitter_mode;    /* 0: each axis by its own local spacing; 1: every axis by the node's
                       * smallest local spacing (keeps stretched near-wall cells valid) */
  int wall_start_i;   /* y=0 face cells with i < wall_start_i carry upstream_tag instead of
                       * tags[2] (a run-in ahead of a wall's leading edge; 0 = none) */
  int upstream_tag;
  double wall_ar_max; /* y clustering with a floor on the first wall cell: at least the x
                       * spacing / wall_ar_max high; the spacing grows by y_ratio from there
                       * and stops growing at the spacing that fills ly (0: one geometric
                       * series over the whole height, however thin its first cell) */
} pcfd_box_params;

typedef void* pcfd_mesh_t;

/* Mesh arrays in the reference's layout (Mesh<T> members, ucs/mesh.h:202-203;
 * Edges/HalfEdges, ucs/uns_base.h:13,28).  Phantom node of half-edge k is
 * nnode + k.  All arrays are host memory. */
typedef struct pcfd_mesh_view {
  int nnode;               /* interior nodes */
  int nbnode;              /* phantom (boundary) nodes = nbedge */
  int nedge;               /* interior edges */
  int nbedge;              /* boundary half-edges */
  const int* edges;        /* [nedge][2] (Edges::n) */
  const double* edge_area; /* [nedge][4] unit normal + magnitude (Edges::a) */
  const int* bedges;       /* [nbedge][2] node, phantom id (HalfEdges::n) */
  const double* bedge_area;/* [nbedge][4] (HalfEdges::a) */
  const int* bfactag;      /* [nbedge] (HalfEdges::factag) */
  const double* xyz;       /* [nnode][3] */
  const double* vol;       /* [nnode] dual volumes */
  const double* sw;        /* [nnode][6] weighted LSQ normal matrix (Mesh::sw) */
  const int* ipsp;         /* [nnode+1] */
  const int* psp;          /* [ipsp[nnode]] */
} pcfd_mesh_view;

/* Generator for the synthetic boxes (no reference counterpart: the reference
 * reads meshes from files, ucs/mesh.tcc:2820). */
PCFD_API pcfd_mesh_t pcfd_mesh_box_create(const pcfd_box_params* p);
/* Element-list input, the data a UGRID reader would produce
 * (ucs/mesh.tcc:6740): triangles [ntri][3] with tags, tets [ntet][4]. */
PCFD_API pcfd_mesh_t pcfd_mesh_from_elements(int nnode, const double* xyz, int ntri, const int* tri,
                                             const int* tri_tag, int ntet, const int* tet);
/* Mesh::BuildMaps + Mesh::CalcMetrics (ucs/mesh.tcc:265,1576) and
 * ComputeNodeLSQCoefficients (ucs/gradient.tcc:115). */
PCFD_API int pcfd_mesh_build(pcfd_mesh_t m);
PCFD_API int pcfd_mesh_view_get(pcfd_mesh_t m, pcfd_mesh_view* v);
PCFD_API int pcfd_mesh_stats(pcfd_mesh_t m, int* nelem_tri, int* nelem_tet, int* rewound, int* unclosed,
                             double* max_open, double* total_vol);
/* The array Mesh::ReorderMeshCuthillMcKee(1) leaves in Mesh::ordering
 * (ucs/mesh.tcc:2412-2490), bit for bit: Cuthill-McKee from node 0 with
 * degree-sorted neighbour lists, reversed.  The reference then uses it as an
 * old-to-new map (ReorderC2nMap, :224): node n becomes ordering[n].  Computed
 * on the current numbering; builds the point-surrounding-point map if needed. */
PCFD_API int pcfd_mesh_rcm_order(pcfd_mesh_t m, int* order_out);
/* The reference's set-up reorder (SolutionSpace constructor,
 * ucs/solutionSpace.tcc:61-66: BuildMapsDecomp, ReorderMeshCuthillMcKee(1),
 * ReorderC2nMap) applied to the element list and coordinates; call
 * pcfd_mesh_build afterwards.  order_out (optional, [nnode]) receives the
 * ordering array. */
PCFD_API int pcfd_mesh_reorder_rcm(pcfd_mesh_t m, int* order_out);
/* Renumber nodes by an explicit permutation, order[new] = old (a
 * ReorderC2nMap with a caller's map); rebuild afterwards. */
PCFD_API int pcfd_mesh_renumber(pcfd_mesh_t m, const int* order);
PCFD_API void pcfd_mesh_destroy(pcfd_mesh_t m);
PCFD_API const char* pcfd_mesh_last_error(void);

/* ---- device solver ------------------------------------------------------- */

/* The subset of Param<T> (ucs/param.h:31) the hot path reads.  Values are the
 * reference's non-dimensional ones (velocity scale = freestream sound speed). */
typedef struct pcfd_params {
  double gamma;           /* Param::gamma */
  double mach;            /* Param::velocity (= Mach number) */
  double flowdir[3];      /* Param::flowdir */
  double Re;              /* Param::Re */
  double Pr, PrT;         /* Param::Pr, Param::PrT */
  double ref_temperature; /* Param::ref_temperature [K] (Sutherland, wall T) */
  int sorder;             /* spatial order 1 or 2 (Param::sorder) */
  double chi;             /* MUSCL blend (Param::chi) */
  int viscous;            /* 0 Euler, 1 laminar Navier-Stokes */
  int limiter;            /* Param::limiter: 0 none, 1 Barth, 2 Venkatakrishnan, 3 modified Venkatakrishnan */
  double venkat_K;        /* modified Venkatakrishnan K; the reference hard-codes 1.0 */
  int no_cvbc;            /* Param::no_cvbc */
  int jac_boundary_eval;  /* Param::boundaryJacEval: 0 re-derive the phantom state from each
                           * perturbed interior state (reference default), 1 keep it frozen;
                           * 3 re-derive it for the base state too, so the boundary
                           * condition's sub-iteration drift cancels (no reference counterpart) */
  int ntags;              /* entries in bc_type/bc_twall, indexed by factag */
  const int* bc_type;     /* pcfd_bc_type per factag */
  const double* bc_twall; /* BCObj::twall per factag [K]; < 0 = adiabatic */
  int torder;             /* Param::torder: 1 adds the temporal residual (TemporalResidual,
                           * ucs/residual.tcc:125) as the reference always does (its default
                           * and minimum); 0 leaves it out */
  double time_step;       /* Param::dt ("timeStep"): must be <= 0, a steady run; the reference's
                           * default -1.0 makes the temporal residual b += vol (q - q_old), with
                           * q_old the state at the start of the step (0 reads as -1.0) */
  double tinf, pinf;      /* non-dimensional freestream temperature and pressure,
                           * initialTemperature/ref_temperature and initialPressure/ref_pressure
                           * (CompressibleEqnSet::UpdateQinf, ucs/compressible.tcc:835-836); the
                           * reference's scaling makes both 1 up to rounding; 0 reads as 1 */
} pcfd_params;

typedef void* pcfd_solver_t;

/* Allocates device mirrors of the mesh and all fields (SolutionSpace::Init,
 * ucs/solutionSpace.tcc:148) and initialises q to the freestream
 * (CompressibleEqnSet::SetInitialConditions, ucs/compressible.tcc:884). */
PCFD_API int pcfd_create(const pcfd_mesh_view* mesh, const pcfd_params* params, pcfd_solver_t* out);
PCFD_API int pcfd_destroy(pcfd_solver_t s);

/* q in the reference layout: [nnode+nbnode][nvars], nvars = 10
 * (rho, rho u, rho v, rho w, rho E | T, P, u, v, w), ucs/compressible.tcc:11-22.
 * The state set also becomes q_old, the start-of-step state of the temporal
 * residual (SolutionSpace::Init copies q into qold, ucs/solutionSpace.tcc:279). */
PCFD_API int pcfd_set_state(pcfd_solver_t s, const double* q, int nvars, int nrows);
/* q_old alone (SolutionField STATE_N of the state, ucs/solutionField.tcc:203):
 * the first 5 values of the first nnode rows of q, rows of nvars = 10 or 5
 * values.  pcfd_newton_step sets it itself at the start of each step. */
PCFD_API int pcfd_set_qold(pcfd_solver_t s, const double* q, int nvars, int nrows);
PCFD_API int pcfd_get_state(pcfd_solver_t s, double* q, int nvars, int nrows);
/* freestream state Qinf (10 values), CompressibleEqnSet::UpdateQinf (ucs/compressible.tcc:827) */
PCFD_API int pcfd_get_qinf(pcfd_solver_t s, double* qinf10);

/* UpdateBCs (ucs/bc.tcc:1400): phantom states and hard-set boundary nodes. */
PCFD_API int pcfd_update_bcs(pcfd_solver_t s);
/* Gradient<T>::Compute (ucs/gradient.tcc:57), weighted LSQ; qgrad_out
 * optional [nnode][9][3] in the reference layout. */
PCFD_API int pcfd_gradient(pcfd_solver_t s, double* qgrad_out);
/* Limiter<T>::Compute (ucs/limiters.tcc:53); l_out optional [nnode][5]. */
PCFD_API int pcfd_limiter(pcfd_solver_t s, double* l_out);
/* The limiter values the next residual uses, [nnode][5] (Limiter<T>::l,
 * ucs/limiters.h), without recomputing them. */
PCFD_API int pcfd_get_limiter(pcfd_solver_t s, double* l_out);
/* Installs limiter values [nnode][5] as final (no pressure-clip pass); with
 * pcfd_newton_opts.limiter_freeze they stay fixed. */
PCFD_API int pcfd_set_limiter(pcfd_solver_t s, const double* l);
/* ComputeResiduals (ucs/residual.tcc:13): b (= -R) into b_out [nnode][5]
 * (optional) and norms_out[0..5] = {resGlobal, per-equation norms}. */
PCFD_API int pcfd_residual(pcfd_solver_t s, double* b_out, double* norms_out);
/* Forces::ComputeYpCf -> FORCE_Kernel (ucs/forces.tcc:124-197,376-408) on the
 * body made of the given boundary tags (a composite body of the .bc file):
 * out6[0..2] pressure force sum p |a| n, out6[3..5] viscous force on its
 * no-slip half-edges (the stress of ComputeStressVector, ucs/compressible.tcc:
 * 1113, which reads the gradients of the momentum components).  Uses the
 * current state and the last FP64 gradient (computed here first when there is
 * none).  Summed in a fixed order; moments are not formed. */
PCFD_API int pcfd_forces(pcfd_solver_t s, const int* tags, int ntags, double* out6);
/* b (= -R) of the last residual evaluation, [nnode][5], without recomputing. */
PCFD_API int pcfd_get_residual(pcfd_solver_t s, double* b_out);
/* UpdateBCs + gradient + limiter + residual in one call, the sequence
 * NewtonIterate runs (ucs/solutionSpace.tcc:662-697), without copying fields
 * back; norms_out as for pcfd_residual. */
PCFD_API int pcfd_residual_full(pcfd_solver_t s, double* norms_out);

/* ComputeTimesteps (ucs/timestep.tcc:7), local time stepping: dt_i = CFL
 * vol_i / sum(max eigenvalue * area).  dt_out [nnode] and dtmin optional. */
PCFD_API int pcfd_timestep(pcfd_solver_t s, double cfl, double* dt_out, double* dtmin);
/* Storage precision of the off-diagonal Jacobian blocks: 0 FP64, 1 FP32,
 * 2 BF16 (FP64 accumulation in every product; the diagonal stays FP64).
 * The reference stores everything in FP64 (CRSMatrix<T>, ucs/crsmatrix.h:10). */
PCFD_API int pcfd_set_jacobian_precision(pcfd_solver_t s, int precision);
/* ComputeJacobians (ucs/jacobian.tcc:13): finite-difference Roe blocks
 * (Kernel_NumJac :254, Bkernel_NumJac :459), analytic viscous blocks
 * (:734), diagonal column sums (:437), vol/dtau with the last time step
 * (ContributeTemporalTerms :214), no-slip row changes (ucs/bc.tcc:748), and
 * the diagonal LU of CRSMatrix::PrepareSGS (ucs/crsmatrix.tcc:840).  Applies
 * the boundary conditions to the state first, as the reference's boundary
 * kernel does. */
PCFD_API int pcfd_jacobian(pcfd_solver_t s);
/* The assembled matrix in the reference layout: blocks [nblocks][5][5],
 * row-major, diagonal first in each row (before its LU). */
PCFD_API int pcfd_get_jacobian(pcfd_solver_t s, double* blocks, long long nblocks);
PCFD_API long long pcfd_nblocks(pcfd_solver_t s);
/* CRS row pointers ia [nnode+1], column ids ja [nblocks] and the number of
 * colours of the Gauss-Seidel sweeps; any pointer may be null. */
PCFD_API int pcfd_crs_structure(pcfd_solver_t s, int* ia, int* ja, int* ncolor);
/* The colouring of the Gauss-Seidel sweeps: rows of colour c are
 * rows[color_ptr[c] .. color_ptr[c+1]); color_ptr has ncolor+1 entries, rows
 * nnode.  No reference counterpart (the reference sweeps rows in order). */
PCFD_API int pcfd_coloring(pcfd_solver_t s, int* color_ptr, int* rows);
/* CRS::SGS (ucs/crs.tcc:62) with x = 0 and b = the last residual: nsweeps
 * multicolour symmetric block Gauss-Seidel sweeps.  x_out [nnode][5] and
 * dnorm (|norm change of x over the last sweep|, the reference's return
 * value) optional. */
PCFD_API int pcfd_sgs(pcfd_solver_t s, int nsweeps, double* x_out, double* dnorm);
/* CRS<T>::GMRES's role (ucs/crs.tcc:176) for the Newton system: restarted
 * flexible GMRES, right-preconditioned by nsgs block-SGS sweeps (>= 1), on
 * the assembled matrix (pcfd_jacobian) with the residual of the last
 * residual call as the right-hand side, from x = 0: m directions per restart
 * (1..60), at most `restarts` restarts, until the relative residual falls
 * below rtol.  x_out (optional) [nnode][5]; *relres (optional) the final
 * relative residual estimate, *iters (optional) the Krylov iterations.  The
 * Krylov vectors are FP32 when the matrix is stored in FP32 or BF16, FP64
 * otherwise; x accumulates in FP64.  PCFD_ERR_STATE before a Jacobian. */
PCFD_API int pcfd_fgmres(pcfd_solver_t s, int m, int restarts, double rtol, int nsgs, double* x_out, double* relres,
                         int* iters);
/* CRSMatrix::MatVecMultiply (ucs/crs.tcc:484): y = A x with the assembled
 * matrix, x and y host arrays [nnode][5].  vec_precision 0 multiplies FP64
 * vectors (the FGMRES solver of an FP64 system); 1 FP32 vectors (the FP32
 * Krylov solver, FP32 or BF16 matrix storage only), returned widened. */
PCFD_API int pcfd_matvec(pcfd_solver_t s, const double* x, double* y, int vec_precision);
/* CRS::SGS (ucs/crs.tcc:62) with x = 0 and the right-hand side b (host,
 * [nnode][5]): nsweeps sweeps into x_out.  vec_precision as pcfd_matvec:
 * 1 runs the FP32 Krylov solver's preconditioner sweep. */
PCFD_API int pcfd_sgs_rhs(pcfd_solver_t s, int nsweeps, const double* b, double* x_out, int vec_precision);
/* NaN/Inf zeroing and CompressibleEqnSet::ApplyDQ (ucs/compressible.tcc:929)
 * of x (x_in [nnode][5] if given, else the last linear solution); dqnorm =
 * ParallelL2Norm of x (ucs/solutionSpace.tcc:817). */
PCFD_API int pcfd_apply_dq(pcfd_solver_t s, const double* x_in, double* dqnorm);

typedef struct pcfd_newton_opts {
  int iter;             /* SolutionSpace::iter: the reference's counter, 0 on the first step
                         * (which is therefore first order, ucs/solutionSpace.tcc:663,671) */
  double cfl;           /* Param::cfl */
  double cfl_start;     /* Param::cflStart (ramp start; <= 0: no ramp) */
  int cfl_ramp_steps;   /* Param::cflRampingSteps */
  int nsgs;             /* Param::nSgs: SGS sweeps, or FGMRES preconditioner sweeps */
  int jac_update_freq;  /* Param::jacobianFreq */
  int jac_precision;    /* 0 FP64, 1 FP32, 2 BF16 off-diagonal storage */
  int linear_solver;    /* 0 block SGS (the reference's), 1 FGMRES preconditioned by SGS,
                           2 FGMRES preconditioned by SGS plus the learned correction
                           (pcfd_lp_*), with plain SGS-preconditioned FGMRES as the fallback,
                           3 FGMRES preconditioned by SGS whose second direction in each cycle
                           is the learned vector of the cycle's residual direction (the space
                           holds plain SGS's first direction too, so no fallback) */
  int fgmres_m;         /* Krylov dimension per restart (FGMRES) */
  int fgmres_restarts;  /* restarts (FGMRES) */
  double fgmres_rtol;   /* relative tolerance (FGMRES) */
  int limiter_refresh;  /* Param::limiterRefresh: recompute the limiter every n iterations (<= 0: 1) */
  int limiter_freeze;   /* Param::limiterFreeze: keep the limiter fixed from this iteration on (<= 0: never) */
  int first_order_steps;/* Param::nFirstOrderSteps: first-order fluxes up to this iteration */
  int lp_directions;    /* linear_solver 2: the learned correction applies to the first lp_directions
                           Krylov directions of each cycle, plain SGS to the rest (<= 0: all) */
} pcfd_newton_opts;

typedef struct pcfd_newton_report {
  double res[6];  /* resGlobal and per-equation residual norms before the update */
  double dqnorm;  /* update norm */
  double dtmin;   /* smallest local time step */
  double lin_res; /* SGS: norm change of the last sweep; FGMRES: final relative residual */
  int lin_iters;  /* sweeps or Krylov iterations */
  double cfl;     /* CFL used */
  int lp_fallbacks; /* linear_solver 2: restarts that fell back to SGS-only preconditioning */
} pcfd_newton_report;

/* One outer iteration in the reference's order: PreTimeAdvance (Jacobian,
 * time step; ucs/solutionSpace.tcc:573) then NewtonIterate (:640: boundary
 * conditions, gradient, limiter, residual, linear solve, update). */
PCFD_API int pcfd_newton_step(pcfd_solver_t s, const pcfd_newton_opts* opts, pcfd_newton_report* report);

/* ---- learned right preconditioner -------------------------------------
 * No reference counterpart: it sits where CRS<T>::PrecondBackSolve sits
 * (ucs/crs.tcc:591).  For a Krylov vector v the preconditioner returns
 *   z = y + sigma * N(x),   y = nsgs block-SGS sweeps on v,
 *   sigma = RMS of y over all nodes and equations,
 * where N is an edge message-passing network applied to the node features x
 * (PCFD_LP_NIN per node: y/sigma (5), the state as rho/rho_inf - 1,
 * u/c_inf, v/c_inf, w/c_inf, p/p_inf - 1 (5), log(vol/mean vol) (1)) and
 * the edge features (unit face normal oriented away from the node (3), edge
 * length / mean edge length (1)).  Network: encoder 11 -> 64 (ReLU); three
 * layers h' = ReLU(Ws h + Wm m + b) with m_i = (1/deg_i) sum_j
 * (We e_ij + ce) * h_j (channel-wise gate); decoder 64 -> 5.  Matrices are
 * BF16, biases and accumulation FP32; the 64x128 layer products run on the
 * tensor cores.  Parameters are one FP32 array of PCFD_LP_NPARAM values in
 * the order: Win[64][11], bin[64], then per layer We[64][4], ce[64],
 * Ws[64][64], Wm[64][64], b[64], then Wout[5][64], bout[5]. */
#define PCFD_LP_NIN 11
#define PCFD_LP_HIDDEN 64
#define PCFD_LP_NEDGE 4
#define PCFD_LP_NOUT 5
#define PCFD_LP_LAYERS 3
#define PCFD_LP_NPARAM 26821

/* Allocates the network on the handle with seeded initial parameters
 * (decoder zero, so the preconditioner starts as plain SGS). */
PCFD_API int pcfd_lp_init(pcfd_solver_t s, unsigned long long seed);
PCFD_API int pcfd_lp_get_params(pcfd_solver_t s, float* params);
PCFD_API int pcfd_lp_set_params(pcfd_solver_t s, const float* params);
/* Network output for host features x [nnode][PCFD_LP_NIN] -> out [nnode][5]. */
PCFD_API int pcfd_lp_forward(pcfd_solver_t s, const float* x, float* out);
/* Loss sum((out - t)^2) / (5 nnode) and its gradient with respect to the
 * parameters, for host features x and targets t [nnode][5]. */
PCFD_API int pcfd_lp_loss_grad(pcfd_solver_t s, const float* x, const float* t, float* grad, double* loss);
/* Node features of a base-preconditioned vector y [nnode][5] (host) with
 * the handle's current state; sigma_out receives sigma. */
PCFD_API int pcfd_lp_features(pcfd_solver_t s, const double* y, float* x, double* sigma_out);
/* Training pairs from the current linear system (the Jacobian and residual
 * of the last pcfd_newton_step), stored on the device as the features of
 * y = SGS(r) and the target (x - y)/sigma for pairs (r, x) with A x = r:
 * (b, dq) with dq solved to the relative tolerance rtol by SGS-preconditioned
 * FGMRES(30), and, for the first krylov_pairs directions z_j of that solve,
 * (A z_j, z_j) - exact pairs drawn from the vectors the Krylov solver itself
 * preconditions. */
PCFD_API int pcfd_lp_collect(pcfd_solver_t s, int nsgs, double rtol, int krylov_pairs, int* nsamples_out);
PCFD_API int pcfd_lp_clear_samples(pcfd_solver_t s);
/* Adam over the stored pairs (one pair per step, epochs passes).
 * loss_first/loss_last: mean loss of the first and last pass. */
PCFD_API int pcfd_lp_train(pcfd_solver_t s, int epochs, double lr, double* loss_first, double* loss_last);
/* Applies the preconditioner to v [nnode][5] (host) -> z (host). */
PCFD_API int pcfd_lp_apply(pcfd_solver_t s, int nsgs, const double* v, double* z);

/* ---- finite-rate chemistry (reacting air) ------------------------------
 * Mass production rates of a finite-rate mechanism per node, the per-node
 * chemistry of the reacting equation set: ChemModel<T>::
 * GetMassProductionRates (ucs/chem.tcc:575) with Reaction<T>::
 * GetForwardReactionRate / GetEquilibriumReactionRate /
 * GetBackwardReactionRate / GetMassProductionRate (ucs/reaction.tcc:608,
 * 629,683,763) and the NASA-7 curve selection of Species<T>::GetThermoCoeff
 * (ucs/species.tcc:96).  Backward rates come from the equilibrium constant
 * of the Gibbs energies.  Units are the reference's: densities kg/m^3,
 * temperature K, rates kg/(m^3 s), molecular weights kg/mol, EA as each
 * rate form expects it (J/mol, or K for the Gupta form). */
#define PCFD_CHEM_MAX_SPECIES 16
#define PCFD_CHEM_MAX_REACTIONS 32
#define PCFD_CHEM_MAX_LOCAL 16
#define PCFD_CHEM_MAX_TRANSPORT_FITS 4

typedef struct pcfd_chem_reaction {
  int type;          /* Reaction::rxnType: 0 Arrhenius, 1 ModArrhenius, 2 GuptaModArrhenius, 3 Power */
  double A, EA, n;   /* forward-rate coefficients (SI) */
  int third_bodies;  /* thirdBodiesPresent */
  int nlocal;        /* the reaction's species: reactants, products, then listed third bodies */
  int global[PCFD_CHEM_MAX_LOCAL];      /* index in the model's species list */
  double nup[PCFD_CHEM_MAX_LOCAL];      /* Nup: reactant stoichiometric coefficients */
  double nupp[PCFD_CHEM_MAX_LOCAL];     /* Nupp: product stoichiometric coefficients */
  double tbeff[PCFD_CHEM_MAX_LOCAL];    /* TBEff: third-body efficiencies */
} pcfd_chem_reaction;

typedef struct pcfd_chem_model {
  int nspecies;
  double mw[PCFD_CHEM_MAX_SPECIES];          /* Species::MW, kg/mol */
  double nasa_lo[PCFD_CHEM_MAX_SPECIES][7];  /* NASA-7 coefficients used up to 1000 K (and below 200 K) */
  double nasa_hi[PCFD_CHEM_MAX_SPECIES][7];  /* above 1000 K (and above 6000 K) */
  int nreactions;
  pcfd_chem_reaction rx[PCFD_CHEM_MAX_REACTIONS];
  /* transport (Species::GetViscosity / GetThermalConductivity,
   * ucs/species.tcc:393,430): NASA RP-1311 fits ln(y) = A ln T + B/T + C/T^2 + D,
   * rows {T_lo, T_hi, A, B, C, D}, viscosity in micropoise, conductivity in
   * microwatt/(cm K); the last row whose range holds T is used.  At or below
   * 1000 K every species takes White's Sutherland forms instead, as the
   * reference does.  nmu/nk = 0: no transport data (the viscous flux is then
   * refused). */
  int nmu[PCFD_CHEM_MAX_SPECIES];
  double mu_fit[PCFD_CHEM_MAX_SPECIES][PCFD_CHEM_MAX_TRANSPORT_FITS][6];
  int nk[PCFD_CHEM_MAX_SPECIES];
  double k_fit[PCFD_CHEM_MAX_SPECIES][PCFD_CHEM_MAX_TRANSPORT_FITS][6];
} pcfd_chem_model;

typedef struct pcfd_chem_s* pcfd_chem_t;

PCFD_API int pcfd_chem_create(const pcfd_chem_model* model, pcfd_chem_t* out);
PCFD_API int pcfd_chem_destroy(pcfd_chem_t c);
/* host arrays: rhoi [n][nspecies], T [n], wdot [n][nspecies] */
PCFD_API int pcfd_chem_production_rates(pcfd_chem_t c, long long n, const double* rhoi, const double* T, double* wdot);
/* the same on device arrays, on the handle's stream; ms_out (optional)
 * receives the kernel's device time */
PCFD_API int pcfd_chem_production_rates_dev(pcfd_chem_t c, long long n, const double* rhoi, const double* T,
                                            double* wdot, double* ms_out);

/* Node state of the reacting equation set (CompressibleFREqnSet, ideal-gas
 * mixture, Dalton's law).  Variables are non-dimensional as in the reference,
 * with these scales (Param::ref_*, ucs/param.tcc:372-397). */
typedef struct {
  double density, pressure, temperature, specific_enthalpy, velocity;
  /* Param::ref_viscosity and ref_k (inputs refViscosity, refThermalConductivity,
   * ucs/param.tcc:210-211; default 1, and 0 here reads as 1) */
  double viscosity, conductivity;
} pcfd_chem_ref;
/* With dev = 0 the arrays are host arrays (copied through the handle's
 * buffers); with dev = 1 they are device arrays, used in place on the
 * handle's stream.  Per node, ns = the model's species count. */
/* NewtonFindTGivenP (ucs/compressibleFR.tcc:2343): rhoi [n][ns], P [n],
 * T_init [n] -> T [n]; *nonconverged (optional) counts nodes that used all 28
 * iterations (the reference warns). */
PCFD_API int pcfd_chem_find_T_given_P(pcfd_chem_t c, const pcfd_chem_ref* ref, long long n, const double* rhoi,
                                      const double* P, const double* T_init, double* T, long long* nonconverged,
                                      int dev);
/* GetMolecularViscosity / GetThermalConductivity (ucs/compressibleFR.tcc:
 * 1580,1590): the mixture's viscosity and conductivity by Wilke's rule
 * (ChemModel::WilkesMixtureRule, ucs/chem.tcc:876) from non-dimensional
 * rhoi [n][ns] and T [n], returned non-dimensional (over ref->viscosity and
 * ref->conductivity).  A temperature above every fit's range returns
 * PCFD_ERR_ARG (the reference aborts). */
PCFD_API int pcfd_chem_transport(pcfd_chem_t c, const pcfd_chem_ref* ref, long long n, const double* rhoi,
                                 const double* T, double* mu, double* k, int dev);
/* ConservativeToNative (:2133): the FP64 temperature Newton from total
 * energy.  q [n][ns+4] = (rhoi, rho u, rho v, rho w, rho Et), P [n] the
 * stored pressure (initial guess) -> native [n][4] = (u, v, w, T).  Returns
 * PCFD_ERR_NUMERIC when a node needs more than 20 iterations (the reference
 * aborts). */
PCFD_API int pcfd_chem_conservative_to_native(pcfd_chem_t c, const pcfd_chem_ref* ref, long long n, const double* q,
                                              const double* P, double* native, int dev);
/* NativeToConservative (:2117) with GetTotalEnergy (:1219): rhoi [n][ns],
 * native [n][4] = (u, v, w, T), P [n] -> q [n][4] = (rho u, rho v, rho w,
 * rho Et). */
PCFD_API int pcfd_chem_native_to_conservative(pcfd_chem_t c, const pcfd_chem_ref* ref, long long n, const double* rhoi,
                                              const double* native, const double* P, double* q, int dev);
/* ComputeAuxiliaryVariables (:755): rhoi [n][ns], T [n] -> P [n], cvi
 * [n][ns], concentrations [n][ns] (ChemModel::MassToMole, ucs/chem.tcc:980). */
PCFD_API int pcfd_chem_aux(pcfd_chem_t c, const pcfd_chem_ref* ref, long long n, const double* rhoi, const double* T,
                           double* P, double* cvi, double* mol, int dev);
/* Options of the reacting inviscid flux: beta of the eigenvalue
 * modification (1 = none; Gupta's low-Mach form otherwise), the reference
 * gauge pressure Pref (GetPressure(Qinf), ucs/compressibleFR.tcc:1517) and
 * Param::symmetry2D (0 off, 1..3 zero the x, y or z momentum flux). */
typedef struct {
  double beta, pref;
  int symmetry2D;
} pcfd_chem_flux_opts;
/* EqnSet::SourceTermJacobian (ucs/eqnset.tcc:163) of the reacting set as
 * the Jacobian assembly takes it (ucs/jacobian.tcc:201, which subtracts it
 * from the diagonal block): q [n][6 + 3 ns] node records (rhoi and T read),
 * vol [n] dual volumes -> A [n][(ns + 4)^2] row-major, A[j (ns + 4) + i] =
 * (S_j(Q + h e_i) - S_j(Q)) / h with h = 1e-8 on the non-dimensional native
 * value i, S = SourceTerm (ucs/compressibleFR.tcc:1276, reactions on) =
 * vol * wdot / (ref_density / ref_time) in the species rows, zero in the
 * momentum and energy rows.  dev as above (q, vol, A). */
PCFD_API int pcfd_chem_source_jacobian(pcfd_chem_t c, const pcfd_chem_ref* ref, double ref_time, long long n,
                                       const double* q, const double* vol, double* A, int dev);
/* CompressibleFREqnSet::ContributeTemporalTerms (ucs/compressibleFR.tcc:1319)
 * as ComputeJacobians' temporal loop calls it per node (ucs/jacobian.tcc:214):
 * q [n][6 + 3 ns] node records, vol [n], dtau [n] (pseudo-time steps), beta
 * [n] (Gupta's preconditioning parameter), cnp1 (1, or 1.5 for second order
 * in time), dt (the real time step, read when local_ts != 0) -> A [n][(ns +
 * 4)^2] row-major diagonal blocks, IN AND OUT: the temporal terms (vol/dt
 * times dq/dQ, conservative over native, with the beta terms in the
 * temperature column) are added to what A holds.  dev as above. */
PCFD_API int pcfd_chem_temporal_terms(pcfd_chem_t c, const pcfd_chem_ref* ref, long long n, const double* q,
                                      const double* vol, const double* dtau, const double* beta, double cnp1,
                                      double dt, int local_ts, double* A, int dev);
/* CompressibleFREqnSet::HLLCFlux (ucs/compressibleFR.tcc:301; RoeFlux
 * forwards to it, :293) on a static grid: q [nnode][6 + 3 ns] node records
 * (rhoi, u, v, w, T | P, rho, cvi, concentrations, as ComputeAuxiliaryVariables
 * leaves them), edges [nedge][2] (left, right), avec [nedge][4] (unit normal,
 * area) -> flux [nedge][ns + 4] out of the left node.  *nfail (optional)
 * counts edges whose wave speeds left no HLLC branch (the reference's soft
 * abort); their flux is zero and the call returns PCFD_ERR_NUMERIC. */
PCFD_API int pcfd_chem_hllc_flux(pcfd_chem_t c, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o, long long nnode,
                                 const double* q, long long nedge, const int* edges, const double* avec, double* flux,
                                 long long* nfail, int dev);
/* Attaches a mesh (pcfd_mesh_view as for pcfd_create) to the chemistry
 * handle for pcfd_chem_residual: edges, areas, boundary half-edges, dual
 * volumes and the node -> edge lists are copied to HBM once. */
PCFD_API int pcfd_chem_attach_mesh(pcfd_chem_t c, const pcfd_mesh_view* m);
/* SpatialResidual (ucs/residual.tcc:66) of the reacting equation set, first
 * order and inviscid, on the attached mesh: q [nnode + nbedge][6 + 3 ns]
 * records, the phantom records after the nodes as the boundary conditions
 * leave them -> b [nnode][ns + 4] (optional) = -sum of the HLLC fluxes out of
 * each node (edges in ascending id, then boundary half-edges) + vol * wdot
 * (SourceTerm, ucs/compressibleFR.tcc:1276, when reactions != 0; wdot made
 * non-dimensional by ref_density / ref_time), and norms [1 + ns + 4]
 * (optional; ParallelL2Norm and StridedParallelL2Norm).  dev as above (q, b). */
PCFD_API int pcfd_chem_residual(pcfd_chem_t c, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o,
                                double ref_time, int reactions, const double* q, double* b, double* norms, int dev);
/* The same residual at second order (Kernel_Inviscid_Flux past the
 * first-order steps, ucs/residual.tcc:192): each edge's records extrapolated
 * to the midpoint by ExtrapolateVariables (ucs/compressibleFR.tcc:734),
 * q + lim (chi/2 dQ + (1 - chi) grad.dx) on rhoi, u, v, w, T, their pressure
 * and density recomputed, then HLLC; boundary half-edges stay first order
 * (one partition).  grad [nnode][2 ns + 4][3] as pcfd_chem_gradient forms
 * it, lim [nnode][ns + 4] the limiter (ones: unlimited).  Needs the attached
 * mesh's coordinates.  dev as above (q, grad, lim, b). */
PCFD_API int pcfd_chem_residual_ho(pcfd_chem_t c, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o, double chi,
                                   double ref_time, int reactions, const double* q, const double* grad,
                                   const double* lim, double* b, double* norms, int dev);
/* Limiter<T>::Compute with the modified Venkatakrishnan kernel (limiter 3,
 * ucs/limiters.tcc:53,534; K = 1 as the reference hard-codes it) on the
 * reacting set's native variables rhoi, u, v, w, T over the attached mesh
 * (with coordinates): neighbour bounds from 0, each incident edge's
 * unlimited extrapolation, the minimum, negatives clamped to 0.  The
 * pressure clip (Kernel_PressureClip, :737) is not applied.  q, grad as for
 * pcfd_chem_residual_ho -> lim [nnode][ns + 4].  dev as above. */
PCFD_API int pcfd_chem_limiter(pcfd_chem_t c, double chi, const double* q, const double* grad, double* lim, int dev);
/* UpdateBCs (ucs/bc.tcc:1400) of the reacting set on the attached mesh (which
 * must carry face tags), in place on q (as for pcfd_chem_residual): each
 * half-edge in order through CalculateBoundaryVariables (:1059), then
 * ComputeAuxiliaryVariables of its phantom and node.  Built types, per face
 * tag (bc_type, twall and qref have ntags entries): sonic inflow / Dirichlet
 * (node and phantom take qref[tag], a full record), sonic outflow / Neumann,
 * the isothermal no-slip wall at rest (twall[tag] > 0 K;
 * GetViscousWallBoundaryVariables, ucs/compressibleFR.tcc:2049) and, with
 * no_cvbc = 1, the impermeable wall and symmetry plane
 * (GetInviscidWallBoundaryVariables' mirror, :1042).  Any other type (far
 * field, the characteristic wall, the adiabatic no-slip wall) returns
 * PCFD_ERR_ARG and leaves its half-edges as they were.  dev as above (q). */
PCFD_API int pcfd_chem_update_bcs(pcfd_chem_t c, const pcfd_chem_ref* ref, int ntags, const int* bc_type,
                                  const double* twall, const double* qref, int no_cvbc, double* q, int dev);
/* Gradient<T>::Compute of the reacting set on the attached mesh (which must
 * carry coordinates and LSQ matrices): the weighted least-squares gradient
 * (Kernel_LSQ_Gradient, ucs/gradient.tcc:251) of the gradient list rhoi, u,
 * v, w, T, concentrations (GetGradientsLocation, ucs/compressibleFR.tcc:693)
 * over the interior edges, then Bkernel_Symmetry_Fix (:545) on the
 * half-edges whose tag is one of sym_tags (at most 8).  q as for
 * pcfd_chem_residual -> grad [nnode][2 ns + 4][3].  dev as above (q, grad). */
PCFD_API int pcfd_chem_gradient(pcfd_chem_t c, const double* q, const int* sym_tags, int nsym, double* grad, int dev);
/* The viscous part of the reacting residual on the attached mesh:
 * Kernel_Viscous_Flux and Bkernel_Viscous_Flux (ucs/residual.tcc:390,473)
 * with CompressibleFREqnSet::ViscousFlux (ucs/compressibleFR.tcc:551), laminar,
 * no species diffusion, mixture viscosity and conductivity as
 * pcfd_chem_transport forms them.  q as for pcfd_chem_residual; grad
 * [nnode][2 ns + 4][3] the node gradients of the reacting gradient list
 * (rhoi, u, v, w, T, concentrations; GetGradientsLocation, :693); Re
 * Param::Re; directional: 1 for the directional correction of the face
 * gradient along each edge (second order past the first-order steps), which
 * needs the attached mesh's coordinates.  b [nnode][ns + 4] receives the
 * viscous contributions alone, summed per node in ascending edge order then
 * half-edges; the caller adds them to pcfd_chem_residual's.  A face above
 * every transport fit's range returns PCFD_ERR_ARG.  dev as above (q, grad, b). */
PCFD_API int pcfd_chem_viscous_residual(pcfd_chem_t c, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o,
                                        double Re, int directional, const double* q, const double* grad, double* b,
                                        int dev);

/* Arithmetic of the composite residual calls (pcfd_residual_full,
 * pcfd_bench_residual_full, pcfd_newton_step): 0 FP64 (default), 1
 * double-float - the same kernels with every FP64 operation replaced by a
 * pair of FP32 numbers (about 48 significant bits), which GB300 executes on
 * its FP32 pipes at many times its FP64 rate.  The state, b and the norms
 * stay FP64.  Mode 1 also evaluates the interior fluxes of the
 * finite-difference Jacobian in double-float (about 1e-6 relative error in
 * its coefficients).  The single-stage calls (pcfd_gradient, pcfd_limiter,
 * pcfd_residual) always use FP64.  No reference counterpart. */
PCFD_API int pcfd_set_residual_arithmetic(pcfd_solver_t s, int mode);

/* Runs nsteps of pcfd_residual_full back to back on the handle's stream and
 * returns their device time from CUDA events recorded on that stream (the
 * reference's ResidualTimer, ucs/solutionSpace.tcc:692-701). */
PCFD_API int pcfd_bench_residual_full(pcfd_solver_t s, int nsteps, double* ms_out, double* norms_out);
/* Device time (CUDA events on the library's stream) of nrep back-to-back
 * products y = A x of the assembled matrix (MatVecMultiply, ucs/crs.tcc:484)
 * on device-resident vectors: FP64 vectors with vec_precision 0, the FP32
 * Krylov solver's product with 1 (FP32 or BF16 storage). */
PCFD_API int pcfd_bench_spmv(pcfd_solver_t s, int nrep, int vec_precision, double* ms_out);
/* Device time (CUDA events on the library's stream) of nrep calls of nsweeps
 * block-SGS sweeps (CRS<T>::SGS, ucs/crs.tcc:62) on the assembled matrix,
 * right-hand side the last residual, device-resident vectors: FP64 vectors
 * with vec_precision 0 (the matrix in its stored precision), the FP32 Krylov
 * preconditioner's sweep with 1 (FP32 or BF16 storage). */
PCFD_API int pcfd_bench_sgs(pcfd_solver_t s, int nrep, int nsweeps, int vec_precision, double* ms_out);
/* Selects the CUDA device for handles created afterwards on this thread. */
PCFD_API int pcfd_set_device(int device);
/* Waits for all work on the current device. */
PCFD_API int pcfd_device_sync(void);

/* Per-kernel device time accumulated since the last reset, in the spirit of
 * the reference's TimerList (ucs/timer.h:29).  Timing uses CUDA events on the
 * handle's stream and is off unless enabled. */
PCFD_API int pcfd_profile_enable(pcfd_solver_t s, int on);
PCFD_API int pcfd_profile_reset(pcfd_solver_t s);
/* name_buf receives the i-th timer's name; returns PCFD_ERR_ARG past the end */
PCFD_API int pcfd_profile_get(pcfd_solver_t s, int i, char* name_buf, int name_len, double* ms_total,
                              long long* launches);
/* number of kernel launches issued by the library on this handle */
PCFD_API long long pcfd_launch_count(pcfd_solver_t s);

/* Health word the device kernels maintain (NaN fluxes kneecapped, clips,
 * ...), replacing the reference's warnings/soft aborts (ucs/eqnset.tcc:73-88,
 * ucs/exceptions.h:51-63).  counters[0..7]. */
PCFD_API int pcfd_get_health(pcfd_solver_t s, long long* counters8);

/* Residual norms of a caller-provided device array, with no device
 * allocation at all - for callers that cannot let a library allocate GPU
 * memory: applications that hand out every byte from their own pool or fixed
 * per-tenant budget, or solver loops that must not allocate once running.
 * This entry point has no counterpart in the reference.
 * b: device pointer to [nnode][5] doubles; norms: device pointer to 6
 * doubles, written as pcfd_residual's norms_out (resGlobal, then the five
 * per-equation norms); stream: a cudaStream_t of the current device, or null
 * for the default stream (another device's stream returns PCFD_ERR_ARG).  The
 * call synchronizes the stream before it returns, so it cannot be part of a
 * CUDA graph: on a capturing stream it returns PCFD_ERR_ARG and enqueues
 * nothing.  The only scratch is one fixed array inside the library (768 KiB
 * per GPU, held until the process exits), which limits nnode to 33,554,432;
 * larger inputs return PCFD_ERR_ARG.  All calls share the array: calls that
 * overlap on the GPU race on it and must be serialised by the caller. */
PCFD_API int pcfd_residual_norms_noalloc(const double* b, long long nnode, double* norms, void* stream);

PCFD_API const char* pcfd_last_error(void);
PCFD_API const char* pcfd_build_info(void);

#ifdef __cplusplus
}
#endif

#endif /* PCFD_H_ */
