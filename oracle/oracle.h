/*
 * CPU ORACLE - test infrastructure only (see oracle.c).  Plain-C restatement
 * of the reference's residual path used to check the CUDA implementation.
 */
#ifndef PCFD_ORACLE_H_
#define PCFD_ORACLE_H_

#include "../include/pcfd.h"

#ifdef __cplusplus
extern "C" {
#endif

void oracle_aux(double gamma, double* Q);
void oracle_qinf(const pcfd_params* prm, double* Qinf);
void oracle_init_state(const pcfd_params* prm, int nrows, double* q);
void oracle_matvec(const double* a, const double* x, double* y, int n);
void oracle_roe_flux(const double* QL, const double* QR, const double* avec, double vdotn, double gamma,
                     double* flux);
void oracle_viscous_flux(const pcfd_params* prm, const double* Q, const double* grad, const double* avec, double mut,
                         double* flux);
int oracle_normal_node(const pcfd_mesh_view* m, int node, const double* avec);
int oracle_update_bcs(const pcfd_mesh_view* m, const pcfd_params* prm, double* q);
int oracle_gradient(const pcfd_mesh_view* m, const pcfd_params* prm, const double* q, double* grad);
int oracle_limiter(const pcfd_mesh_view* m, const pcfd_params* prm, const double* q, const double* grad,
                   double* l, long long* nclip);
int oracle_residual(const pcfd_mesh_view* m, const pcfd_params* prm, const double* q, const double* grad,
                    const double* lim, double* b, double* norms, long long* nkneecap);
int oracle_residual_full(const pcfd_mesh_view* m, const pcfd_params* prm, const double* q, const double* qold,
                         const double* grad, const double* lim, double* b, double* babs, double* norms,
                         long long* nkneecap);
int oracle_residual_scaled(const pcfd_mesh_view* m, const pcfd_params* prm, const double* q, const double* grad,
                           const double* lim, double* b, double* babs, double* norms, long long* nkneecap);
int oracle_lu(double* a, int* p, int n);
void oracle_lusolve(const double* a, double* b, const int* p, double* x, int n);
void oracle_tri_area(const double* p1, const double* p2, const double* p3, double* r);
double oracle_tet_vol(const double* p1, const double* p2, const double* p3, const double* p4);

double oracle_timestep(const pcfd_mesh_view* m, const pcfd_params* prm, const double* q, double cfl, double* dt);
void oracle_crs_init(const pcfd_mesh_view* m, int* ia, int* ja);
void oracle_prepare_sgs(int nnode, const int* ia, double* M, int* pv);
int oracle_jacobian(const pcfd_mesh_view* m, const pcfd_params* prm, double* q, const double* dt, const int* ia,
                    const int* ja, double* M);
double oracle_sgs(int nnode, const int* ia, const int* ja, const double* M, const int* pv, const double* b, double* x,
                  int nsweeps);
void oracle_sgs_colored(int nnode, const int* ia, const int* ja, const double* M, const int* pv, const double* b,
                        double* x, int nsweeps, int ncolor, const int* cptr, const int* rows);
double oracle_apply_dq(const pcfd_mesh_view* m, const pcfd_params* prm, double* x, double* q);

void oracle_forces(const pcfd_mesh_view* m, const pcfd_params* prm, const double* q, const double* grad,
                   const int* in_body, double* out);

/* mesh generator and preprocessing (mesh.c) */
typedef struct oracle_mesh_s oracle_mesh;
oracle_mesh* oracle_mesh_box(const pcfd_box_params* p);
oracle_mesh* oracle_mesh_elements(int nnode, const double* xyz, int ntri, const int* tri, const int* tri_tag, int ntet,
                                  const int* tet);
int oracle_mesh_build(oracle_mesh* m);
int oracle_mesh_view(const oracle_mesh* m, pcfd_mesh_view* v);
void oracle_mesh_free(oracle_mesh* m);

/* learned preconditioner network (learned.c) */
double oracle_bf16(double v);
int oracle_lp_nparam(void);
void oracle_lp_graph(const pcfd_mesh_view* m, int* nptr, int* nbr, float* ef);
double oracle_lp_features(int nnode, const double* y, const double* q, const double* vol, const double* qinf,
                          double gamma, float* x);
void oracle_lp_forward(int n, const int* nptr, const int* nbr, const float* ef, const float* x, const float* w,
                       int emulate, double* out);
double oracle_lp_loss_grad(int n, const int* nptr, const int* nbr, const float* ef, const float* x, const float* t,
                           const float* w, int emulate, double* grad);

/* finite-rate chemistry (chem.c) */
double oracle_chem_kf(const pcfd_chem_reaction* r, double T);
double oracle_chem_kc(const pcfd_chem_model* m, const pcfd_chem_reaction* r, double T);
void oracle_chem_rates(const pcfd_chem_model* m, const double* rhoi, double T, double* wdot);
void oracle_chem_rates_n(const pcfd_chem_model* m, long long n, const double* rhoi, const double* T, double* wdot);
int oracle_chem_find_T(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* rhoi, double P, double Tinit,
                       double* T);
int oracle_chem_c2n(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* q, double P, double* native);
long long oracle_chem_c2n_n(const pcfd_chem_model* m, const pcfd_chem_ref* ref, long long n, const double* q,
                            const double* P, double* native);
void oracle_chem_n2c(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* rhoi, const double* native,
                     double P, double* q);
void oracle_chem_aux(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* rhoi, double T, double* P,
                     double* cvi, double* mol);
int oracle_chem_hllc(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o,
                     const double* QL, const double* QR, const double* avec, double* flux);
long long oracle_chem_hllc_n(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o,
                             const double* q, long long nedge, const int* edges, const double* avec, double* flux);
void oracle_chem_residual(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o,
                          const pcfd_mesh_view* mv, const double* q, double ref_time, int reactions, double* b,
                          double* norms);
void oracle_chem_source_jacobian(const pcfd_chem_model* m, const pcfd_chem_ref* ref, double ref_time,
                                 const double* Q, double vol, double* A);
void oracle_chem_source_jacobian_n(const pcfd_chem_model* m, const pcfd_chem_ref* ref, double ref_time, long long n,
                                   const double* q, const double* vol, double* A);
void oracle_chem_temporal(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* Q, double vol,
                          double cnp1, double dt, double dtau, double beta, int local_ts, double* A);
int oracle_chem_transport(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const double* rhoi, double T,
                          double* mu, double* k);
long long oracle_chem_transport_n(const pcfd_chem_model* m, const pcfd_chem_ref* ref, long long n, const double* rhoi,
                                  const double* T, double* mu, double* k);
int oracle_chem_viscous_residual(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o,
                                 const pcfd_mesh_view* mv, double Re, int directional, const double* q,
                                 const double* grad, double* b);
void oracle_lsq_coeff(const double* s, const double* dxbar, double* we);
int oracle_chem_gradient(const pcfd_chem_model* m, const pcfd_mesh_view* mv, const double* q, const int* sym_tags,
                         int nsym, double* grad);
int oracle_chem_update_bcs(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_mesh_view* mv, int ntags,
                           const int* bc_type, const double* twall, const double* qref, int no_cvbc, double* q);
void oracle_chem_residual_ho(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_chem_flux_opts* o,
                             const pcfd_mesh_view* mv, const double* q, const double* grad, const double* lim,
                             double chi, double ref_time, int reactions, double* b, double* norms);
void oracle_chem_limiter(const pcfd_chem_model* m, const pcfd_mesh_view* mv, const double* q, const double* grad,
                         double chi, double* lim);
double oracle_chem_timestep(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_mesh_view* mv,
                            const double* q, double beta, double cfl, double* dt);
void oracle_chem_limiter_clip(const pcfd_chem_model* m, const pcfd_chem_ref* ref, const pcfd_mesh_view* mv,
                              const double* q, const double* grad, double chi, double* lim);
void oracle_chem_temporal_n(const pcfd_chem_model* m, const pcfd_chem_ref* ref, long long n, const double* q,
                            const double* vol, const double* dtau, const double* beta, double cnp1, double dt,
                            int local_ts, double* A);

#ifdef __cplusplus
}
#endif

#endif
