/*
 * ORACLE — test infrastructure, not the product.  See sdfc_oracle.c.
 */
#ifndef SDFC_ORACLE_H
#define SDFC_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

/* An SDF grid as BodySDFObj holds it (simulation/redmax/Body/BodySDFObj.h:13-16). */
typedef struct {
    int ni, nj, nk;
    double min_box[3], max_box[3];
    double dx[3];   /* _dx, _dy, _dz */
    double col_th;  /* _col_th, added to every distance */
    const double* v; /* ni*nj*nk values, i fastest */
} orc_grid;

/* ForceGeneralSDFContact coefficients (simulation/redmax/Force/ForceGeneralSDFContact.h:16-20)
 * plus the contact body's _contact_scale. */
typedef struct {
    double kn, kt, mu, damping, scale, contact_scale;
} orc_params;

/* Layout of orc_collision's output (row-major blocks). */
enum {
    ORC_COLLISION_VALUE = 11, /* d, n[3], ddot, tdot[3], xi2[3] */
    ORC_C_DD_DXW = 11,
    ORC_C_DD_DQ2 = 14,
    ORC_C_DN_DXW = 20,
    ORC_C_DN_DQ2 = 29,
    ORC_C_DDDOT_DXW = 47,
    ORC_C_DDDOT_DXWDOT = 50,
    ORC_C_DDDOT_DQ2 = 53,
    ORC_C_DDDOT_DPHI2 = 59,
    ORC_C_DTDOT_DXW = 65,
    ORC_C_DTDOT_DXWDOT = 74,
    ORC_C_DTDOT_DQ2 = 83,
    ORC_C_DTDOT_DPHI2 = 101,
    ORC_C_DXI2_DXW = 119,
    ORC_C_DXI2_DQ2 = 128,
    ORC_COLLISION_DERIV = 146
};

double orc_query_sdf(const orc_grid* g, const double* x, int outside_accurate);
void orc_query_dsdf(const orc_grid* g, const double* x, double* v);
void orc_query_ddsdf(const orc_grid* g, const double* x, double* H);
double orc_distance(const orc_grid* g, const double* E_B, const double* xw);
void orc_collision(const orc_grid* g, const double* E_B, const double* phi_B, const double* xw,
                   const double* xw_dot, int want_deriv, double* out);
int orc_detect(const orc_grid* g, const double* E_A, const double* E_B, const double* pts, int n, int* ids,
               double* dist_out);
int orc_pair_eval(const orc_grid* g, const double* pts, int n_pts, const double* E_A, const double* phi_A,
                  const double* E_B, const double* phi_B, const orc_params* prm, int want_deriv, double* fm,
                  double* Km, double* Dm, int* ids);
/* Sum over the active contacts of the norm of each contact's own 12-vector term of fm (the
 * error scale of fm where contact forces cancel); not in the reference. */
double orc_pair_force_norm_sum(const orc_grid* g, const double* pts, int n_pts, const double* E_A,
                               const double* phi_A, const double* E_B, const double* phi_B, const orc_params* prm);

/* Penetration energy of a pair (sum of kn d^2 / 2 over the active contacts) and its gradient
 * dE[12] wrt the twists of A then B (w, v each). */
double orc_pair_energy(const orc_grid* g, const double* pts, int n_pts, const double* E_A, const double* E_B,
                       const orc_params* prm, double* dE);

/* Simulation::get_body_distance: min over the `from` body's vertices V (n x 3, body frame) of the
 * `to` body's distance(), vertices posed as get_body_vertices computes them. */
double orc_body_distance(const orc_grid* g, const double* E_from, const double* E_to, const double* V, int n,
                         double* d_out);

/* sdfgen::make_level_set3: the signed distance grid phi (ni*nj*nk floats, i fastest) of a closed
 * triangle mesh (verts: nv x 3 floats, tris: nt x 3 indices), grid origin and spacing, exact band. */
void orc_make_level_set3(const float* verts, int nv, const unsigned* tris, int nt, const float* origin, float dx,
                         float dy, float dz, int ni, int nj, int nk, int band, float* phi);

/* ---------------------------------------------------------------- one moving body, BDF1 */

/* The moving part of the planner's scene (examples/run_joint_plan.py:140-178): one
 * body on a joint attached to the world, every other part fixed: ndof 3 = translational
 * (rm/Joint/JointTranslational.cpp), ndof 6 = free3d-exp (rm/Joint/JointFree3DExp.cpp,
 * q = (p, r) with r exponential rotation coordinates).  Fields are the reference's:
 * Body::_mass, Body::_Inertia, Joint::_E_pj_0, Body::_E_ji, Simulation option gravity and
 * timestep, Body::_f_external (world frame, torque then force), Joint::_Kr/_Dr/_q_rest. */
typedef struct {
    double mass, inertia[6], E_pj0[16], E_ji[16], gravity[3], h, f_ext[6];
    double joint_stiffness, joint_damping, q_rest[6];
    int ndof;
    double newton_tol; /* 0: the reference's 1e-8 (Simulation.cpp:1008); smaller only for
                          finite-difference checks of the adjoint, which differentiates g = 0 */
} orc_mover;

/* One ForceGeneralSDFContact of the scene: the mover against one fixed body. */
typedef struct {
    const orc_grid* grid; /* the SDF body's grid */
    const double* pts;    /* the contact body's points (n x 3, body frame) */
    int n_pts;
    int mover_is_contact; /* 1: mover's points vs the fixed body's grid; 0: the reverse */
    double E_fixed[16];   /* pose of the fixed body */
    orc_params prm;
} orc_pair;

/* Mover pose and body twist for joint state (q, qdot) (Joint::update + Body::update). */
void orc_mover_pose(const orc_mover* m, const double* q, const double* qdot, double* E0i, double* phi);
/* g and H of BDF1 at q1 (Simulation::evaluate_g[_with_derivatives]_BDF1), H may be NULL. */
void orc_bdf1_eval(const orc_mover* m, const orc_pair* pairs, int n_pairs, const double* q0, const double* qdot0,
                   const double* q1, double* g, double* H);
/* orc_bdf1_eval plus the reduced M and D = df/dqdot at q1 (either may be NULL). */
void orc_bdf1_eval_full(const orc_mover* m, const orc_pair* pairs, int n_pairs, const double* q0,
                        const double* qdot0, const double* q1, double* g, double* H, double* M, double* D);
/* One implicit-Euler step (Simulation::integration_BDF1 + newton, then the free joint's
 * reparameterisation); updates q, qdot (ndof each).  Returns 1 if Newton converged.
 * iters / evals may be NULL.  g, H, M, D above are ndof and ndof x ndof. */
int orc_bdf1_step(const orc_mover* m, const orc_pair* pairs, int n_pairs, double* q, double* qdot, int* iters,
                  int* evals);

/* Adjoint of T BDF1 steps (Simulation::backward_BDF1) from the trajectory q_his[(T+1) x ndof]
 * and qdot_0: dL/dq_0, dL/dqdot_0 and dL/df_ext[6] for dL/dq_k = df_dq[(k-1) x ndof].
 * Any output may be NULL. */
void orc_bdf1_backward(const orc_mover* m, const orc_pair* pairs, int n_pairs, const double* q_his,
                       const double* qdot0, int T, const double* df_dq, double* df_dq0, double* df_dqdot0,
                       double* df_dfext);

#ifdef __cplusplus
}
#endif
#endif
