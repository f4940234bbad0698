// extern "C" harness over the reference redmax simulator, compiled together
// with the reference's own sources by oracle/ref/Makefile.  Test
// infrastructure only: it lets the oracle tests (and the golden-fixture
// generator) run the reference's SDF contact path on injected inputs.
//
// Every entry point returns 0 on success and a negative code on failure; C++
// exceptions (the reference throws std::string) never cross the boundary.
// Matrices cross as row-major double arrays.
#include <cstring>
#include <string>
#include <vector>

#include "Simulation.h"
#include "Robot.h"
#include "Body/Body.h"
#include "Body/BodySDFObj.h"
#include "Force/ForceGeneralSDFContact.h"
#include "CollisionDetection/CollisionDetection.h"
#include "CollisionDetection/Contact.h"
#include "makelevelset3.h"
#include "Mesh.h"

using namespace redmax;

namespace {

Body* body_of(void* sim, const char* name) {
    return static_cast<Simulation*>(sim)->get_body(std::string(name));
}

template <typename M>
void put_rowmajor(const M& m, double* out) {
    for (int r = 0; r < m.rows(); ++r)
        for (int c = 0; c < m.cols(); ++c) *out++ = m(r, c);
}

#define HARNESS_TRY try {
#define HARNESS_CATCH                                  \
    }                                                  \
    catch (const std::string& s) {                     \
        std::fprintf(stderr, "[ref] %s\n", s.c_str()); \
        return -2;                                     \
    }                                                  \
    catch (const char* s) {                            \
        std::fprintf(stderr, "[ref] %s\n", s);         \
        return -2;                                     \
    }                                                  \
    catch (...) { return -3; }

}  // namespace

extern "C" {

// ---------------------------------------------------------------- lifetime
void* ref_sim_create(const char* xml_string, const char* asset_folder) {
    try {
        return new Simulation(std::string(xml_string), std::string(asset_folder), false);
    } catch (const std::string& s) {
        std::fprintf(stderr, "[ref] %s\n", s.c_str());
    } catch (...) {
    }
    return nullptr;
}

void ref_sim_destroy(void* sim) { delete static_cast<Simulation*>(sim); }

int ref_sim_ndof(void* sim, int* ndof_r, int* ndof_m) {
    auto* s = static_cast<Simulation*>(sim);
    *ndof_r = s->_ndof_r;
    *ndof_m = s->_ndof_m;
    return 0;
}

// ---------------------------------------------------------------- bodies
int ref_body_index(void* sim, const char* name) {
    Body* b = body_of(sim, name);
    return b ? b->_index[0] : -1;
}

// mass, principal inertia diagonal (6: I_x I_y I_z m m m), E_ji (4x4), E_0i (4x4)
int ref_body_mass_props(void* sim, const char* name, double* mass, double* inertia6,
                        double* E_ji16, double* E_0i16) {
    HARNESS_TRY
    Body* b = body_of(sim, name);
    if (!b) return -1;
    *mass = b->_mass;
    for (int i = 0; i < 6; ++i) inertia6[i] = b->_Inertia(i);
    put_rowmajor(b->_E_ji, E_ji16);
    put_rowmajor(b->_E_0i, E_0i16);
    return 0;
    HARNESS_CATCH
}

int ref_body_num_contact_points(void* sim, const char* name) {
    Body* b = body_of(sim, name);
    return b ? (int)b->_contact_points.size() : -1;
}

int ref_body_get_contact_points(void* sim, const char* name, double* xyz, int cap) {
    Body* b = body_of(sim, name);
    if (!b) return -1;
    int n = (int)b->_contact_points.size();
    for (int i = 0; i < n && i < cap; ++i)
        for (int k = 0; k < 3; ++k) xyz[3 * i + k] = b->_contact_points[i](k);
    return n;
}

int ref_body_set_contact_points(void* sim, const char* name, const double* xyz, int n) {
    Body* b = body_of(sim, name);
    if (!b) return -1;
    b->_contact_points.resize(n);
    for (int i = 0; i < n; ++i) b->_contact_points[i] = Vector3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    return 0;
}

// Overwrites the SDF grid of an SDF body. values: ni*nj*nk doubles, i fastest.
int ref_body_set_sdf(void* sim, const char* name, int ni, int nj, int nk, const double* min_box,
                     const double* max_box, const double* dxyz, double col_th, const double* values) {
    auto* b = dynamic_cast<BodySDFObj*>(body_of(sim, name));
    if (!b) return -1;
    b->_SDF.resize(ni, nj, nk);
    std::memcpy(b->_SDF.a.data(), values, sizeof(double) * (size_t)ni * nj * nk);
    for (int k = 0; k < 3; ++k) {
        b->_min_box[k] = min_box[k];
        b->_max_box[k] = max_box[k];
    }
    b->_dx = dxyz[0];
    b->_dy = dxyz[1];
    b->_dz = dxyz[2];
    b->_col_th = col_th;
    return 0;
}

int ref_body_get_sdf_shape(void* sim, const char* name, int* nijk, double* min_box, double* max_box,
                           double* dxyz, double* col_th) {
    auto* b = dynamic_cast<BodySDFObj*>(body_of(sim, name));
    if (!b) return -1;
    nijk[0] = b->_SDF.ni;
    nijk[1] = b->_SDF.nj;
    nijk[2] = b->_SDF.nk;
    for (int k = 0; k < 3; ++k) {
        min_box[k] = b->_min_box[k];
        max_box[k] = b->_max_box[k];
    }
    dxyz[0] = b->_dx;
    dxyz[1] = b->_dy;
    dxyz[2] = b->_dz;
    *col_th = b->_col_th;
    return 0;
}

// The body-frame mesh BodySDFObj::precompute_SDF was given (BodyMeshObj::_V, _F): sizes when
// V or F is null, else copies (V: nv x 3, F: nt x 3).
int ref_body_mesh(void* sim, const char* name, int* nv, int* nt, double* V, int* F) {
    auto* b = dynamic_cast<BodySDFObj*>(body_of(sim, name));
    if (!b) return -1;
    const Matrix3X Vb = b->get_vertices();
    const Matrix3Xi Fb = b->get_faces();
    *nv = (int)Vb.cols();
    *nt = (int)Fb.cols();
    if (V && F) {
        for (int c = 0; c < Vb.cols(); ++c)
            for (int r = 0; r < 3; ++r) V[3 * c + r] = Vb(r, c);
        for (int c = 0; c < Fb.cols(); ++c)
            for (int r = 0; r < 3; ++r) F[3 * c + r] = Fb(r, c);
    }
    return 0;
}

int ref_body_get_sdf_values(void* sim, const char* name, double* values) {
    auto* b = dynamic_cast<BodySDFObj*>(body_of(sim, name));
    if (!b) return -1;
    std::memcpy(values, b->_SDF.a.data(), sizeof(double) * b->_SDF.a.size());
    return 0;
}

// Directly overwrites pose E_0i (4x4 row-major) and body velocity phi (w, v).
int ref_body_set_pose(void* sim, const char* name, const double* E16, const double* phi6) {
    Body* b = body_of(sim, name);
    if (!b) return -1;
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) b->_E_0i(r, c) = E16[4 * r + c];
    for (int i = 0; i < 6; ++i) b->_phi(i) = phi6[i];
    return 0;
}

int ref_body_set_contact_scale(void* sim, const char* name, double s) {
    Body* b = body_of(sim, name);
    if (!b) return -1;
    b->_contact_scale = s;
    return 0;
}

// ---------------------------------------------------------------- one contact query
// BodySDFObj::collision on body `name`.  out receives (row-major):
//  value part (11): d, n[3], ddot, tdot[3], xi2[3]
//  derivative part (135, want_deriv only): dd_dxw[3] dd_dq2[6] dn_dxw[9] dn_dq2[18]
//  dddot_dxw[3] dddot_dxwdot[3] dddot_dq2[6] dddot_dphi2[6] dtdot_dxw[9]
//  dtdot_dxwdot[9] dtdot_dq2[18] dtdot_dphi2[18] dxi2_dxw[9] dxi2_dq2[18]
int ref_collision(void* sim, const char* name, const double* xw, const double* xw_dot, int want_deriv,
                  double* out) {
    HARNESS_TRY
    auto* b = dynamic_cast<BodySDFObj*>(body_of(sim, name));
    if (!b) return -1;
    Vector3 x(xw[0], xw[1], xw[2]), xd(xw_dot[0], xw_dot[1], xw_dot[2]);
    dtype d, ddot;
    Vector3 n, tdot, xi2;
    if (!want_deriv) {
        b->collision(x, xd, d, n, ddot, tdot, xi2);
    } else {
        RowVector3 dd_dxw, dddot_dxw, dddot_dxwdot;
        RowVector6 dd_dq2, dddot_dq2, dddot_dphi2;
        Matrix3 dn_dxw, dtdot_dxw, dtdot_dxwdot, dxi2_dxw;
        Matrix36 dn_dq2, dtdot_dq2, dtdot_dphi2, dxi2_dq2;
        b->collision(x, xd, d, n, ddot, tdot, xi2, dd_dxw, dd_dq2, dn_dxw, dn_dq2, dddot_dxw, dddot_dxwdot,
                     dddot_dq2, dddot_dphi2, dtdot_dxw, dtdot_dxwdot, dtdot_dq2, dtdot_dphi2, dxi2_dxw, dxi2_dq2);
        double* o = out + 11;
        put_rowmajor(dd_dxw, o); o += 3;
        put_rowmajor(dd_dq2, o); o += 6;
        put_rowmajor(dn_dxw, o); o += 9;
        put_rowmajor(dn_dq2, o); o += 18;
        put_rowmajor(dddot_dxw, o); o += 3;
        put_rowmajor(dddot_dxwdot, o); o += 3;
        put_rowmajor(dddot_dq2, o); o += 6;
        put_rowmajor(dddot_dphi2, o); o += 6;
        put_rowmajor(dtdot_dxw, o); o += 9;
        put_rowmajor(dtdot_dxwdot, o); o += 9;
        put_rowmajor(dtdot_dq2, o); o += 18;
        put_rowmajor(dtdot_dphi2, o); o += 18;
        put_rowmajor(dxi2_dxw, o); o += 9;
        put_rowmajor(dxi2_dq2, o); o += 18;
    }
    out[0] = d;
    for (int k = 0; k < 3; ++k) out[1 + k] = n(k);
    out[4] = ddot;
    for (int k = 0; k < 3; ++k) out[5 + k] = tdot(k);
    for (int k = 0; k < 3; ++k) out[8 + k] = xi2(k);
    return 0;
    HARNESS_CATCH
}

// BodySDFObj::distance (world point, includes col_th).
int ref_distance(void* sim, const char* name, const double* xw, int n, double* out) {
    HARNESS_TRY
    auto* b = dynamic_cast<BodySDFObj*>(body_of(sim, name));
    if (!b) return -1;
    for (int i = 0; i < n; ++i) out[i] = b->distance(Vector3(xw[3 * i], xw[3 * i + 1], xw[3 * i + 2]));
    return 0;
    HARNESS_CATCH
}

// ---------------------------------------------------------------- one pair evaluation
// Runs ForceGeneralSDFContact(contact body A, SDF body B) through its public
// Force interface on the bodies' current poses and extracts the 12-dof
// sub-blocks [A; B] of fm, Km, Dm.  ids receives the active contact ids
// (ascending) found by collision_detection_general_SDF; with ids null that second
// detection is skipped (the timed CPU baseline: one Force call per pair, nothing more)
// and n_active is left unset.
int ref_pair_eval(void* sim, const char* name_a, const char* name_b, double kn, double kt, double mu,
                  double damping, double scale, int want_deriv, double* fm12, double* Km144, double* Dm144,
                  int* ids, int ids_cap, int* n_active) {
    HARNESS_TRY
    auto* s = static_cast<Simulation*>(sim);
    Body* a = body_of(sim, name_a);
    Body* b = body_of(sim, name_b);
    if (!a || !b) return -1;
    ForceGeneralSDFContact force(s, a, b, kn, kt, mu, damping);
    force.set_scale(scale);
    int ndof_m = s->_ndof_m;
    VectorX fm = VectorX::Zero(ndof_m), fr = VectorX::Zero(s->_ndof_r);
    MatrixX Km = MatrixX::Zero(ndof_m, ndof_m), Dm = MatrixX::Zero(ndof_m, ndof_m);
    MatrixX Kr = MatrixX::Zero(s->_ndof_r, s->_ndof_r), Dr = Kr;
    if (want_deriv)
        force.computeForceWithDerivative(fm, fr, Km, Dm, Kr, Dr, false);
    else
        force.computeForce(fm, fr, false);
    int ia = a->_index[0], ib = b->_index[0];
    int idx[12];
    for (int k = 0; k < 6; ++k) {
        idx[k] = ia + k;
        idx[6 + k] = ib + k;
    }
    for (int r = 0; r < 12; ++r) {
        fm12[r] = fm(idx[r]);
        for (int c = 0; c < 12; ++c) {
            Km144[12 * r + c] = want_deriv ? Km(idx[r], idx[c]) : 0.0;
            Dm144[12 * r + c] = want_deriv ? Dm(idx[r], idx[c]) : 0.0;
        }
    }
    if (!ids) return 0;
    std::vector<Contact> contacts;
    collision_detection_general_SDF(a, dynamic_cast<BodySDFObj*>(b), contacts);
    *n_active = (int)contacts.size();
    for (int i = 0; i < (int)contacts.size() && i < ids_cap; ++i) ids[i] = contacts[i]._id;
    return 0;
    HARNESS_CATCH
}

// ---------------------------------------------------------------- stepping
int ref_sim_reset(void* sim, int backward) {
    HARNESS_TRY
    static_cast<Simulation*>(sim)->reset(backward != 0, false);
    return 0;
    HARNESS_CATCH
}

int ref_sim_set_state_init(void* sim, const double* q, const double* qdot) {
    HARNESS_TRY
    auto* s = static_cast<Simulation*>(sim);
    VectorX q0(s->_ndof_r), qd0(s->_ndof_r);
    for (int i = 0; i < s->_ndof_r; ++i) {
        q0(i) = q[i];
        qd0(i) = qdot[i];
    }
    s->set_state_init(q0, qd0);
    return 0;
    HARNESS_CATCH
}

int ref_sim_set_external_force(void* sim, const char* name, const double* f6) {
    HARNESS_TRY
    VectorX f(6);
    for (int i = 0; i < 6; ++i) f(i) = f6[i];
    static_cast<Simulation*>(sim)->set_body_external_force(std::string(name), f);
    return 0;
    HARNESS_CATCH
}

int ref_sim_forward(void* sim, int num_steps) {
    HARNESS_TRY
    static_cast<Simulation*>(sim)->forward(num_steps, false, false);
    return 0;
    HARNESS_CATCH
}

int ref_sim_is_converged(void* sim) { return static_cast<Simulation*>(sim)->is_converged() ? 1 : 0; }

int ref_sim_get_state(void* sim, double* q, double* qdot) {
    HARNESS_TRY
    auto* s = static_cast<Simulation*>(sim);
    VectorX a = s->get_q(), b = s->get_qdot();
    for (int i = 0; i < s->_ndof_r; ++i) {
        q[i] = a(i);
        qdot[i] = b(i);
    }
    return 0;
    HARNESS_CATCH
}

// Reverse pass of a run started with ref_sim_reset(sim, 1).  df_dq holds
// ndof_r*T terminal/per-step loss derivatives; df_dq0/df_dqdot0 receive the
// reference's backward_BDF1 results.
int ref_sim_backward(void* sim, const double* df_dq, int T, double* df_dq0, double* df_dqdot0) {
    HARNESS_TRY
    auto* s = static_cast<Simulation*>(sim);
    int n = s->_ndof_r;
    auto& info = s->_backward_info;
    info.set_flags(true, true, false, false);
    info._df_dq0 = VectorX::Zero(n);
    info._df_dqdot0 = VectorX::Zero(n);
    info._df_dq = VectorX::Zero(n * T);
    for (int i = 0; i < n * T; ++i) info._df_dq(i) = df_dq[i];
    info._df_dvar = VectorX::Zero(s->_ndof_var * T);
    s->backward();
    for (int i = 0; i < n; ++i) {
        df_dq0[i] = s->_backward_results._df_dq0(i);
        df_dqdot0[i] = s->_backward_results._df_dqdot0(i);
    }
    return 0;
    HARNESS_CATCH
}

/* sdfgen::make_level_set3 as the reference builds its grids (BodySDFObj::precompute_SDF):
 * phi (ni*nj*nk floats, i fastest). */
int ref_make_level_set3(const float* verts, int nv, const unsigned* tris, int nt, const float* origin, float dx,
                        float dy, float dz, int ni, int nj, int nk, int exact_band, float* phi) {
    HARNESS_TRY
    std::vector<sdfgen::Vec3f> x(nv);
    for (int k = 0; k < nv; ++k) x[k] = sdfgen::Vec3f(verts[3 * k], verts[3 * k + 1], verts[3 * k + 2]);
    std::vector<sdfgen::Vec3ui> t(nt);
    for (int k = 0; k < nt; ++k) t[k] = sdfgen::Vec3ui(tris[3 * k], tris[3 * k + 1], tris[3 * k + 2]);
    sdfgen::Array3f out;
    sdfgen::make_level_set3(t, x, sdfgen::Vec3f(origin[0], origin[1], origin[2]), dx, dy, dz, ni, nj, nk, out,
                            exact_band);
    for (int k = 0; k < nk; ++k)
        for (int j = 0; j < nj; ++j)
            for (int i = 0; i < ni; ++i) phi[i + ni * (j + nj * k)] = out(i, j, k);
    return 0;
    HARNESS_CATCH
}

// redmax::SDFMesh (rm/Mesh.cpp:41-198): V nv x 3, F nt x 3 (the reference takes 3 x n).
void* ref_sdfmesh_create(const double* V, int nv, const int* F, int nt, double dx, const char* load_path,
                         const char* save_path) {
    try {
        Matrix3X Vm(3, nv);
        Matrix3Xi Fm(3, nt);
        for (int c = 0; c < nv; ++c)
            for (int r = 0; r < 3; ++r) Vm(r, c) = V[3 * c + r];
        for (int c = 0; c < nt; ++c)
            for (int r = 0; r < 3; ++r) Fm(r, c) = F[3 * c + r];
        return new SDFMesh(Vm, Fm, dx, load_path ? load_path : "", save_path ? save_path : "");
    } catch (...) {
        return nullptr;
    }
}

void ref_sdfmesh_destroy(void* m) { delete static_cast<SDFMesh*>(m); }

int ref_sdfmesh_shape(void* m, int* nijk, double* min_box, double* max_box, double* dxyz) {
    auto* s = static_cast<SDFMesh*>(m);
    nijk[0] = s->_SDF.ni;
    nijk[1] = s->_SDF.nj;
    nijk[2] = s->_SDF.nk;
    for (int k = 0; k < 3; ++k) {
        min_box[k] = s->_min_box[k];
        max_box[k] = s->_max_box[k];
    }
    dxyz[0] = s->_dx;
    dxyz[1] = s->_dy;
    dxyz[2] = s->_dz;
    return 0;
}

int ref_sdfmesh_values(void* m, double* values) {
    auto* s = static_cast<SDFMesh*>(m);
    std::memcpy(values, s->_SDF.a.data(), sizeof(double) * s->_SDF.a.size());
    return 0;
}

// SDFMesh::distance of n points (n x 3) and min_distance
int ref_sdfmesh_distance(void* m, const double* X, int n, double* d, double* min_d) {
    HARNESS_TRY
    auto* s = static_cast<SDFMesh*>(m);
    Matrix3X Xm(3, n);
    for (int c = 0; c < n; ++c)
        for (int r = 0; r < 3; ++r) Xm(r, c) = X[3 * c + r];
    VectorX dv = s->distance(Xm);
    for (int c = 0; c < n; ++c) d[c] = dv(c);
    *min_d = s->min_distance(Xm);
    return 0;
    HARNESS_CATCH
}

// Simulation::get_body_distance / body_in_contact (rm/Simulation.cpp:276-303)
int ref_body_distance(void* sim, const char* from, const char* to, double* d) {
    HARNESS_TRY
    *d = static_cast<Simulation*>(sim)->get_body_distance(from, to);
    return 0;
    HARNESS_CATCH
}

int ref_body_in_contact(void* sim, const char* a, const char* b, double eps) {
    try {
        return static_cast<Simulation*>(sim)->body_in_contact(a, b, eps) ? 1 : 0;
    } catch (...) {
        return -1;
    }
}

}  // extern "C"
