// See ForceGeneralSDFContactGPU.h.
#include "ForceGeneralSDFContactGPU.h"

#include <cstring>
#include <string>
#include <vector>

#include "Body/Body.h"
#include "Body/BodyCuboid.h"
#include "Body/BodySDFObj.h"

namespace redmax {

namespace {

// One libsdfcontact context per process, on device 0 (the reference runs one
// simulation per process, utils/parallel.py:10).
sdfc_context* shared_context() {
    static sdfc_context* ctx = nullptr;
    if (!ctx && sdfc_create(&ctx, 0) != SDFC_OK) throw_error("libsdfcontact: no usable CUDA device");
    return ctx;
}

void check(int rc, const char* what) {
    if (rc != SDFC_OK)
        throw_error(std::string("libsdfcontact ") + what + ": " + sdfc_last_error(shared_context()));
}

void pose_of(const Body* b, double* E16, double* phi6) {
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) E16[4 * r + c] = b->_E_0i(r, c);
    for (int k = 0; k < 6; ++k) phi6[k] = b->_phi(k);
}

}  // namespace

ForceGeneralSDFContactGPU::ForceGeneralSDFContactGPU(Simulation* sim, Body* contact_body, Body* SDF_body, dtype kn,
                                                     dtype kt, dtype mu, dtype damping)
    : Force(sim) {
    _contact_body = contact_body;
    _SDF_body = dynamic_cast<BodySDFObj*>(SDF_body);
    if (_SDF_body == nullptr) throw_error("The second body in Contact should be SDF body.");
    _kn = kn;
    _kt = kt;
    _mu = mu;
    _damping = damping;
    _scale = 1.;
}

ForceGeneralSDFContactGPU::~ForceGeneralSDFContactGPU() {}

void ForceGeneralSDFContactGPU::set_stiffness(dtype kn, dtype kt) { _kn = kn; _kt = kt; }
void ForceGeneralSDFContactGPU::set_friction(dtype mu) { _mu = mu; }
void ForceGeneralSDFContactGPU::set_damping(dtype damping) { _damping = damping; }
void ForceGeneralSDFContactGPU::set_scale(dtype scale) { _scale = scale; }
void ForceGeneralSDFContactGPU::set_derivative_mode(int mode) {
    if (mode != SDFC_DERIV_ANALYTIC && mode != SDFC_DERIV_STENCIL) throw_error("unknown derivative mode");
    _deriv_mode = mode;
}

void ForceGeneralSDFContactGPU::upload_if_needed() {
    sdfc_context* ctx = shared_context();
    // the contact points detection reads (CollisionDetection.cpp:126-131): a cuboid's
    // general contact points, any other body's contact points
    std::vector<Vector3> pts = _contact_body->get_contact_points();
    if (BodyCuboid* cuboid = dynamic_cast<BodyCuboid*>(_contact_body)) pts = cuboid->get_general_contact_points();
    std::vector<double> xyz(3 * pts.size());
    for (size_t i = 0; i < pts.size(); ++i)
        for (int k = 0; k < 3; ++k) xyz[3 * i + k] = pts[i](k);
    if (_points < 0 || xyz != _points_seen) {
        check(sdfc_upload_points(ctx, xyz.data(), (int)pts.size(), SDFC_STORAGE_F64, &_points), "upload_points");
        _points_seen.swap(xyz);
    }
    const BodySDFObj* b = _SDF_body;
    const size_t n = (size_t)b->_SDF.ni * b->_SDF.nj * b->_SDF.nk;
    const double head[13] = {(double)b->_SDF.ni, (double)b->_SDF.nj, (double)b->_SDF.nk, b->_min_box[0], b->_min_box[1],
                             b->_min_box[2], b->_max_box[0], b->_max_box[1], b->_max_box[2], b->_dx, b->_dy, b->_dz,
                             b->_col_th};
    const bool same = _grid >= 0 && _grid_seen.size() == 13 + n &&
                      std::memcmp(_grid_seen.data(), head, sizeof head) == 0 &&
                      std::memcmp(_grid_seen.data() + 13, b->_SDF.a.data(), n * sizeof(double)) == 0;
    if (!same) {
        check(sdfc_upload_grid(ctx, b->_SDF.a.data(), b->_SDF.ni, b->_SDF.nj, b->_SDF.nk, head + 3, head + 6, head + 9,
                               b->_col_th, SDFC_STORAGE_F64, &_grid),
              "upload_grid");
        _grid_seen.assign(head, head + 13);
        _grid_seen.insert(_grid_seen.end(), b->_SDF.a.data(), b->_SDF.a.data() + n);
    }
}

int ForceGeneralSDFContactGPU::evaluate(bool deriv, double* fm12, double* Km144, double* Dm144) {
    upload_if_needed();
    double EA[16], phiA[6], EB[16], phiB[6];
    pose_of(_contact_body, EA, phiA);
    pose_of(_SDF_body, EB, phiB);
    sdfc_params p{_kn, _kt, _mu, _damping, _scale, _contact_body->_contact_scale};
    int n_active = 0;
    check(sdfc_set_derivative_mode(shared_context(), _deriv_mode), "set_derivative_mode");
    check(sdfc_evaluate(shared_context(), _points, _grid, EA, phiA, EB, phiB, &p, deriv ? 1 : 0, fm12, Km144, Dm144,
                        &n_active),
          "evaluate");
    // the detection's side effect (CollisionDetection.cpp:143-146)
    if (n_active > 0) {
        _contact_body->add_contact_body(_SDF_body->_name);
        _SDF_body->add_contact_body(_contact_body->_name);
    }
    return n_active;
}

// ForceGeneralSDFContact::computeForce, ForceGeneralSDFContact.cpp:46-67
void ForceGeneralSDFContactGPU::computeForce(VectorX& fm, VectorX& fr, bool verbose) {
    auto t0 = clock();
    double f[12];
    evaluate(false, f, nullptr, nullptr);
    for (int k = 0; k < 6; ++k) {
        fm(_contact_body->_index[0] + k) += f[k];
        fm(_SDF_body->_index[0] + k) += f[6 + k];
    }
    _time.add("compute force", clock() - t0);
}

// ForceGeneralSDFContact::computeForceWithDerivative, ForceGeneralSDFContact.cpp:69-105
void ForceGeneralSDFContactGPU::computeForceWithDerivative(VectorX& fm, VectorX& fr, MatrixX& Km, MatrixX& Dm,
                                                           MatrixX& Kr, MatrixX& Dr, bool verbose) {
    auto t0 = clock();
    double f[12], K[144], D[144];
    evaluate(true, f, K, D);
    const int idx[2] = {_contact_body->_index[0], _SDF_body->_index[0]};
    for (int r = 0; r < 12; ++r) {
        const int gr = idx[r / 6] + r % 6;
        fm(gr) += f[r];
        for (int c = 0; c < 12; ++c) {
            const int gc = idx[c / 6] + c % 6;
            Km(gr, gc) += K[12 * r + c];
            Dm(gr, gc) += D[12 * r + c];
        }
    }
    _time.add("compute force", clock() - t0);
}

}  // namespace redmax
