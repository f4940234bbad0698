// ForceGeneralSDFContactGPU: a drop-in for redmax's ForceGeneralSDFContact
// (simulation/redmax/Force/ForceGeneralSDFContact.h:12-54) that evaluates the
// contact on the GPU through libsdfcontact (include/sdfc.h).
//
// It keeps the reference's Force interface (simulation/redmax/Force/Force.h:40-47),
// constructor arguments, setters and side effects, so Robot, Simulation and the
// Python bindings use it unchanged.  Compiled against the reference's headers; the
// XML parser creates it where it creates ForceGeneralSDFContact
// (simulation/redmax/Simulation_Constructor.cpp:300-312).
//
// Each call evaluates the contact points and grid as they are at that moment: the
// plugin keeps a host copy of what it uploaded and re-uploads whatever changed
// (values, box, spacing, threshold), so points or SDF values edited in place are
// seen.  Derivatives follow set_derivative_mode: SDFC_DERIV_ANALYTIC (default,
// the interpolant's analytic cell derivatives: Km, Dm within about 1e-6 of the
// reference's finite-difference stencil) or SDFC_DERIV_STENCIL (the reference's
// stencil, bit for bit in the SDF derivatives: Km, Dm to FP64 round-off).
#pragma once
#include "Common.h"
#include "Force/Force.h"
#include "Utils.h"
#include "sdfc.h"

#include <vector>

namespace redmax {

class Body;
class BodySDFObj;

class ForceGeneralSDFContactGPU : public Force {
public:
    Body* _contact_body;    // its contact points are queried (ForceGeneralSDFContact.h:14)
    BodySDFObj* _SDF_body;  // its grid is queried (ForceGeneralSDFContact.h:15)
    dtype _kn, _kt, _mu, _damping, _scale;

    ForceGeneralSDFContactGPU(Simulation* sim, Body* contact_body, Body* SDF_body, dtype kn = 1., dtype kt = 0.,
                              dtype mu = 0., dtype damping = 0.);
    ~ForceGeneralSDFContactGPU();

    void set_stiffness(dtype kn, dtype kt);
    void set_friction(dtype mu);
    void set_damping(dtype damping);
    void set_scale(dtype scale);
    // SDFC_DERIV_ANALYTIC or SDFC_DERIV_STENCIL (no counterpart in the reference, which
    // always takes the stencil)
    void set_derivative_mode(int mode);

    void computeForce(VectorX& fm, VectorX& fr, bool verbose = false) override;
    void computeForceWithDerivative(VectorX& fm, VectorX& fr, MatrixX& Km, MatrixX& Dm, MatrixX& Kr, MatrixX& Dr,
                                    bool verbose = false) override;

private:
    int _points = -1, _grid = -1;     // handles in the process-wide context
    int _deriv_mode = SDFC_DERIV_ANALYTIC;
    std::vector<double> _points_seen;  // the points as last uploaded (x, y, z per point)
    std::vector<double> _grid_seen;    // the grid as last uploaded: ni, nj, nk, box, spacing, col_th, values
    void upload_if_needed();
    int evaluate(bool deriv, double* fm12, double* Km144, double* Dm144);
};

}  // namespace redmax
