// ForceGeneralSDFContactGPU: a drop-in for redmax's ForceGeneralSDFContact
// (simulation/redmax/Force/ForceGeneralSDFContact.h:12-54) that evaluates the
// contact on the GPU through libsdfcontact (include/sdfc.h).
//
// It keeps the reference's Force interface (simulation/redmax/Force/Force.h:40-47),
// constructor arguments, setters and side effects, so Robot, Simulation and the
// Python bindings use it unchanged.  Compiled against the reference's headers;
// see INTEGRATION.md for the two lines the XML parser needs.
#pragma once
#include "Common.h"
#include "Force/Force.h"
#include "Utils.h"
#include "sdfc.h"

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

    void computeForce(VectorX& fm, VectorX& fr, bool verbose = false) override;
    void computeForceWithDerivative(VectorX& fm, VectorX& fr, MatrixX& Km, MatrixX& Dm, MatrixX& Kr, MatrixX& Dr,
                                    bool verbose = false) override;

private:
    int _points = -1, _grid = -1;     // handles in the process-wide context
    size_t _points_n = 0;             // uploaded point count (re-upload when it changes)
    const void* _grid_data = nullptr; // uploaded grid storage (re-upload when it changes)
    void upload_if_needed();
    int evaluate(bool deriv, double* fm12, double* Km144, double* Dm144);
};

}  // namespace redmax
