// Drop-in check of the GPU Force plugin (test infrastructure, compiled only into
// oracle/_ref/libredmax_gpu_plugin.so together with the reference objects, ref_harness.cpp and
// the plugin).  It puts ForceGeneralSDFContactGPU where the reference's XML parser put
// ForceGeneralSDFContact (simulation/redmax/Simulation_Constructor.cpp:300-312), with the same
// bodies and coefficients, so that one scene can be stepped by the stock force and by the plugin.
#include <string>

#include "Body/Body.h"
#include "Body/BodySDFObj.h"
#include "Force/ForceGeneralSDFContact.h"
#include "ForceGeneralSDFContactGPU.h"
#include "Robot.h"
#include "Simulation.h"

using namespace redmax;

extern "C" {

// Replaces every ForceGeneralSDFContact of the simulation's robot by a ForceGeneralSDFContactGPU
// (derivative mode `deriv_mode`, SDFC_DERIV_*).  Returns the number replaced, or -1 on an error.
// The replaced forces stay allocated, as the robot never deletes its forces.
int ref_sim_use_gpu_contacts(void* sim, int deriv_mode) {
    try {
        Simulation* s = static_cast<Simulation*>(sim);
        int n = 0;
        for (Force*& f : s->_robot->_forces) {
            ForceGeneralSDFContact* c = dynamic_cast<ForceGeneralSDFContact*>(f);
            if (!c) continue;
            auto* g = new ForceGeneralSDFContactGPU(s, c->_contact_body, c->_SDF_body, c->_kn, c->_kt, c->_mu,
                                                    c->_damping);
            g->set_scale(c->_scale);
            g->set_derivative_mode(deriv_mode);
            f = g;
            ++n;
        }
        return n;
    } catch (...) {
        return -1;
    }
}

}  // extern "C"
