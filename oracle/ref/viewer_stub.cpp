// Replaces the reference's interactive replay viewer (SimViewer.cpp, which
// needs OpenGL) in the oracle build.  Simulation.cpp names these members only
// on its replay path; the oracle never replays, so every body throws.
#include "SimViewer.h"

namespace redmax {

SimViewer::SimViewer(Simulation* sim) : _sim(sim), _timer(nullptr), _keyboard_handler(nullptr) {
    throw std::string("replay viewer is not part of the oracle build");
}
SimViewer::~SimViewer() {}
void SimViewer::initialize() { throw std::string("replay viewer is not part of the oracle build"); }
void SimViewer::run() { throw std::string("replay viewer is not part of the oracle build"); }

}  // namespace redmax
