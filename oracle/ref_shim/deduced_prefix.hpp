/*
 * deduced_prefix.hpp -- minimal stand-in for the sim::Fluid class so that the
 * reference's Fluid::update_deduced_attributes (PCISPH/src/sim/Fluid.cpp:377-443,
 * everything above its "// buffers" comment) compiles on the host. TEST
 * INFRASTRUCTURE ONLY (see build_ref.sh). The extracted function body is
 * appended right after this header; build_ref.sh closes it and namespace sim.
 */
#include <algorithm>
#include <cmath>
#include <utils/constants.h>

namespace sim {
struct Fluid {
    Simulation_Params params;
    void update_deduced_attributes();
};
