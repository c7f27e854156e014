// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/physics.hh: flow equations,
// loop integrals, regulators and the request_data/update_data fan-out helpers.  (The reference
// also includes its Litim threshold functions, which are outside the integration path.)
#pragma once
#include "gbint/flow_equations.hh"
#include "gbint/flow_utils.hh"
#include "gbint/loop_integrals.hh"
#include "gbint/math_compat.hh"
#include "gbint/regulators.hh"
