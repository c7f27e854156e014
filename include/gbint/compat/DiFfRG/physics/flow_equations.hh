// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/flow_equations.hh:
// FlowEquations and FlowEquationsFiniteT are provided by gbint/flow_equations.hh.
#pragma once
#include "gbint/flow_equations.hh"
