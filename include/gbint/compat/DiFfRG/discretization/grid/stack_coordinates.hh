// Forwarding header at the path of DiFfRG/include/DiFfRG/discretization/grid/stack_coordinates.hh:
// the coordinate classes are provided by gbint/interpolators.hh.
#pragma once
#include "gbint/interpolators.hh"
