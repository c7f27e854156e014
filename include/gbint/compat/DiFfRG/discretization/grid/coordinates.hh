// Forwarding header at the path of DiFfRG/include/DiFfRG/discretization/grid/coordinates.hh:
// LinearCoordinates1D, LogarithmicCoordinates1D, CoordinatePackND are provided by
// gbint/interpolators.hh, make_grid by gbint/flow_utils.hh.
#pragma once
#include "gbint/interpolators.hh"
#include "gbint/flow_utils.hh"
