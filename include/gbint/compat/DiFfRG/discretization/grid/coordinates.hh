// Forwarding header at the path of DiFfRG/include/DiFfRG/discretization/grid/coordinates.hh:
// LinearCoordinates1D, LogarithmicCoordinates1D, CoordinatePackND are provided by gbint/interpolators.hh.
#pragma once
#include "gbint/interpolators.hh"
