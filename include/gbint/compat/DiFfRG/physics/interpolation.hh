// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/interpolation.hh: the
// interpolators and coordinates (gbint/interpolators.hh).
#pragma once
#include "gbint/interpolators.hh"
