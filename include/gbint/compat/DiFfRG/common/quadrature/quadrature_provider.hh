// Forwarding header at the path of DiFfRG/include/DiFfRG/common/quadrature/quadrature_provider.hh:
// DiFfRG::QuadratureProvider is provided by gbint/integrators.hh (libgbint).
#pragma once
#include "gbint/integrators.hh"
