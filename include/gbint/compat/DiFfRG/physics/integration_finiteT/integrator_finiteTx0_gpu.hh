// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/integration_finiteT/integrator_finiteTx0_gpu.hh:
// the class templates of that header are provided by gbint/integrators.hh (libgbint).
#pragma once
#include "gbint/integrators.hh"
