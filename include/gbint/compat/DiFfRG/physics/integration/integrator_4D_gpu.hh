// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/integration/integrator_4D_gpu.hh:
// the class templates of that header are provided by gbint/integrators.hh (libgbint).
#pragma once
#include "gbint/integrators.hh"
