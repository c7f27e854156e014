// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/integration/integrator_4D_qmc.hh:
// the class templates of that header are provided by gbint/qmc.hh (libgbint).
#pragma once
#include "gbint/qmc.hh"
