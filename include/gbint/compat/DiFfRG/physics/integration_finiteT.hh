// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/integration_finiteT.hh: the
// finite-temperature q0 (Matsubara) and x0 (sum + tail) families (gbint/integrators.hh).
#pragma once
#include "gbint/integrators.hh"
#include "gbint/math_compat.hh"
#include "gbint/json.hh"
