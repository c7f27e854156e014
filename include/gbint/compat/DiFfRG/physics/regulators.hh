// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/regulators.hh: every regulator
// class (gbint/regulators.hh).
#pragma once
#include "gbint/math_compat.hh"
#include "gbint/regulators.hh"
