// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/integration.hh: every zero-T
// integrator family, IntegratorConstant and QuadratureProvider (gbint/integrators.hh), the QMC
// integrators (gbint/qmc.hh), with the result types double, float, complex and autodiff::real
// (gbint/math_compat.hh).
#pragma once
#include "gbint/integrators.hh"
#include "gbint/qmc.hh"
#include "gbint/math_compat.hh"
#include "gbint/json.hh"
