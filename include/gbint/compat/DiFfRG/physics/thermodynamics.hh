// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/thermodynamics.hh: Cosh ...
// Csch, CothFiniteT, TanhFiniteT, SechFiniteT, CschFiniteT, cothS/tanhS and derivatives, nB, nF
// (gbint/thermodynamics.hh); like the reference header it brings in the common utilities.
#pragma once
#include "gbint/utils_compat.hh"
#include "gbint/thermodynamics.hh"
