// Forwarding header at the path of DiFfRG/include/DiFfRG/common/math.hh: powr, S_d, V_d,
// is_close, sign, heaviside_theta, dot and autodiff::real (gbint/math_compat.hh).
#pragma once
#include "gbint/math_compat.hh"
