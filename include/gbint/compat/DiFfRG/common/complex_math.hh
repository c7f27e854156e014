// Forwarding header at the path of DiFfRG/include/DiFfRG/common/complex_math.hh: complex,
// real, imag, cot and mixed-type complex arithmetic (gbint/math_compat.hh).
#pragma once
#include "gbint/math_compat.hh"
