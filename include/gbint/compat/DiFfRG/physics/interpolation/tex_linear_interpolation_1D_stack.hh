// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/interpolation/tex_linear_interpolation_1D_stack.hh:
// the interpolator templates are provided by gbint/interpolators.hh.
#pragma once
#include "gbint/interpolators.hh"
