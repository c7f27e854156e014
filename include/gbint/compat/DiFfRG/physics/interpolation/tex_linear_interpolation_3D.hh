// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/interpolation/tex_linear_interpolation_3D.hh:
// the interpolator templates are provided by gbint/interpolators.hh.
#pragma once
#include "gbint/interpolators.hh"
