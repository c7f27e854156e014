// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/integration/integrator_1D_cartesian_cpu.hh: the CPU (TBB)
// class name is an alias of the GPU class in gbint/integrators.hh.
#pragma once
#include "gbint/integrators.hh"
