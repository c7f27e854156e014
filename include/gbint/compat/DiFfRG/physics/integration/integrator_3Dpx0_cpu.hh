// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/integration/integrator_3Dpx0_cpu.hh: the CPU (TBB)
// class name is an alias of the GPU class in gbint/integrators.hh.
#pragma once
#include "gbint/integrators.hh"
