// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/integration_finiteT/integrator_4D_finiteTx0_cpu.hh: the CPU (TBB)
// class name is an alias of the GPU class in gbint/integrators.hh.
#pragma once
#include "gbint/integrators.hh"
