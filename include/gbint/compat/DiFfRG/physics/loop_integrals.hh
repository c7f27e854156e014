// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/loop_integrals.hh:
// DiFfRG::LoopIntegrals (and QGauss<1> without deal.II) are provided by gbint/loop_integrals.hh.
#pragma once
#include "gbint/loop_integrals.hh"
