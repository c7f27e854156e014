// Forwarding header at the path of DiFfRG/include/DiFfRG/physics/utils.hh: request_data,
// update_data, update_interpolator and get_data are provided by gbint/flow_utils.hh.
#pragma once
#include "gbint/flow_utils.hh"
