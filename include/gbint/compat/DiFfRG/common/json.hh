// Forwarding header at the path of DiFfRG/include/DiFfRG/common/json.hh: DiFfRG::JSONValue
// without boost::json (gbint/json.hh).
#pragma once
#include "gbint/json.hh"
