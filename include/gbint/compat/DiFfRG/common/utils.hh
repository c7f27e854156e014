// Forwarding header at the path of DiFfRG/include/DiFfRG/common/utils.hh (the first include of
// every generated flows/def.hh): host utilities, JSONValue and the math helpers, from
// gbint/utils_compat.hh, gbint/json.hh and gbint/math_compat.hh.
#pragma once
#include "gbint/utils_compat.hh"
