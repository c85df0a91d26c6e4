// Internal helpers of the C ABI implementation.
#pragma once

#include <string>

#include "../../include/ek_gb300.h"

namespace ek_internal
{
// record a thread-local error message and return the status
ek_status fail(ek_status s, const std::string & msg);
} // namespace ek_internal
