// Internal helpers of the C ABI implementation.
#pragma once

#include <string>

#include "../../include/ek_gb300.h"
#include "ek_common.cuh"

namespace ek_internal
{
// record a thread-local error message and return the status
ek_status fail(ek_status s, const std::string & msg);
// parameter checks shared by the single solver and the ensemble
ek_status validate(const ek_params & p);
// kernel parameters of a run
ekc::KParams make_kparams(const ek_params & p);
// device bytes of one state in the run's precision
size_t state_bytes(const ek_params & p, const ekc::KParams & kp);
} // namespace ek_internal
