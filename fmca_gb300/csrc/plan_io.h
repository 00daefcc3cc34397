// Plan files (plan_io.cpp): save and load a built plan on the host.
#pragma once

#include <cstdint>
#include <string>

#include "h2_plan.h"

namespace fmca {
// both throw std::runtime_error on I/O errors and on malformed files
void save_plan(const Plan& plan, int64_t min_leaf, const std::string& path);
void load_plan(const std::string& path, Plan* plan, int64_t* min_leaf);
}  // namespace fmca
