// Packed near groups of the tensor-core kernel sum with one target half
// (host side; h2_gpu.cu uploads them, fmca_plan_near_packed reports them).
#pragma once

#include <cstdint>
#include <vector>

#include "h2_plan.h"

namespace fmca {

// Groups of up to cap targets (rows in cluster order) over source intervals
// (columns in cluster order) that carry the leaves they serve.
struct PackedNear {
  std::vector<uint32_t> tbegin, tcount;     // per group: first target, targets
  std::vector<int32_t> ivl_begin, ivl_end;  // per group: its intervals
  std::vector<uint32_t> split;              // per group: targets of the first leaf
  std::vector<uint32_t> ivl;                // pairs (begin, end)
  std::vector<uint32_t> imask;              // per interval: bit 0 first leaf, bit 1 second
  size_t ngroups() const { return tbegin.size(); }
};

// The rows of consecutive row leaves back to back in groups of up to cap
// targets, at most two leaves per group; see near_pack.cpp.  false: no
// packed list (it would not save a tenth of the groups of one leaf each,
// leaves chunked to cap, or a check of the result failed).
bool build_near_packed(const Plan& plan, uint32_t cap, PackedNear* out);

}  // namespace fmca
