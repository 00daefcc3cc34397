// Private definition of the opaque fmca_plan handle, shared by the C ABI
// translation units.
#pragma once

#include <atomic>
#include <cstddef>
#include <cstdint>
#include <string>

#include "../../include/fmca_gb300.h"
#include "h2_gpu.h"
#include "h2_plan.h"

struct fmca_plan {
  fmca::Plan plan;
  fmca::gpu::DevPlan* dev = nullptr;
  // device staging for fmca_matvec_host
  void* hx = nullptr;
  void* hy = nullptr;
  size_t hx_bytes = 0, hy_bytes = 0;
  int64_t min_leaf = 0;
  // stage events on the following matvecs (fmca_plan_set_profiling)
  std::atomic<bool> profile{false};
  // limit of the kernel sums' bounded waits in ns (0: the default of 2 s)
  std::atomic<uint64_t> wait_ns{0};
  // test hook of fmca_plan_set_stalled_wait
  std::atomic<int> stall{0};
  std::atomic<bool> autotune{false};
};

namespace fmca {
namespace capi {
// records msg as the calling thread's last error and returns s
fmca_status fail(fmca_status s, const std::string& msg);
// argument checks shared by the matvec entry points
fmca_status check_matvec_args(const fmca_plan* p, const fmca_kernel_desc* kernel,
                              int precision, int dtype, int order, int nrhs,
                              const void* x, const void* y);
gpu::KernelDesc to_desc(const fmca_kernel_desc* k);
// the options of a call on plan p: its settings (profiling, wait limit,
// stalled-wait hook, autotuner)
gpu::CallOpts call_opts(const fmca_plan* p);
}  // namespace capi
}  // namespace fmca
