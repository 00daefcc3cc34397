// GPU side of the H2 matvec: device copy of a Plan and the matvec driver.
#pragma once

#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>
#include <memory>
#include <string>

#include "h2_plan.h"

namespace fmca {
namespace gpu {

struct DevPlan;

struct KernelDesc {
  int type;
  double l, c, nu, sigma2;
};

// Options of one call, set on the device plan under its mutex (so that
// concurrent calls on one plan do not race on them).
struct CallOpts {
  bool profile = false;  // stage events for fmca_plan_profile
  uint64_t wait_ns = 0;  // limit of the kernel sums' bounded waits (0: 2 s)
  int stall = 0;         // test hook: the kernel sums' first wait runs out
  bool autotune = false; // tune launch shapes on the first call of a key
};

// status codes are the fmca_status values of include/fmca_gb300.h
int upload(const Plan& plan, int precision, DevPlan** dev, std::string* err);
void destroy(DevPlan* dev);
size_t workspace_bytes(const Plan& plan, int precision, int nrhs);
int matvec(const Plan& plan, DevPlan* dev, const KernelDesc& k, int precision,
           int dtype, int order, int nrhs, const void* x, int64_t sxi,
           int64_t sxr, void* y, int64_t syi, int64_t syr, void* ws,
           size_t ws_bytes, cudaStream_t stream, std::string* err, const CallOpts& opts);
int check_device_error(DevPlan* dev, std::string* err);
// Assembled plans: device bytes the stored blocks take (host count, no
// device needed); storing them for kernel k (FP64 values for
// FMCA_PREC_FP64, FP32 otherwise; replaces earlier ones); their release; the
// precision they were assembled in (-1: none); the matvec that streams them.
size_t assembled_bytes(const Plan& plan, int precision);
int assemble(const Plan& plan, DevPlan* dev, const KernelDesc& k, int precision,
             cudaStream_t stream, std::string* err, const CallOpts& opts);
void release_assembled(DevPlan* dev);
int assembled_precision(DevPlan* dev);
int matvec_assembled(const Plan& plan, DevPlan* dev, int precision, int dtype, int order,
                     int nrhs, const void* x, int64_t sxi, int64_t sxr, void* y, int64_t syi,
                     int64_t syr, void* ws, size_t ws_bytes, cudaStream_t stream,
                     std::string* err, const CallOpts& opts);
int dense_eval(const KernelDesc& k, int dim, const double* PR, int64_t nr,
               const double* PC, int64_t nc, double* out, std::string* err);
// device the plan lives on (-1 if not uploaded)
int device_of(const DevPlan* dev);
size_t adjoint_workspace_bytes(const Plan& plan, int precision, int nrhs);
// values (device, 3 doubles): f, df/dl, df/dsigma2; dX (device, natural
// order); Kx (strides of y) = K x, Ky (strides of x) = K y.  Any output may
// be null.
int adjoint(const Plan& plan, DevPlan* dev, const KernelDesc& k, int precision, int dtype,
            int nrhs, const void* x, int64_t sxi, int64_t sxr, const void* y, int64_t syi,
            int64_t syr, double* values, void* dX, int64_t sdi, int64_t sdd, void* Kx,
            void* Ky, void* ws, size_t ws_bytes, cudaStream_t stream, std::string* err,
            const CallOpts& opts);
// Launch shapes for (precision, kernel type, nrhs): out[FMCA_TUNE_*] (see
// include/fmca_gb300.h); the defaults if the autotuner has not run for it.
void tuned_config(DevPlan* dev, int precision, int type, int nrhs, int32_t* out);
// Stores launch shapes for (precision, kernel type, nrhs) as if tuned
// (validated; FMCA_ERR_INVALID_ARGUMENT when out of range).
int set_tuned_config(DevPlan* dev, int precision, int type, int nrhs, const int32_t* in,
                     std::string* err);
// re-uploads the point coordinates held by the plan (tree and boxes fixed)
int update_points(const Plan& plan, DevPlan* dev, std::string* err);
// true if the plan's device data for this precision lives on the current
// device (so a matvec needs no further device allocation besides workspace)
bool resident(const DevPlan* dev, int precision);
// device bytes the plan holds: uploaded data plus the workspace it owns
size_t device_bytes(const DevPlan* dev);
int profile(DevPlan* dev, double* stage_ms, int64_t* launches, std::string* err);
// The level sorter of Tree::build_with on the current device
// (h2_tree_gpu.cu): every level of a cluster tree as one segmented radix
// sort.
std::unique_ptr<LevelSorter> make_gpu_level_sorter();
// The block-pattern builder of Plan::build on the current device
// (h2_tree_gpu.cu): the block tree level by level, leaves sorted into the
// reference's depth-first order.
std::unique_ptr<PatternBuilder> make_gpu_pattern_builder();

}  // namespace gpu
}  // namespace fmca
