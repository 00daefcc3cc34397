// fmca_matvec_static_scratch: the H2 matvec for callers that cannot allocate
// device memory while they run it.
//
// Some callers cannot call cudaMalloc on their working path: a host
// application may own all of the GPU's memory through its own allocator or a
// fixed budget and forbid plugins from allocating, and latency-bound loops
// cannot afford cudaMalloc / cudaFree, which can synchronise the device and
// take milliseconds.  This entry point takes its scratch (the workspace that
// fmca_matvec otherwise gets from the caller or allocates itself) from the
// fixed device array below, so a call allocates nothing; the caller still
// passes x and y.
//
// The array is a file-scope __device__ variable of kStaticScratchBytes
// (64 MiB).  Every GPU that loads this part of the library holds it until the
// process exits.  Host code cannot use the array's name as a device address,
// so the first call on each device looks the address up with
// cudaGetSymbolAddress (with that device current) and caches it; that first
// call should therefore come before any stream capture.  All calls share the
// one array, which keeps the contents of the last call: the matvec writes
// every part of its scratch before reading it and clears what must start at
// zero (the column maxima) itself.  Calls whose GPU work overlaps (on
// different streams, or from different threads) race on the array and give
// wrong results; serialise them.
#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/fmca_gb300.h"
#include "c_api_internal.h"
#include "h2_gpu.h"

namespace {

constexpr size_t kStaticScratchBytes = size_t(64) << 20;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

std::mutex g_scratch_mu;
void* g_scratch_addr[kMaxDevices] = {};

// device address of the scratch array on the current device (looked up once
// per device)
fmca_status scratch_address(void** out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess)
    return fmca::capi::fail(FMCA_ERR_CUDA, std::string("cudaGetDevice failed: ") +
                                               cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices)
    return fmca::capi::fail(FMCA_ERR_UNSUPPORTED, "device index out of range");
  std::lock_guard<std::mutex> lock(g_scratch_mu);
  if (!g_scratch_addr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess || !p)
      return fmca::capi::fail(FMCA_ERR_CUDA,
                              std::string("cudaGetSymbolAddress of the static scratch failed: ") +
                                  cudaGetErrorString(e));
    g_scratch_addr[dev] = p;
  }
  *out = g_scratch_addr[dev];
  return FMCA_OK;
}

}  // namespace

extern "C" fmca_status fmca_matvec_static_scratch(
    fmca_plan* p, const fmca_kernel_desc* kernel, int precision, int dtype, int order,
    int nrhs, const void* x, int64_t x_stride_i, int64_t x_stride_r, void* y,
    int64_t y_stride_i, int64_t y_stride_r, void* stream) {
  fmca_status s =
      fmca::capi::check_matvec_args(p, kernel, precision, dtype, order, nrhs, x, y);
  if (s != FMCA_OK) return s;
  const size_t need = fmca::gpu::workspace_bytes(p->plan, precision, nrhs);
  if (need > kStaticScratchBytes)
    return fmca::capi::fail(
        FMCA_ERR_UNSUPPORTED,
        "fmca_matvec_static_scratch: this plan needs " + std::to_string(need) +
            " bytes of scratch for " + std::to_string(nrhs) +
            " right-hand sides, more than the " + std::to_string(kStaticScratchBytes) +
            " bytes of the static scratch; use fmca_matvec with a workspace");
  if (!fmca::gpu::resident(p->dev, precision))
    return fmca::capi::fail(
        FMCA_ERR_INVALID_ARGUMENT,
        "fmca_matvec_static_scratch: the plan is not resident on the current device for "
        "this precision; it becomes resident (allocating once) on its first fmca_matvec "
        "or fmca_matvec_host call there");
  void* scratch = nullptr;
  s = scratch_address(&scratch);
  if (s != FMCA_OK) return s;
  // no stage events (they would be created, that is allocated, on first
  // use) and no tuning (its events are allocated too): the launch shapes
  // tuned earlier for this key by fmca_matvec, if any, else the defaults
  fmca::gpu::CallOpts opts = fmca::capi::call_opts(p);
  opts.profile = false;
  opts.autotune = false;
  std::string err;
  const int st = fmca::gpu::matvec(p->plan, p->dev, fmca::capi::to_desc(kernel), precision,
                                   dtype, order, nrhs, x, x_stride_i, x_stride_r, y,
                                   y_stride_i, y_stride_r, scratch, kStaticScratchBytes,
                                   (cudaStream_t)stream, &err, opts);
  if (st != FMCA_OK) return fmca::capi::fail((fmca_status)st, err);
  return FMCA_OK;
}
