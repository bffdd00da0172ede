// ogs_noalloc.cu -- host-buffer GatherScatter that allocates nothing.
//
// ogs_gather_scatter_host copies the caller's host field into a device
// staging buffer that the handle allocates with cudaMalloc the first time a
// field of that size comes by.  Some callers cannot let a library allocate
// device memory once they are running: latency-critical loops (cudaMalloc
// and cudaFree synchronise the device and take unpredictable time),
// applications whose device memory is owned by a framework's caching
// allocator (a second allocator fragments it and can fail where the
// framework would have succeeded), and services that fix their memory
// footprint at start-up.  ogs_gather_scatter_host_noalloc gives them the same
// operation with the staging buffer in a fixed device array that exists as
// soon as the library is loaded: no cudaMalloc, cudaFree or allocating
// library call happens inside it.
//
// The array holds kNoAllocStageBytes (32 MiB) per device for as long as the
// process runs, whether or not the entry point is used.  Every call shares
// it, so calls that overlap on the GPU (from two threads, or on two streams
// without ordering between them) race and corrupt each other's fields.  Each
// call overwrites the bytes it uses with the caller's field before the
// kernel reads them, so nothing in the array has to start at zero and what
// the last call left there is never read.
#include <cstddef>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

#include "ogs_internal.hpp"

namespace ogsgb {
namespace {

constexpr size_t kNoAllocStageBytes = size_t(32) << 20;
constexpr int kMaxDevices = 64;

// The staging array.  In host code this name is only a stand-in for the
// device symbol; its device address comes from cudaGetSymbolAddress.
__device__ __align__(256) unsigned char g_noalloc_stage[kNoAllocStageBytes];

std::mutex g_stage_mu;
void* g_stage_addr[kMaxDevices] = {};

// Device address of the staging array on the current device, looked up once
// per device (with that device current) and cached.
ogs_status stage_address(int dev, void** out) {
  std::lock_guard<std::mutex> g(g_stage_mu);
  if (!g_stage_addr[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_stage);
    if (e != cudaSuccess || !p)
      return set_error(OGS_EDEVICE, std::string("ogs_gather_scatter_host_noalloc: cudaGetSymbolAddress: ") +
                                        cudaGetErrorString(e));
    g_stage_addr[dev] = p;
  }
  *out = g_stage_addr[dev];
  return OGS_OK;
}

ogs_status cuda_fail(cudaError_t e, const char* what) {
  return set_error(OGS_EDEVICE, std::string("ogs_gather_scatter_host_noalloc: ") + what + ": " +
                                    cudaGetErrorString(e));
}

}  // namespace
}  // namespace ogsgb

using namespace ogsgb;

extern "C" ogs_status ogs_gather_scatter_host_noalloc(ogs_handle h, void* v, int k, int type, int op, int trans,
                                                      void* stream) {
  const char* fn = "ogs_gather_scatter_host_noalloc";
  if (!h) return set_error(OGS_EINVAL, std::string(fn) + ": handle is NULL");
  if (h->host_only) return set_error(OGS_EINVAL, std::string(fn) + ": handle was set up host-only");
  if (!h->distinct_cols)
    return set_error(OGS_EINVAL, std::string(fn) + ": a local node appears in two rows of this operator's map");
  if (k < 1) return set_error(OGS_EINVAL, std::string(fn) + ": k must be >= 1");
  if (type < OGS_FLOAT || type > OGS_INT64) return set_error(OGS_EINVAL, std::string(fn) + ": unknown type");
  if (op < OGS_ADD || op > OGS_MIN) return set_error(OGS_EINVAL, std::string(fn) + ": unknown op");
  if (trans < OGS_SYM || trans > OGS_TRANS) return set_error(OGS_EINVAL, std::string(fn) + ": unknown transpose");
  if (h->N == 0) return OGS_OK;
  if (!v) return set_error(OGS_EINVAL, std::string(fn) + ": v is NULL");
  const size_t ts = (type == OGS_DOUBLE || type == OGS_INT64) ? 8 : 4;
  const size_t bytes = static_cast<size_t>(h->N) * static_cast<size_t>(k) * ts;
  if (bytes > kNoAllocStageBytes)
    return set_error(OGS_ERANGE, std::string(fn) + ": the field takes " + std::to_string(bytes) +
                                     " bytes, more than the " + std::to_string(kNoAllocStageBytes) +
                                     "-byte staging array; use ogs_gather_scatter_host");
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(e, "cudaGetDevice");
  if (dev != h->device)
    return set_error(OGS_EINVAL, std::string(fn) + ": handle lives on device " + std::to_string(h->device) +
                                     ", current device is " + std::to_string(dev));
  if (dev < 0 || dev >= kMaxDevices) return set_error(OGS_ERANGE, std::string(fn) + ": device index too large");
  void* stage = nullptr;
  ogs_status s = stage_address(dev, &stage);
  if (s != OGS_OK) return s;

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if ((e = cudaMemcpyAsync(stage, v, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess) return cuda_fail(e, "copy in");
  // Members read and written, as for ogs_gather_scatter (ogsOperator.cpp:321-339).
  Pattern pat{0, 0, 0};
  if (h->kind == OGS_SIGNED) {
    if (trans == OGS_TRANS) pat = Pattern{0, 1, 1};
    else if (trans == OGS_NOTRANS) pat = Pattern{1, 0, 0};
  }
  FieldArgs f{};
  f.v = stage;
  f.K = k;
  int le = 0;
  switch (type) {
    case OGS_FLOAT: le = launch_f32(h->dmaps, f, kModeGS, op, pat, stream); break;
    case OGS_DOUBLE: le = launch_f64(h->dmaps, f, kModeGS, op, pat, stream); break;
    case OGS_INT32: le = launch_i32(h->dmaps, f, kModeGS, op, pat, stream); break;
    default: le = launch_i64(h->dmaps, f, kModeGS, op, pat, stream); break;
  }
  if (le != 0) return cuda_fail(static_cast<cudaError_t>(le), "kernel launch");
  if ((e = cudaMemcpyAsync(v, stage, bytes, cudaMemcpyDeviceToHost, st)) != cudaSuccess) return cuda_fail(e, "copy out");
  if ((e = cudaStreamSynchronize(st)) != cudaSuccess) return cuda_fail(e, "synchronize");
  return OGS_OK;
}
