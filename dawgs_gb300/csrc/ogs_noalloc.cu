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
// the last call left there is never read.  The cached address of the array
// belongs to the device's primary context: after a cudaDeviceReset the entry
// point must not be called again in that process.
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
// per device (with that device current) and cached for the life of the
// process.  A cudaDeviceReset destroys the context that address belongs to:
// after one, this entry point must not be called again in the process.
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
  if (k < 1) return set_error(OGS_EINVAL, std::string(fn) + ": k must be >= 1");
  if (type < OGS_FLOAT || type > OGS_INT64) return set_error(OGS_EINVAL, std::string(fn) + ": unknown type");
  // The field must fit the array: N*k*sizeof(T) <= kNoAllocStageBytes, tested
  // by division so that no product can wrap around.
  const size_t ts = type_size(type);
  if (h->N > 0 && static_cast<size_t>(k) > kNoAllocStageBytes / ts / static_cast<size_t>(h->N))
    return set_error(OGS_ERANGE, std::string(fn) + ": the field (" + std::to_string(h->N) + " nodes x k=" +
                                     std::to_string(k) + " x " + std::to_string(ts) + " bytes) is larger than the " +
                                     std::to_string(kNoAllocStageBytes) +
                                     "-byte staging array; use ogs_gather_scatter_host");
  // the same refusals as ogs_gather_scatter_host (host-only and gslib handles,
  // a local node in two rows, unknown op or transpose, another device)
  ogs_status s = check_common(h, k, type, trans, fn);
  if (s == OGS_OK) s = check_writes(h, fn);
  if (s == OGS_OK) s = check_op(op, fn);
  if (s != OGS_OK) return s;
  if (h->N == 0) return OGS_OK;
  if (!v) return set_error(OGS_EINVAL, std::string(fn) + ": v is NULL");
  const size_t bytes = static_cast<size_t>(h->N) * static_cast<size_t>(k) * ts;
  const int dev = h->device;
  if (dev < 0 || dev >= kMaxDevices) return set_error(OGS_ERANGE, std::string(fn) + ": device index too large");
  void* stage = nullptr;
  if ((s = stage_address(dev, &stage)) != OGS_OK) return s;

  cudaStream_t st = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if ((e = cudaMemcpyAsync(stage, v, bytes, cudaMemcpyHostToDevice, st)) != cudaSuccess) return cuda_fail(e, "copy in");
  FieldArgs f{};
  f.v = stage;
  f.K = k;
  int le = 0;
  const Pattern pat = pattern_for(h, kModeGS, trans);
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
