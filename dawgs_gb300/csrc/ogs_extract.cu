// ogs_extract.cu -- packing of exchange send buffers.
//
// out[n*k + c] = q[ids[n]*k + c] for n < N, c < k: the reference's extract
// kernel (libs/ogs/okl/ogsKernels.okl:167-177), which the all-to-all exchange
// runs on the halo buffer before sending (ogsAllToAll.cpp:126-131, and the
// host form at 47-50).  One thread per output element, so the writes are
// coalesced; the reads follow ids.
#include <string>

#include <cuda_runtime.h>

#include "ogs_internal.hpp"

using namespace ogsgb;

namespace {

template <typename T>
__global__ void extract_kernel(int64_t total, int k, const int32_t* __restrict__ ids, const T* __restrict__ q,
                               T* __restrict__ out) {
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
       i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
    const int64_t n = i / k;
    const int c = static_cast<int>(i - n * k);
    out[i] = q[static_cast<int64_t>(ids[n]) * k + c];
  }
}

template <typename T>
cudaError_t launch_extract(int64_t N, int k, const int32_t* ids, const void* q, void* out, cudaStream_t s) {
  const int64_t total = N * k;
  int64_t blocks = (total + 255) / 256;
  if (blocks > 152 * 32) blocks = 152 * 32;
  extract_kernel<T><<<static_cast<unsigned>(blocks), 256, 0, s>>>(total, k, ids, static_cast<const T*>(q),
                                                                   static_cast<T*>(out));
  return cudaGetLastError();
}

}  // namespace

extern "C" ogs_status ogs_extract(int64_t N, int k, int type, const int32_t* d_ids, const void* d_q, void* d_out,
                                  void* stream) {
  const char* fn = "ogs_extract";
  if (N < 0) return set_error(OGS_EINVAL, std::string(fn) + ": N < 0");
  if (k < 1) return set_error(OGS_EINVAL, std::string(fn) + ": k must be >= 1");
  if (type < OGS_FLOAT || type > OGS_INT64) return set_error(OGS_EINVAL, std::string(fn) + ": unknown type");
  if (N == 0) return OGS_OK;
  if (!d_ids || !d_q || !d_out) return set_error(OGS_EINVAL, std::string(fn) + ": NULL buffer");
  if (N > INT32_MAX) return set_error(OGS_ERANGE, std::string(fn) + ": N exceeds 32-bit device indices");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  switch (type) {
    case OGS_FLOAT: e = launch_extract<float>(N, k, d_ids, d_q, d_out, s); break;
    case OGS_DOUBLE: e = launch_extract<double>(N, k, d_ids, d_q, d_out, s); break;
    case OGS_INT32: e = launch_extract<int32_t>(N, k, d_ids, d_q, d_out, s); break;
    default: e = launch_extract<long long>(N, k, d_ids, d_q, d_out, s); break;
  }
  if (e != cudaSuccess) return set_error(OGS_EDEVICE, std::string(fn) + ": launch: " + cudaGetErrorString(e));
  return OGS_OK;
}
