// ogs_alloc.cpp -- every device and page-locked host allocation the library
// makes goes through here, so that a test can make the n-th one fail (the
// OGS_ENOMEM paths are exercised on the host, without exhausting a GPU) and
// can count what is still held after a failed call (nothing may leak).
#include <atomic>
#include <mutex>
#include <unordered_map>

#include <cuda_runtime.h>

#include "ogs_internal.hpp"

namespace ogsgb {
namespace {

// > 0: allocations left before the injected failure (1 = the next one fails)
std::atomic<int64_t> g_fail_countdown{0};

struct Ledger {
  std::mutex mu;
  std::unordered_map<void*, size_t> dev, host;
  int64_t dev_bytes = 0, host_bytes = 0;
};

Ledger& ledger() {
  static Ledger* l = new Ledger();  // never destroyed: frees may run during exit
  return *l;
}

bool injected_failure() {
  int64_t c = g_fail_countdown.load();
  while (c > 0) {
    if (g_fail_countdown.compare_exchange_weak(c, c - 1)) return c == 1;
  }
  return false;
}

}  // namespace

cudaError_t dev_malloc_raw(void** p, size_t bytes) {
  *p = nullptr;
  if (injected_failure()) return cudaErrorMemoryAllocation;
  const cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    return e;
  }
  Ledger& l = ledger();
  std::lock_guard<std::mutex> g(l.mu);
  l.dev[*p] = bytes;
  l.dev_bytes += static_cast<int64_t>(bytes);
  return e;
}

void dev_free(void* p) {
  if (!p) return;
  {
    Ledger& l = ledger();
    std::lock_guard<std::mutex> g(l.mu);
    auto it = l.dev.find(p);
    if (it != l.dev.end()) {
      l.dev_bytes -= static_cast<int64_t>(it->second);
      l.dev.erase(it);
    }
  }
  cudaFree(p);
}

cudaError_t host_malloc_raw(void** p, size_t bytes) {
  *p = nullptr;
  if (injected_failure()) return cudaErrorMemoryAllocation;
  const cudaError_t e = cudaMallocHost(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    return e;
  }
  Ledger& l = ledger();
  std::lock_guard<std::mutex> g(l.mu);
  l.host[*p] = bytes;
  l.host_bytes += static_cast<int64_t>(bytes);
  return e;
}

void host_free(void* p) {
  if (!p) return;
  {
    Ledger& l = ledger();
    std::lock_guard<std::mutex> g(l.mu);
    auto it = l.host.find(p);
    if (it != l.host.end()) {
      l.host_bytes -= static_cast<int64_t>(it->second);
      l.host.erase(it);
    }
  }
  cudaFreeHost(p);
}

}  // namespace ogsgb

extern "C" {

ogs_status ogs_debug_fail_alloc(int64_t nth) {
  if (nth < 0) return ogsgb::set_error(OGS_EINVAL, "ogs_debug_fail_alloc: nth must be >= 0");
  ogsgb::g_fail_countdown.store(nth);
  return OGS_OK;
}

ogs_status ogs_debug_allocations(int64_t* device_blocks, int64_t* device_bytes, int64_t* host_blocks,
                                 int64_t* host_bytes) {
  ogsgb::Ledger& l = ogsgb::ledger();
  std::lock_guard<std::mutex> g(l.mu);
  if (device_blocks) *device_blocks = static_cast<int64_t>(l.dev.size());
  if (device_bytes) *device_bytes = l.dev_bytes;
  if (host_blocks) *host_blocks = static_cast<int64_t>(l.host.size());
  if (host_bytes) *host_bytes = l.host_bytes;
  return OGS_OK;
}

}  // extern "C"
