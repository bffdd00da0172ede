// ogs_batch.cpp -- batched gather-scatter over many handles (C ABI part of
// ogs_c.h): the device entry table and record prefix, CUDA-graph capture of
// the launch, and the launch-shape tuner.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "ogs_internal.hpp"

struct ogs_batch_s {
  int type = 0;
  int device = -1;
  unsigned flags = 0;
  std::vector<ogs_batch_entry> entries;
  std::vector<ogsgb::BatchEntry> host_entries;
  std::vector<int64_t> starts;         // prefix of warp records over entries
  std::vector<int> general;            // entries whose mesh has rows above degree 8
  ogsgb::BatchEntry* d_entries = nullptr;
  int64_t* d_starts = nullptr;
  int grid = 0;                        // 0 = one full wave
  cudaGraphExec_t graph = nullptr;
  cudaStream_t capture = nullptr;
};

namespace ogsgb {
namespace {

ogs_status cuda_err(cudaError_t e, const char* fn, const char* what) {
  if (e == cudaSuccess) return OGS_OK;
  cudaGetLastError();
  return set_error(e == cudaErrorMemoryAllocation ? OGS_ENOMEM : OGS_EDEVICE,
                   std::string(fn) + ": " + what + ": " + cudaGetErrorString(e));
}

// Members read and written per transpose, as pattern_for in ogs_capi.cpp.
void fill_pattern(const ogs_handle_s* h, int trans, BatchEntry& e) {
  e.gather_n = e.scatter_n = e.limit_n = 0;
  if (h->kind == OGS_SIGNED) {
    if (trans == OGS_TRANS) e.scatter_n = e.limit_n = 1;
    else if (trans == OGS_NOTRANS) e.gather_n = 1;
  }
  e.use_mask = (e.gather_n || e.scatter_n) && h->kind == OGS_SIGNED;
}

int launch_batch(const ogs_batch_s* b, void* stream) {
  const int n = static_cast<int>(b->entries.size());
  const int64_t nitems = b->starts.back();
  switch (b->type) {
    case OGS_FLOAT: return launch_batch_f32(b->d_entries, b->d_starts, n, nitems, b->grid, stream);
    case OGS_DOUBLE: return launch_batch_f64(b->d_entries, b->d_starts, n, nitems, b->grid, stream);
    case OGS_INT32: return launch_batch_i32(b->d_entries, b->d_starts, n, nitems, b->grid, stream);
    default: return launch_batch_i64(b->d_entries, b->d_starts, n, nitems, b->grid, stream);
  }
}

// Rows above degree 8 of the entries that have any: one direct launch each.
int launch_general(const ogs_batch_s* b, void* stream) {
  for (int i : b->general) {
    const ogs_batch_entry& be = b->entries[i];
    const ogs_handle_s* h = be.h;
    DevMaps g = h->dmaps;
    g.nwtiles = 0;
    g.ntiles = g.ngtiles;
    FieldArgs f{};
    f.v = be.d_v;
    f.K = be.k;
    Pattern pat{b->host_entries[i].gather_n, b->host_entries[i].scatter_n, b->host_entries[i].limit_n};
    int e = 0;
    switch (b->type) {
      case OGS_FLOAT: e = launch_f32(g, f, kModeGS, be.op, pat, stream); break;
      case OGS_DOUBLE: e = launch_f64(g, f, kModeGS, be.op, pat, stream); break;
      case OGS_INT32: e = launch_i32(g, f, kModeGS, be.op, pat, stream); break;
      default: e = launch_i64(g, f, kModeGS, be.op, pat, stream); break;
    }
    if (e) return e;
  }
  return 0;
}

int launch_all(const ogs_batch_s* b, void* stream) {
  int e = launch_batch(b, stream);
  if (!e) e = launch_general(b, stream);
  return e;
}

void drop_graph(ogs_batch_s* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
}

}  // namespace
}  // namespace ogsgb

using namespace ogsgb;

extern "C" {

ogs_status ogs_batch_create(ogs_batch* out, int type, const ogs_batch_entry* entries, int n, unsigned flags) {
  const char* fn = "ogs_batch_create";
  if (!out) return set_error(OGS_EINVAL, "ogs_batch_create: out is NULL");
  *out = nullptr;
  if (type < OGS_FLOAT || type > OGS_INT64) return set_error(OGS_EINVAL, "ogs_batch_create: unknown type");
  if (n < 1 || !entries) return set_error(OGS_EINVAL, "ogs_batch_create: need at least one entry");
  int dev = 0;
  ogs_status s;
  if ((s = cuda_err(cudaGetDevice(&dev), fn, "device")) != OGS_OK) return s;
  ogs_batch_s* b = new (std::nothrow) ogs_batch_s();
  if (!b) return set_error(OGS_ENOMEM, "ogs_batch_create: out of host memory");
  b->type = type;
  b->device = dev;
  b->flags = flags;
  b->entries.assign(entries, entries + n);
  b->starts.assign(1, 0);
  for (int i = 0; i < n; ++i) {
    const ogs_batch_entry& e = entries[i];
    const char* bad = nullptr;
    if (!e.h) bad = "handle is NULL";
    else if (e.h->host_only) bad = "handle was set up host-only";
    else if (!e.h->distinct_cols) bad = "a local node appears in two rows of this operator's map";
    else if (e.h->device != dev) bad = "handle lives on another device";
    else if (e.k < 1) bad = "k must be >= 1";
    else if (e.op < OGS_ADD || e.op > OGS_MIN) bad = "unknown op";
    else if (e.trans < OGS_SYM || e.trans > OGS_TRANS) bad = "unknown transpose";
    else if (!e.d_v && e.h->N > 0) bad = "field is NULL";
    if (bad) {
      delete b;
      return set_error(OGS_EINVAL, std::string(fn) + ": entry " + std::to_string(i) + ": " + bad);
    }
    BatchEntry be{};
    be.recs = e.h->dmaps.wrecs;
    be.wemask = e.h->dmaps.wemask;
    be.v = e.d_v;
    be.K = e.k;
    be.op = e.op;
    fill_pattern(e.h, e.trans, be);
    b->host_entries.push_back(be);
    b->starts.push_back(b->starts.back() + static_cast<int64_t>(e.h->dmaps.nwtiles) * e.k);
    if (e.h->dmaps.ngtiles > 0) b->general.push_back(i);
  }
  if ((s = cuda_err(dev_malloc(&b->d_entries, sizeof(BatchEntry) * n), fn, "malloc")) != OGS_OK ||
      (s = cuda_err(dev_malloc(&b->d_starts, sizeof(int64_t) * (n + 1)), fn, "malloc")) != OGS_OK ||
      (s = cuda_err(cudaMemcpy(b->d_entries, b->host_entries.data(), sizeof(BatchEntry) * n,
                               cudaMemcpyHostToDevice), fn, "copy")) != OGS_OK ||
      (s = cuda_err(cudaMemcpy(b->d_starts, b->starts.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice),
                    fn, "copy")) != OGS_OK) {
    ogs_batch_free(b);
    return s;
  }
  *out = b;
  return OGS_OK;
}

ogs_status ogs_batch_free(ogs_batch b) {
  if (!b) return OGS_OK;
  drop_graph(b);
  if (b->capture) cudaStreamDestroy(b->capture);
  if (b->d_entries) dev_free(b->d_entries);
  if (b->d_starts) dev_free(b->d_starts);
  delete b;
  return OGS_OK;
}

ogs_status ogs_batch_set_fields(ogs_batch b, void* const* d_vs, void* stream) {
  const char* fn = "ogs_batch_set_fields";
  if (!b || !d_vs) return set_error(OGS_EINVAL, "ogs_batch_set_fields: NULL argument");
  for (size_t i = 0; i < b->entries.size(); ++i) {
    if (!d_vs[i] && b->entries[i].h->N > 0) return set_error(OGS_EINVAL, "ogs_batch_set_fields: a field is NULL");
    b->entries[i].d_v = d_vs[i];
    b->host_entries[i].v = d_vs[i];
  }
  // the direct launches of rows above degree 8 bake the field into the graph
  if (!b->general.empty()) drop_graph(b);
  ogs_status s = cuda_err(cudaMemcpyAsync(b->d_entries, b->host_entries.data(),
                                          sizeof(BatchEntry) * b->host_entries.size(), cudaMemcpyHostToDevice,
                                          static_cast<cudaStream_t>(stream)),
                          fn, "copy");
  if (s != OGS_OK) return s;
  // the host copy must outlive the asynchronous copy
  return cuda_err(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)), fn, "synchronize");
}

ogs_status ogs_batch_gather_scatter(ogs_batch b, void* stream) {
  const char* fn = "ogs_batch_gather_scatter";
  if (!b) return set_error(OGS_EINVAL, "ogs_batch_gather_scatter: batch is NULL");
  int dev = -1;
  ogs_status s;
  if ((s = cuda_err(cudaGetDevice(&dev), fn, "device")) != OGS_OK) return s;
  if (dev != b->device) return set_error(OGS_EINVAL, "ogs_batch_gather_scatter: batch lives on another device");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!(b->flags & OGS_BATCH_GRAPH)) {
    const int e = launch_all(b, stream);
    return e ? cuda_err(static_cast<cudaError_t>(e), fn, "launch") : OGS_OK;
  }
  if (!b->graph) {
    if (!b->capture && (s = cuda_err(cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking), fn,
                                     "stream")) != OGS_OK)
      return s;
    if ((s = cuda_err(cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal), fn, "capture")) !=
        OGS_OK)
      return s;
    const int e = launch_all(b, b->capture);
    cudaGraph_t g = nullptr;
    const cudaError_t ec = cudaStreamEndCapture(b->capture, &g);
    if (e) {
      if (g) cudaGraphDestroy(g);
      return cuda_err(static_cast<cudaError_t>(e), fn, "launch during capture");
    }
    if ((s = cuda_err(ec, fn, "end capture")) != OGS_OK) return s;
    s = cuda_err(cudaGraphInstantiate(&b->graph, g, 0), fn, "instantiate");
    cudaGraphDestroy(g);
    if (s != OGS_OK) return s;
  }
  return cuda_err(cudaGraphLaunch(b->graph, st), fn, "graph launch");
}

ogs_status ogs_batch_tune(ogs_batch b, void* stream, int* chosen) {
  const char* fn = "ogs_batch_tune";
  if (!b) return set_error(OGS_EINVAL, "ogs_batch_tune: batch is NULL");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  int sms = 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, b->device);
  // candidate launch shapes: 1..6 CTAs per SM of the persistent kernel
  std::vector<int> cand;
  for (int c = 1; c <= 6; ++c) cand.push_back(c * sms);
  cudaEvent_t e0, e1;
  ogs_status s;
  if ((s = cuda_err(cudaEventCreate(&e0), fn, "event")) != OGS_OK) return s;
  if ((s = cuda_err(cudaEventCreate(&e1), fn, "event")) != OGS_OK) { cudaEventDestroy(e0); return s; }
  // the fields are updated in place by every trial; timing only
  float best = 1e30f;
  int best_grid = 0;
  const int saved = b->grid;
  for (int g : cand) {
    b->grid = g;
    float tsum = 0.f;
    for (int rep = 0; rep < 4; ++rep) {
      cudaEventRecord(e0, st);
      const int e = launch_all(b, st);
      cudaEventRecord(e1, st);
      if (e) { s = cuda_err(static_cast<cudaError_t>(e), fn, "launch"); break; }
      cudaEventSynchronize(e1);
      float ms = 0.f;
      cudaEventElapsedTime(&ms, e0, e1);
      if (rep > 0) tsum += ms;  // first run warms up
    }
    if (s != OGS_OK) break;
    if (tsum < best) { best = tsum; best_grid = g; }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (s != OGS_OK) { b->grid = saved; return s; }
  b->grid = best_grid;
  drop_graph(b);
  if (chosen) *chosen = best_grid;
  return OGS_OK;
}

ogs_status ogs_batch_items(ogs_batch b, int64_t* items) {
  if (!b || !items) return set_error(OGS_EINVAL, "ogs_batch_items: NULL argument");
  *items = b->starts.back();
  return OGS_OK;
}

}  // extern "C"
