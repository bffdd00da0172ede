// ogs_batch.cpp -- batched gather-scatter over many handles (C ABI part of
// ogs_c.h): the device entry table and record prefix, CUDA-graph capture of
// the launch, and the tuner with its cache.
//
// A batch runs as one CUDA graph: the entries below a size threshold go to one
// persistent launch of the batched kernel (ogs_batch.cuh, the register
// pipeline over the entries' (record, component) items), and
// the entries at or above it each run the single-mesh kernel (ogs_async.cuh,
// the cp.async ring) on their own launch, spread over parallel branches of
// the graph so that they run beside the persistent launch.  The tuner chooses
// the threshold, the number of branches, and the persistent launch's block
// size and CTAs per SM by timing candidates on scratch copies of the fields
// (the caller's fields are never touched), and caches its choice under a key
// made of the value type, the k range and the histogram of entry sizes.
#include <algorithm>
#include <chrono>
#include <cstring>
#include <map>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "ogs_internal.hpp"
#include "ogs_trace.hpp"

struct ogs_batch_s {
  int type = 0;
  int device = -1;
  unsigned flags = 0;
  std::vector<ogs_batch_entry> entries;
  std::vector<ogsgb::BatchEntry> host_entries;  // every entry, field and pattern filled in
  int plain = 1;  // no entry has N masks, a store mode or a row limit
  std::vector<int64_t> items;                   // per entry: warp records x k
  ogs_batch_config cfg{};
  // derived from cfg
  std::vector<int> batched, solo;               // entry indices
  std::vector<ogsgb::BatchEntry> batched_entries;
  std::vector<int64_t> starts;                  // prefix of items over the batched entries
  std::vector<int> general;                     // batched entries with rows above degree 8
  ogsgb::BatchEntry* d_entries = nullptr;       // room for every entry
  int64_t* d_starts = nullptr;
  cudaGraphExec_t graph = nullptr;
  cudaStream_t capture = nullptr;
  std::vector<cudaStream_t> branches;           // streams of the single-mesh launches
  std::vector<cudaEvent_t> joins;               // fork event, then one per branch
};

namespace ogsgb {
namespace {

constexpr int kMaxBranches = 8;

ogs_status cuda_err(cudaError_t e, const char* fn, const char* what) {
  if (e == cudaSuccess) return OGS_OK;
  cudaGetLastError();
  return set_error(e == cudaErrorMemoryAllocation ? OGS_ENOMEM : OGS_EDEVICE,
                   std::string(fn) + ": " + what + ": " + cudaGetErrorString(e));
}

void fill_pattern(const ogs_handle_s* h, int trans, BatchEntry& e) {
  const Pattern p = pattern_for(h, kModeGS, trans);
  e.gather_n = p.gather_n;
  e.scatter_n = p.scatter_n;
  e.limit_n = p.limit_n;
  e.use_mask = (e.gather_n || e.scatter_n) && h->kind == OGS_SIGNED;
}

void drop_graph(ogs_batch_s* b) {
  if (b->graph) cudaGraphExecDestroy(b->graph);
  b->graph = nullptr;
}

// Split the entries by the configuration and upload the persistent launch's tables.
ogs_status apply_config(ogs_batch_s* b, const BatchEntry* fields, cudaStream_t st, const char* fn) {
  b->batched.clear();
  b->solo.clear();
  b->batched_entries.clear();
  b->general.clear();
  b->starts.assign(1, 0);
  for (size_t i = 0; i < b->entries.size(); ++i) {
    if (b->cfg.solo_items > 0 && b->items[i] >= b->cfg.solo_items) {
      b->solo.push_back(static_cast<int>(i));
      continue;
    }
    b->batched.push_back(static_cast<int>(i));
    b->batched_entries.push_back(fields[i]);
    b->starts.push_back(b->starts.back() + b->items[i]);
    if (b->entries[i].h->dmaps.ngtiles > 0) b->general.push_back(static_cast<int>(i));
  }
  drop_graph(b);
  const size_t n = b->batched_entries.size();
  ogs_status s = OGS_OK;
  if (n) {
    s = cuda_err(cudaMemcpyAsync(b->d_entries, b->batched_entries.data(), sizeof(BatchEntry) * n,
                                 cudaMemcpyHostToDevice, st), fn, "copy");
    if (s == OGS_OK)
      s = cuda_err(cudaMemcpyAsync(b->d_starts, b->starts.data(), sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice,
                                   st), fn, "copy");
  }
  // the host tables must outlive the asynchronous copies
  if (s == OGS_OK) s = cuda_err(cudaStreamSynchronize(st), fn, "synchronize");
  return s;
}

int launch_typed_entry(int type, const ogs_handle_s* h, void* v, int k, int op, const BatchEntry& be, bool general_only,
                       cudaStream_t st) {
  DevMaps m = h->dmaps;
  if (general_only) {
    m.nwtiles = 0;
    m.ntiles = m.ngtiles;
  }
  FieldArgs f{};
  f.v = v;
  f.K = k;
  const Pattern pat{be.gather_n, be.scatter_n, be.limit_n};
  switch (type) {
    case OGS_FLOAT: return launch_f32(m, f, kModeGS, op, pat, st);
    case OGS_DOUBLE: return launch_f64(m, f, kModeGS, op, pat, st);
    case OGS_INT32: return launch_i32(m, f, kModeGS, op, pat, st);
    default: return launch_i64(m, f, kModeGS, op, pat, st);
  }
}

ogs_status ensure_branches(ogs_batch_s* b, int want, const char* fn) {
  ogs_status s;
  while (static_cast<int>(b->branches.size()) < want) {
    cudaStream_t x = nullptr;
    if ((s = cuda_err(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking), fn, "stream")) != OGS_OK) return s;
    b->branches.push_back(x);
  }
  while (static_cast<int>(b->joins.size()) < want + 1) {
    cudaEvent_t e = nullptr;
    if ((s = cuda_err(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), fn, "event")) != OGS_OK) return s;
    b->joins.push_back(e);
  }
  return OGS_OK;
}

// Everything of one batch call on `st`, with `fields` giving each entry's field
// (the caller's, or the tuner's scratch copies); the single-mesh launches fork
// onto the branch streams and join back.
int launch_all(ogs_batch_s* b, const BatchEntry* fields, cudaStream_t st) {
  int e = 0;
  const int nbr = b->solo.empty() ? 0 : std::max(1, std::min(b->cfg.solo_streams, kMaxBranches));
  if (nbr) {
    e = cudaEventRecord(b->joins[0], st);
    for (int j = 0; !e && j < nbr; ++j) e = cudaStreamWaitEvent(b->branches[j], b->joins[0], 0);
    for (size_t q = 0; !e && q < b->solo.size(); ++q) {
      const int i = b->solo[q];
      const ogs_batch_entry& be = b->entries[i];
      e = launch_typed_entry(b->type, be.h, fields[i].v, be.k, be.op, fields[i], false, b->branches[q % nbr]);
    }
  }
  const int n = static_cast<int>(b->batched.size());
  if (!e && n) {
    // the persistent launch reads its field pointers from the device table
    const int64_t nitems = b->starts.back();
    const int grid = b->cfg.ctas_per_sm > 0 ? b->cfg.ctas_per_sm * std::max(1, b->cfg.sms) : 0;
    switch (b->type) {
      case OGS_FLOAT: e = launch_batch_f32(b->d_entries, b->d_starts, n, nitems, grid, b->cfg.block, b->cfg.occupancy,
                                             b->cfg.pipeline, b->plain, st); break;
      case OGS_DOUBLE: e = launch_batch_f64(b->d_entries, b->d_starts, n, nitems, grid, b->cfg.block, b->cfg.occupancy,
                                             b->cfg.pipeline, b->plain, st); break;
      case OGS_INT32: e = launch_batch_i32(b->d_entries, b->d_starts, n, nitems, grid, b->cfg.block, b->cfg.occupancy,
                                             b->cfg.pipeline, b->plain, st); break;
      default: e = launch_batch_i64(b->d_entries, b->d_starts, n, nitems, grid, b->cfg.block, b->cfg.occupancy,
                                             b->cfg.pipeline, b->plain, st); break;
    }
    for (size_t q = 0; !e && q < b->general.size(); ++q) {
      const int i = b->general[q];
      const ogs_batch_entry& be = b->entries[i];
      e = launch_typed_entry(b->type, be.h, fields[i].v, be.k, be.op, fields[i], true, st);
    }
  }
  for (int j = 0; !e && j < nbr; ++j) {
    e = cudaEventRecord(b->joins[1 + j], b->branches[j]);
    if (!e) e = cudaStreamWaitEvent(st, b->joins[1 + j], 0);
  }
  return e;
}

// ---- tuner cache ----
std::mutex g_tune_mu;
std::map<uint64_t, ogs_batch_config> g_tune_cache;

uint64_t fnv(uint64_t h, uint64_t x) {
  for (int j = 0; j < 8; ++j) {
    h ^= (x >> (8 * j)) & 0xFF;
    h *= 1099511628211ull;
  }
  return h;
}

uint64_t tune_key(int type, int sms, int n, const int64_t* records, const int32_t* ks) {
  int kmin = 1 << 30, kmax = 0;
  int64_t hist[40] = {0};
  for (int i = 0; i < n; ++i) {
    kmin = std::min<int>(kmin, ks[i]);
    kmax = std::max<int>(kmax, ks[i]);
    int bin = 0;
    for (int64_t r = records[i]; r > 1; r >>= 1) bin++;
    hist[std::min(bin, 39)]++;
  }
  uint64_t h = 1469598103934665603ull;
  h = fnv(h, static_cast<uint64_t>(type));
  h = fnv(h, static_cast<uint64_t>(sms));
  h = fnv(h, static_cast<uint64_t>(kmin));
  h = fnv(h, static_cast<uint64_t>(kmax));
  for (int64_t c : hist) h = fnv(h, static_cast<uint64_t>(c));
  return h;
}

uint64_t batch_key(const ogs_batch_s* b) {
  std::vector<int64_t> recs;
  std::vector<int32_t> ks;
  for (const ogs_batch_entry& e : b->entries) {
    recs.push_back(e.h->dmaps.nwtiles);
    ks.push_back(e.k);
  }
  return tune_key(b->type, b->cfg.sms, static_cast<int>(recs.size()), recs.data(), ks.data());
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
  for (int i = 0; i < n; ++i) {
    const ogs_batch_entry& e = entries[i];
    const char* bad = nullptr;
    if (!e.h) bad = "handle is NULL";
    else if (e.h->host_only) bad = "handle was set up host-only";
    else if (e.h->gslib) bad = "handle was made by ogs_gslib_setup";
    else if (!e.h->distinct_cols) bad = "a local node appears in two rows of this operator's map";
    else if (e.h->device != dev) bad = "handle lives on another device";
    else if (e.k < 1) bad = "k must be >= 1";
    else if (static_cast<int64_t>(e.h->dmaps.nwtiles) * e.k > INT32_MAX) bad = "more than 2^31 work items";
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
    be.kmagic = batch_kmagic(e.k);
    be.op = e.op;
    fill_pattern(e.h, e.trans, be);
    b->host_entries.push_back(be);
    if (!batch_plain(be)) b->plain = 0;
    b->items.push_back(static_cast<int64_t>(e.h->dmaps.nwtiles) * e.k);
  }
  int sms = 1;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  b->cfg.block = 256;
  b->cfg.occupancy = 2;
  b->cfg.ctas_per_sm = 0;
  b->cfg.solo_items = 0;
  b->cfg.solo_streams = 1;
  b->cfg.sms = sms;
  if ((s = cuda_err(dev_malloc(&b->d_entries, sizeof(BatchEntry) * n), fn, "malloc")) != OGS_OK ||
      (s = cuda_err(dev_malloc(&b->d_starts, sizeof(int64_t) * (n + 1)), fn, "malloc")) != OGS_OK ||
      (s = ensure_branches(b, 1, fn)) != OGS_OK ||
      (s = apply_config(b, b->host_entries.data(), nullptr, fn)) != OGS_OK) {
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
  for (cudaStream_t x : b->branches) cudaStreamDestroy(x);
  for (cudaEvent_t e : b->joins) cudaEventDestroy(e);
  dev_free(b->d_entries);
  dev_free(b->d_starts);
  delete b;
  return OGS_OK;
}

ogs_status ogs_batch_set_fields(ogs_batch b, void* const* d_vs, void* stream) {
  if (!b || !d_vs) return set_error(OGS_EINVAL, "ogs_batch_set_fields: NULL argument");
  for (size_t i = 0; i < b->entries.size(); ++i)
    if (!d_vs[i] && b->entries[i].h->N > 0) return set_error(OGS_EINVAL, "ogs_batch_set_fields: a field is NULL");
  for (size_t i = 0; i < b->entries.size(); ++i) {
    b->entries[i].d_v = d_vs[i];
    b->host_entries[i].v = d_vs[i];
  }
  // the single-mesh and rows-above-degree-8 launches bake fields into the graph
  return apply_config(b, b->host_entries.data(), static_cast<cudaStream_t>(stream), "ogs_batch_set_fields");
}

ogs_status ogs_batch_gather_scatter(ogs_batch b, void* stream) {
  const char* fn = "ogs_batch_gather_scatter";
  TraceRange trace(fn);
  if (!b) return set_error(OGS_EINVAL, "ogs_batch_gather_scatter: batch is NULL");
  int dev = -1;
  ogs_status s;
  if ((s = cuda_err(cudaGetDevice(&dev), fn, "device")) != OGS_OK) return s;
  if (dev != b->device) return set_error(OGS_EINVAL, "ogs_batch_gather_scatter: batch lives on another device");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (!(b->flags & OGS_BATCH_GRAPH)) {
    const int e = launch_all(b, b->host_entries.data(), st);
    return e ? cuda_err(static_cast<cudaError_t>(e), fn, "launch") : OGS_OK;
  }
  if (!b->graph) {
    if (!b->capture && (s = cuda_err(cudaStreamCreateWithFlags(&b->capture, cudaStreamNonBlocking), fn,
                                     "stream")) != OGS_OK)
      return s;
    if ((s = cuda_err(cudaStreamBeginCapture(b->capture, cudaStreamCaptureModeThreadLocal), fn, "capture")) !=
        OGS_OK)
      return s;
    const int e = launch_all(b, b->host_entries.data(), b->capture);
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

ogs_status ogs_batch_get_config(ogs_batch b, ogs_batch_config* cfg) {
  if (!b || !cfg) return set_error(OGS_EINVAL, "ogs_batch_get_config: NULL argument");
  *cfg = b->cfg;
  return OGS_OK;
}

ogs_status ogs_batch_set_config(ogs_batch b, const ogs_batch_config* cfg, void* stream) {
  const char* fn = "ogs_batch_set_config";
  if (!b || !cfg) return set_error(OGS_EINVAL, "ogs_batch_set_config: NULL argument");
  if ((cfg->block != 128 && cfg->block != 256) || cfg->ctas_per_sm < 0 || cfg->solo_items < 0 ||
      cfg->solo_streams < 1 || cfg->solo_streams > kMaxBranches ||
      (cfg->occupancy != 0 && cfg->occupancy != 2 && cfg->occupancy != 3) || cfg->pipeline < 0 ||
      cfg->pipeline > 1 || (cfg->pipeline == 1 && cfg->block != 256))
    return set_error(OGS_EINVAL, "ogs_batch_set_config: block 128 or 256, ctas_per_sm >= 0, solo_items >= 0, "
                                 "1 <= solo_streams <= 8, occupancy 2 or 3, pipeline 0 or 1 (1: block 256)");
  ogs_status s = ensure_branches(b, cfg->solo_streams, fn);
  if (s != OGS_OK) return s;
  const int sms = b->cfg.sms;
  b->cfg = *cfg;
  b->cfg.sms = sms;
  if (b->cfg.occupancy == 0) b->cfg.occupancy = 2;
  return apply_config(b, b->host_entries.data(), static_cast<cudaStream_t>(stream), fn);
}

ogs_status ogs_batch_tune_ex(ogs_batch b, void* stream, unsigned flags, ogs_batch_config* chosen) {
  const char* fn = "ogs_batch_tune";
  TraceRange trace(fn);
  if (!b) return set_error(OGS_EINVAL, "ogs_batch_tune: batch is NULL");
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  const uint64_t key = batch_key(b);
  if (!(flags & OGS_TUNE_NO_CACHE)) {
    ogs_batch_config hit{};
    bool found = false;
    {
      std::lock_guard<std::mutex> g(g_tune_mu);
      auto it = g_tune_cache.find(key);
      if (it != g_tune_cache.end()) {
        hit = it->second;
        found = true;
      }
    }
    if (found) {
      hit.from_cache = 1;
      ogs_status s = ogs_batch_set_config(b, &hit, stream);
      if (s == OGS_OK) {
        b->cfg.from_cache = 1;
        if (chosen) *chosen = b->cfg;
      }
      return s;
    }
  }
  // scratch copies of the fields: every trial starts from the caller's values
  // and the caller's fields are not touched
  const size_t n = b->entries.size();
  const size_t ts = type_size(b->type);
  std::vector<size_t> off(n + 1, 0);
  for (size_t i = 0; i < n; ++i)
    off[i + 1] = off[i] + (static_cast<size_t>(b->entries[i].h->N) * b->entries[i].k * ts + 255) / 256 * 256;
  char* scratch = nullptr;   // working copies
  char* pristine = nullptr;  // the caller's values, copied once
  ogs_status s = cuda_err(dev_malloc(&scratch, std::max<size_t>(off[n], 256)), fn, "scratch");
  if (s == OGS_OK) s = cuda_err(dev_malloc(&pristine, std::max<size_t>(off[n], 256)), fn, "scratch");
  std::vector<BatchEntry> fields = b->host_entries;
  for (size_t i = 0; s == OGS_OK && i < n; ++i) {
    const size_t bytes = static_cast<size_t>(b->entries[i].h->N) * b->entries[i].k * ts;
    if (bytes)
      s = cuda_err(cudaMemcpyAsync(pristine + off[i], b->entries[i].d_v, bytes, cudaMemcpyDeviceToDevice, st), fn,
                   "copy");
    fields[i].v = scratch + off[i];
  }
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (s == OGS_OK) s = cuda_err(cudaEventCreate(&e0), fn, "event");
  if (s == OGS_OK) s = cuda_err(cudaEventCreate(&e1), fn, "event");
  if (s == OGS_OK) s = ensure_branches(b, kMaxBranches, fn);
  const ogs_batch_config saved = b->cfg;
  // time one configuration: 4 calls, each from the caller's values, first one warms up
  auto time_cfg = [&](const ogs_batch_config& c, float* ms) -> ogs_status {
    b->cfg = c;
    b->cfg.sms = saved.sms;
    ogs_status r = apply_config(b, fields.data(), st, fn);
    float tsum = 0.f;
    for (int rep = 0; r == OGS_OK && rep < 4; ++rep) {
      r = cuda_err(cudaMemcpyAsync(scratch, pristine, off[n], cudaMemcpyDeviceToDevice, st), fn, "restore");
      if (r != OGS_OK) break;
      cudaEventRecord(e0, st);
      const int e = launch_all(b, fields.data(), st);
      cudaEventRecord(e1, st);
      if (e) { r = cuda_err(static_cast<cudaError_t>(e), fn, "launch"); break; }
      if ((r = cuda_err(cudaEventSynchronize(e1), fn, "synchronize")) != OGS_OK) break;
      float t = 0.f;
      cudaEventElapsedTime(&t, e0, e1);
      if (rep > 0) tsum += t;
    }
    *ms = tsum / 3.f;
    return r;
  };
  ogs_batch_config best = saved;
  float best_ms = 1e30f;
  auto consider = [&](const ogs_batch_config& c) -> ogs_status {
    float ms = 0.f;
    ogs_status r = time_cfg(c, &ms);
    if (r == OGS_OK && ms < best_ms) {
      best_ms = ms;
      best = c;
    }
    return r;
  };
  // 1) the persistent launch alone: pipeline x block size x register budget x
  // CTAs per SM (the ring pipeline has 256-thread blocks only)
  for (int pipe = 0; s == OGS_OK && pipe <= 1; ++pipe)
    for (int bi = 0; s == OGS_OK && bi < (pipe ? 1 : 2); ++bi)
      for (int occ = 2; s == OGS_OK && occ <= 3; ++occ)
        for (int c = 1; s == OGS_OK && c <= (bi == 0 ? 2 : 4) * occ; ++c) {
          ogs_batch_config cand = saved;
          cand.pipeline = pipe;
          cand.block = bi == 0 ? 256 : 128;
          cand.occupancy = occ;
          cand.ctas_per_sm = c;
          cand.solo_items = 0;
          cand.solo_streams = 1;
          s = consider(cand);
        }
  // 2) entries from a size on run alone on the single-mesh kernel, over 2, 4
  // or 8 branches: thresholds at 1/16, 1/4, 1 and 4 waves of warps of the
  // persistent grid
  const int64_t wave = static_cast<int64_t>(saved.sms) * 24;
  const ogs_batch_config base = best;
  for (int64_t t : {wave / 16, wave / 4, wave, 4 * wave})
    for (int nb : {2, 4, 8}) {
      if (s != OGS_OK) break;
      bool any = false;
      for (int64_t it : b->items) any = any || it >= t;
      if (!any) continue;
      ogs_batch_config cand = base;
      cand.solo_items = t;
      cand.solo_streams = nb;
      s = consider(cand);
    }
  // 3) the persistent launch's CTAs per SM again, beside the chosen solo entries
  if (s == OGS_OK && best.solo_items > 0) {
    const ogs_batch_config base2 = best;
    for (int c = 1; s == OGS_OK && c <= (base2.block == 256 ? 2 : 4) * base2.occupancy; ++c) {
      ogs_batch_config cand = base2;
      cand.ctas_per_sm = c;
      s = consider(cand);
    }
  }
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  dev_free(scratch);
  dev_free(pristine);
  if (s != OGS_OK) {
    b->cfg = saved;
    apply_config(b, b->host_entries.data(), st, fn);
    return s;
  }
  best.ms = best_ms;
  best.from_cache = 0;
  b->cfg = best;
  b->cfg.sms = saved.sms;
  if ((s = apply_config(b, b->host_entries.data(), st, fn)) != OGS_OK) return s;
  {
    std::lock_guard<std::mutex> g(g_tune_mu);
    g_tune_cache[key] = b->cfg;
  }
  if (chosen) *chosen = b->cfg;
  return OGS_OK;
}

ogs_status ogs_batch_tune(ogs_batch b, void* stream, int* chosen_grid) {
  ogs_batch_config c{};
  const ogs_status s = ogs_batch_tune_ex(b, stream, 0, &c);
  if (s == OGS_OK && chosen_grid) *chosen_grid = c.ctas_per_sm * c.sms;
  return s;
}

ogs_status ogs_batch_tune_key(int type, int sms, int n, const int64_t* records, const int32_t* ks, uint64_t* key) {
  if (!key || n < 0 || (n > 0 && (!records || !ks)))
    return set_error(OGS_EINVAL, "ogs_batch_tune_key: bad arguments");
  *key = tune_key(type, sms, n, records, ks);
  return OGS_OK;
}

ogs_status ogs_batch_tune_cache_clear(void) {
  std::lock_guard<std::mutex> g(g_tune_mu);
  g_tune_cache.clear();
  return OGS_OK;
}

ogs_status ogs_batch_items(ogs_batch b, int64_t* items) {
  if (!b || !items) return set_error(OGS_EINVAL, "ogs_batch_items: NULL argument");
  int64_t t = 0;
  for (int64_t x : b->items) t += x;
  *items = t;
  return OGS_OK;
}

}  // extern "C"
