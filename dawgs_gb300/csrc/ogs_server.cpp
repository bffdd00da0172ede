// ogs_server.cpp -- served gather-scatter: resident meshes, requests admitted
// against an HBM budget, continuous batching (C ABI part of ogs_c.h).
//
// A request names a resident mesh and carries a host field (k interleaved
// components per node) that is gather-scattered in place.  One worker thread
// runs the service loop:
//   admit   -- FIFO: a pending request is admitted when a field buffer of its
//              size fits in the budget pool and an in-flight slot is free;
//   launch  -- everything admitted since the last turn is copied in on the
//              copy-in stream and run as one batched launch per value type
//              (ogs_batch.cuh) on the next of two compute streams, so a batch
//              that arrives while another runs overlaps with it on the GPU;
//   retire  -- each request's copy-out records an event; the worker polls the
//              oldest outstanding events, stamps completions and returns the
//              buffers to the pool.
// Latency is completion minus arrival (the submit time, or the arrival time the
// caller passes).  Every result equals the request's ogs_gather_scatter_host
// alone, bit for bit: batching changes where the rows run, not their fold.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "ogs_internal.hpp"

namespace ogsgb {
namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

size_t tsize(int type) { return (type == OGS_DOUBLE || type == OGS_INT64) ? 8 : 4; }

// First-fit allocator over one device arena, 256-byte granules.
class Pool {
 public:
  void reset(size_t bytes) {
    free_.clear();
    if (bytes) free_[0] = bytes;
  }
  bool alloc(size_t bytes, size_t* off) {
    bytes = (bytes + 255) / 256 * 256;
    for (auto it = free_.begin(); it != free_.end(); ++it) {
      if (it->second >= bytes) {
        *off = it->first;
        const size_t rest = it->second - bytes, at = it->first + bytes;
        free_.erase(it);
        if (rest) free_[at] = rest;
        return true;
      }
    }
    return false;
  }
  void release(size_t off, size_t bytes) {
    bytes = (bytes + 255) / 256 * 256;
    auto it = free_.emplace(off, bytes).first;
    auto nx = std::next(it);
    if (nx != free_.end() && it->first + it->second == nx->first) {
      it->second += nx->second;
      free_.erase(nx);
    }
    if (it != free_.begin()) {
      auto pv = std::prev(it);
      if (pv->first + pv->second == it->first) {
        pv->second += it->second;
        free_.erase(it);
      }
    }
  }

 private:
  std::map<size_t, size_t> free_;
};

struct Req {
  int64_t id;
  ogs_server_request r;
  size_t bytes = 0;
  size_t off = 0;
  double t_arrival = 0, t_done = 0;
  std::atomic<int> state{0};  // 0 pending, 1 in flight, 2 done
  cudaEvent_t copied_out = nullptr;
};

// Device tables of one batched launch, reused once its launch has finished.
struct TableSlot {
  BatchEntry* d_entries = nullptr;
  int64_t* d_starts = nullptr;
  BatchEntry* h_entries = nullptr;  // pinned staging
  int64_t* h_starts = nullptr;
  cudaEvent_t done = nullptr;
  bool used = false;
};

}  // namespace
}  // namespace ogsgb

using namespace ogsgb;

struct ogs_server_s {
  ogs_server_config cfg{};
  int device = 0;
  std::vector<ogs_handle> meshes;
  char* pool_base = nullptr;
  Pool pool;
  cudaStream_t copy_in = nullptr, copy_out = nullptr, compute[2] = {nullptr, nullptr};
  int next_compute = 0;
  std::vector<TableSlot> slots;
  size_t next_slot = 0;

  std::mutex mu;
  std::condition_variable cv;
  std::deque<Req*> pending;
  std::vector<std::unique_ptr<Req>> all;  // by id
  std::deque<Req*> outstanding;          // launched, in copy-out order (worker only)
  std::vector<cudaEvent_t> spare_events; // recycled completion events (worker only)
  std::atomic<int64_t> inflight{0}, completed{0}, submitted{0};
  std::atomic<int64_t> launches{0}, batched_requests{0};
  std::thread worker;
  std::atomic<bool> stop{false};
  std::string error;
};

namespace ogsgb {
namespace {

int batch_launch(int type, const BatchEntry* E, const int64_t* starts, int n, int64_t nitems, cudaStream_t st) {
  switch (type) {
    case OGS_FLOAT: return launch_batch_f32(E, starts, n, nitems, 0, st);
    case OGS_DOUBLE: return launch_batch_f64(E, starts, n, nitems, 0, st);
    case OGS_INT32: return launch_batch_i32(E, starts, n, nitems, 0, st);
    default: return launch_batch_i64(E, starts, n, nitems, 0, st);
  }
}

int general_launch(int type, const ogs_handle_s* h, void* v, int k, int op, const Pattern& pat, cudaStream_t st) {
  DevMaps g = h->dmaps;
  g.nwtiles = 0;
  g.ntiles = g.ngtiles;
  FieldArgs f{};
  f.v = v;
  f.K = k;
  switch (type) {
    case OGS_FLOAT: return launch_f32(g, f, kModeGS, op, pat, st);
    case OGS_DOUBLE: return launch_f64(g, f, kModeGS, op, pat, st);
    case OGS_INT32: return launch_i32(g, f, kModeGS, op, pat, st);
    default: return launch_i64(g, f, kModeGS, op, pat, st);
  }
}

// Launch one group of admitted requests of one value type; returns a CUDA error.
int launch_group(ogs_server_s* s, const std::vector<Req*>& grp, int type, cudaEvent_t copied) {
  TableSlot& slot = s->slots[s->next_slot];
  s->next_slot = (s->next_slot + 1) % s->slots.size();
  if (slot.used) cudaEventSynchronize(slot.done);  // its previous launch must be over
  const int n = static_cast<int>(grp.size());
  slot.h_starts[0] = 0;
  for (int i = 0; i < n; ++i) {
    const Req* q = grp[i];
    const ogs_handle_s* h = s->meshes[q->r.mesh];
    BatchEntry& e = slot.h_entries[i];
    e = BatchEntry{};
    e.recs = h->dmaps.wrecs;
    e.wemask = h->dmaps.wemask;
    e.v = s->pool_base + q->off;
    e.K = q->r.k;
    e.op = q->r.op;
    if (h->kind == OGS_SIGNED) {
      if (q->r.trans == OGS_TRANS) e.scatter_n = e.limit_n = 1;
      else if (q->r.trans == OGS_NOTRANS) e.gather_n = 1;
    }
    e.use_mask = (e.gather_n || e.scatter_n) && h->kind == OGS_SIGNED;
    slot.h_starts[i + 1] = slot.h_starts[i] + static_cast<int64_t>(h->dmaps.nwtiles) * q->r.k;
  }
  cudaStream_t st = s->compute[s->next_compute];
  s->next_compute ^= 1;
  int e = cudaMemcpyAsync(slot.d_entries, slot.h_entries, sizeof(BatchEntry) * n, cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(slot.d_starts, slot.h_starts, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, st);
  if (!e) e = cudaStreamWaitEvent(st, copied, 0);
  if (!e) e = batch_launch(type, slot.d_entries, slot.d_starts, n, slot.h_starts[n], st);
  for (int i = 0; !e && i < n; ++i) {
    const Req* q = grp[i];
    const ogs_handle_s* h = s->meshes[q->r.mesh];
    if (h->dmaps.ngtiles > 0) {
      const BatchEntry& be = slot.h_entries[i];
      e = general_launch(type, h, be.v, be.K, be.op, Pattern{be.gather_n, be.scatter_n, be.limit_n}, st);
    }
  }
  if (!e) e = cudaEventRecord(slot.done, st);
  slot.used = true;
  if (!e) e = cudaStreamWaitEvent(s->copy_out, slot.done, 0);
  for (int i = 0; !e && i < n; ++i) {
    Req* q = grp[i];
    e = cudaMemcpyAsync(q->r.host, s->pool_base + q->off, q->bytes, cudaMemcpyDeviceToHost, s->copy_out);
    if (!e) {
      if (s->spare_events.empty()) {
        cudaEvent_t ev = nullptr;
        e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
        if (!e) s->spare_events.push_back(ev);
      }
    }
    if (!e) {
      q->copied_out = s->spare_events.back();
      s->spare_events.pop_back();
      e = cudaEventRecord(q->copied_out, s->copy_out);
      s->outstanding.push_back(q);
    }
  }
  s->launches.fetch_add(1);
  s->batched_requests.fetch_add(n);
  return e;
}

// Completions arrive in copy-out order: poll from the oldest.
void retire(ogs_server_s* s) {
  int n = 0;
  while (!s->outstanding.empty()) {
    Req* q = s->outstanding.front();
    const cudaError_t e = cudaEventQuery(q->copied_out);
    if (e == cudaErrorNotReady) break;
    const double t = now_s();
    s->outstanding.pop_front();
    s->spare_events.push_back(q->copied_out);
    q->copied_out = nullptr;
    {
      std::lock_guard<std::mutex> g(s->mu);
      if (e != cudaSuccess && s->error.empty()) s->error = cudaGetErrorString(e);
      s->pool.release(q->off, q->bytes);
      q->t_done = t;
      q->state.store(2);
      s->inflight.fetch_sub(1);
    }
    s->completed.fetch_add(1);
    n++;
  }
  if (n) s->cv.notify_all();
}

void worker_loop(ogs_server_s* s) {
  cudaSetDevice(s->device);
  cudaEvent_t copied = nullptr;
  cudaEventCreateWithFlags(&copied, cudaEventDisableTiming);
  std::vector<Req*> admitted;
  while (true) {
    retire(s);
    {
      std::unique_lock<std::mutex> lk(s->mu);
      if (s->pending.empty() && s->stop.load() && s->inflight.load() == 0) break;
      // admission: FIFO against the budget and the in-flight slots
      while (!s->pending.empty() && s->inflight.load() < s->cfg.max_inflight &&
             static_cast<int>(admitted.size()) < s->cfg.max_batch) {
        Req* q = s->pending.front();
        if (!s->pool.alloc(q->bytes, &q->off)) break;
        s->pending.pop_front();
        q->state.store(1);
        s->inflight.fetch_add(1);
        admitted.push_back(q);
      }
      if (admitted.empty()) {
        // nothing to launch: wait for a submission, or come back soon to
        // retire what is in flight (which may free budget for the pending)
        s->cv.wait_for(lk, std::chrono::microseconds(s->outstanding.empty() ? 500 : 20));
        continue;
      }
    }
    int e = 0;
    for (Req* q : admitted)
      if (!e) e = cudaMemcpyAsync(s->pool_base + q->off, q->r.host, q->bytes, cudaMemcpyHostToDevice, s->copy_in);
    if (!e) e = cudaEventRecord(copied, s->copy_in);
    for (int type = OGS_FLOAT; !e && type <= OGS_INT64; ++type) {
      std::vector<Req*> grp;
      for (Req* q : admitted)
        if (q->r.type == type) grp.push_back(q);
      if (!grp.empty()) e = launch_group(s, grp, type, copied);
    }
    if (e) {
      std::lock_guard<std::mutex> g(s->mu);
      s->error = cudaGetErrorString(static_cast<cudaError_t>(e));
    }
    admitted.clear();
  }
  cudaEventDestroy(copied);
}

void destroy(ogs_server_s* s) {
  for (cudaEvent_t ev : s->spare_events) cudaEventDestroy(ev);
  for (TableSlot& t : s->slots) {
    if (t.d_entries) cudaFree(t.d_entries);
    if (t.d_starts) cudaFree(t.d_starts);
    if (t.h_entries) cudaFreeHost(t.h_entries);
    if (t.h_starts) cudaFreeHost(t.h_starts);
    if (t.done) cudaEventDestroy(t.done);
  }
  for (cudaStream_t st : {s->copy_in, s->copy_out, s->compute[0], s->compute[1]})
    if (st) cudaStreamDestroy(st);
  if (s->pool_base) cudaFree(s->pool_base);
  delete s;
}

}  // namespace
}  // namespace ogsgb

extern "C" {

ogs_status ogs_server_create(ogs_server* out, const ogs_server_config* cfg) {
  if (!out || !cfg) return set_error(OGS_EINVAL, "ogs_server_create: NULL argument");
  *out = nullptr;
  if (cfg->field_budget_bytes <= 0 || cfg->max_inflight < 1 || cfg->max_batch < 1)
    return set_error(OGS_EINVAL, "ogs_server_create: budget, max_inflight and max_batch must be positive");
  ogs_server_s* s = new (std::nothrow) ogs_server_s();
  if (!s) return set_error(OGS_ENOMEM, "ogs_server_create: out of host memory");
  s->cfg = *cfg;
  cudaGetDevice(&s->device);
  cudaError_t e = cudaMalloc(&s->pool_base, static_cast<size_t>(cfg->field_budget_bytes));
  if (e == cudaSuccess) {
    s->pool.reset(static_cast<size_t>(cfg->field_budget_bytes));
    for (cudaStream_t* st : {&s->copy_in, &s->copy_out, &s->compute[0], &s->compute[1]})
      if (e == cudaSuccess) e = cudaStreamCreateWithFlags(st, cudaStreamNonBlocking);
  }
  s->slots.resize(16);
  for (TableSlot& t : s->slots) {
    if (e == cudaSuccess) e = cudaMalloc(&t.d_entries, sizeof(BatchEntry) * cfg->max_batch);
    if (e == cudaSuccess) e = cudaMalloc(&t.d_starts, sizeof(int64_t) * (cfg->max_batch + 1));
    if (e == cudaSuccess) e = cudaMallocHost(&t.h_entries, sizeof(BatchEntry) * cfg->max_batch);
    if (e == cudaSuccess) e = cudaMallocHost(&t.h_starts, sizeof(int64_t) * (cfg->max_batch + 1));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&t.done, cudaEventDisableTiming);
  }
  if (e != cudaSuccess) {
    cudaGetLastError();
    destroy(s);
    return set_error(e == cudaErrorMemoryAllocation ? OGS_ENOMEM : OGS_EDEVICE,
                     std::string("ogs_server_create: ") + cudaGetErrorString(e));
  }
  s->worker = std::thread(worker_loop, s);
  *out = s;
  return OGS_OK;
}

ogs_status ogs_server_add_mesh(ogs_server s, ogs_handle h, int* mesh_id) {
  if (!s || !h || !mesh_id) return set_error(OGS_EINVAL, "ogs_server_add_mesh: NULL argument");
  if (h->host_only || h->device != s->device)
    return set_error(OGS_EINVAL, "ogs_server_add_mesh: the handle must live on the server's device");
  if (!h->distinct_cols)
    return set_error(OGS_EINVAL, "ogs_server_add_mesh: a local node appears in two rows of this operator's map");
  std::lock_guard<std::mutex> g(s->mu);
  s->meshes.push_back(h);
  *mesh_id = static_cast<int>(s->meshes.size()) - 1;
  return OGS_OK;
}

ogs_status ogs_server_submit(ogs_server s, const ogs_server_request* r, double arrival, int64_t* id) {
  if (!s || !r) return set_error(OGS_EINVAL, "ogs_server_submit: NULL argument");
  std::unique_ptr<Req> q(new (std::nothrow) Req());
  if (!q) return set_error(OGS_ENOMEM, "ogs_server_submit: out of host memory");
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (r->mesh < 0 || r->mesh >= static_cast<int>(s->meshes.size()))
      return set_error(OGS_EINVAL, "ogs_server_submit: unknown mesh");
    if (r->type < OGS_FLOAT || r->type > OGS_INT64 || r->op < OGS_ADD || r->op > OGS_MIN || r->k < 1 ||
        r->trans < OGS_SYM || r->trans > OGS_TRANS || !r->host)
      return set_error(OGS_EINVAL, "ogs_server_submit: bad request");
    q->r = *r;
    q->bytes = static_cast<size_t>(s->meshes[r->mesh]->N) * r->k * tsize(r->type);
    if (q->bytes > static_cast<size_t>(s->cfg.field_budget_bytes))
      return set_error(OGS_ERANGE, "ogs_server_submit: the field is larger than the whole budget");
    q->t_arrival = arrival > 0 ? arrival : now_s();
    q->id = static_cast<int64_t>(s->all.size());
    if (id) *id = q->id;
    s->pending.push_back(q.get());
    s->all.push_back(std::move(q));
  }
  s->submitted.fetch_add(1);
  s->cv.notify_all();
  return OGS_OK;
}

double ogs_server_clock(void) { return now_s(); }

ogs_status ogs_server_wait(ogs_server s, int64_t id) {
  if (!s) return set_error(OGS_EINVAL, "ogs_server_wait: NULL server");
  Req* q;
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (id < 0 || id >= static_cast<int64_t>(s->all.size())) return set_error(OGS_EINVAL, "ogs_server_wait: unknown id");
    q = s->all[id].get();
  }
  std::unique_lock<std::mutex> lk(s->mu);
  while (q->state.load() != 2) {
    if (!s->error.empty()) return set_error(OGS_EDEVICE, "ogs_server: " + s->error);
    s->cv.wait_for(lk, std::chrono::milliseconds(1));
  }
  return OGS_OK;
}

ogs_status ogs_server_drain(ogs_server s) {
  if (!s) return set_error(OGS_EINVAL, "ogs_server_drain: NULL server");
  std::unique_lock<std::mutex> lk(s->mu);
  while (s->completed.load() < s->submitted.load()) {
    if (!s->error.empty()) return set_error(OGS_EDEVICE, "ogs_server: " + s->error);
    s->cv.wait_for(lk, std::chrono::milliseconds(1));
  }
  return OGS_OK;
}

ogs_status ogs_server_latencies(ogs_server s, int64_t first, int64_t n, double* arrival, double* done) {
  if (!s) return set_error(OGS_EINVAL, "ogs_server_latencies: NULL server");
  std::lock_guard<std::mutex> g(s->mu);
  if (first < 0 || n < 0 || first + n > static_cast<int64_t>(s->all.size()))
    return set_error(OGS_EINVAL, "ogs_server_latencies: range out of bounds");
  for (int64_t i = 0; i < n; ++i) {
    const Req* q = s->all[first + i].get();
    if (arrival) arrival[i] = q->t_arrival;
    if (done) done[i] = q->state.load() == 2 ? q->t_done : -1.0;
  }
  return OGS_OK;
}

ogs_status ogs_server_counters(ogs_server s, int64_t* launches, int64_t* batched_requests) {
  if (!s) return set_error(OGS_EINVAL, "ogs_server_counters: NULL server");
  if (launches) *launches = s->launches.load();
  if (batched_requests) *batched_requests = s->batched_requests.load();
  return OGS_OK;
}

ogs_status ogs_server_free(ogs_server s) {
  if (!s) return OGS_OK;
  {
    std::lock_guard<std::mutex> g(s->mu);
    s->stop.store(true);
  }
  s->cv.notify_all();
  if (s->worker.joinable()) s->worker.join();
  destroy(s);
  return OGS_OK;
}

}  // extern "C"
