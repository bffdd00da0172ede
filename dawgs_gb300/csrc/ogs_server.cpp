// ogs_server.cpp -- served gather-scatter: resident meshes, requests admitted
// against an HBM budget, continuous batching (C ABI part of ogs_c.h).
//
// A request names a resident mesh and carries a host field (k interleaved
// components per node) that is gather-scattered in place.  One worker thread
// runs the service loop and never blocks on the GPU:
//   retire  -- each request's copy-out records an event; the worker polls the
//              oldest outstanding events of each lane, stamps completions and
//              returns the buffers to the pool;
//   admit   -- pending requests are scanned in arrival order, up to
//              kAdmitWindow of them: each one whose field buffer fits in the
//              budget pool (and while in-flight slots remain) is admitted, so
//              one large request cannot hold back the small ones behind it.
//              A request passed over kMaxPassOvers times stops the scan at
//              itself until it fits (no starvation);
//   launch  -- admitted requests go to one of two lanes by size (small fields
//              and large fields), each with its own copy-in, compute and
//              copy-out streams.  A lane's turn copies in its oldest ready
//              requests up to the lane's byte budget and runs them as one
//              batched launch per value type (ogs_batch.cuh); the lanes share
//              the copy engines, so the budgets keep a large-lane turn from
//              holding a small request's copies back.  A launch needs a table
//              slot whose previous launch is over; when none is free the lane
//              waits for the next turn instead of blocking the worker.
// Requests arriving while others are on the GPU are admitted and launched on
// the next turn, so their copies and kernels overlap the earlier ones'.
// Latency is completion minus arrival: the submit time, or the arrival time
// the caller passes.  A request whose arrival lies in the future is not
// admitted before that time, so a caller (a load generator) can hand over a
// whole schedule of arrivals at once and the server sees each request when it
// arrives.  Every result equals the request's ogs_gather_scatter_host
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
#include "ogs_trace.hpp"

namespace ogsgb {
namespace {

double now_s() {
  using namespace std::chrono;
  return duration<double>(steady_clock::now().time_since_epoch()).count();
}

// Pending requests looked at per admission pass, and how often one may be
// passed over by later requests before the scan stops at it.
constexpr int kAdmitWindow = 64;
constexpr int kMaxPassOvers = 16;
// Fields up to this size go to the small lane.
constexpr size_t kSmallBytes = size_t(4) << 20;
// Turns (batched launches with their copies) a lane keeps on the GPU at once.
// While they run, newly admitted requests wait in the lane and go together in
// its next turn: under load the batches grow and the per-launch costs are
// shared; with nothing running a request is launched at once.
#ifndef OGS_SERVER_SMALL_TURNS
#define OGS_SERVER_SMALL_TURNS 2
#endif
#ifndef OGS_SERVER_LARGE_TURNS
#define OGS_SERVER_LARGE_TURNS 4
#endif
static_assert(OGS_SERVER_SMALL_TURNS >= 1 && OGS_SERVER_SMALL_TURNS < 8, "a lane rotates 8 turn events");
static_assert(OGS_SERVER_LARGE_TURNS >= 1 && OGS_SERVER_LARGE_TURNS < 8, "a lane rotates 8 turn events");
// Field bytes one turn copies in (at least one request).  Both lanes share
// the copy engines: a large-lane turn of many fields would hold a small
// request's copies back for milliseconds, so large-lane turns are short and
// more of them are kept in flight to keep the copies streaming.
#ifndef OGS_SERVER_SMALL_TURN_BYTES
#define OGS_SERVER_SMALL_TURN_BYTES (size_t(64) << 20)
#endif
#ifndef OGS_SERVER_LARGE_TURN_BYTES
#define OGS_SERVER_LARGE_TURN_BYTES (size_t(16) << 20)
#endif
// Copies longer than this are issued in pieces of this size (0: whole), so
// the other lane's copies can go between them.
#ifndef OGS_SERVER_COPY_CHUNK
#define OGS_SERVER_COPY_CHUNK 0
#endif
// Launch tables per server (shared by both lanes), and completion events made
// at creation (more are made when requests in flight need them).
constexpr int kTableSlots = 64;
constexpr int kSpareEvents = 512;

enum ReqState : int { kPending = 0, kInFlight = 1, kDone = 2, kCancelled = 3 };

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
  double t_arrival = 0, t_launch = -1, t_done = -1;
  int passed_over = 0;
  std::atomic<int> state{kPending};
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

// Streams and queues of one size class.
struct Lane {
  cudaStream_t in = nullptr, compute = nullptr, out = nullptr;
  cudaEvent_t copied = nullptr;  // all of a turn's copies in are done
  std::vector<Req*> ready;       // admitted, not yet launched (worker only)
  std::deque<Req*> outstanding;  // launched, in copy-out order (worker only)
  std::deque<cudaEvent_t> running;  // its turns' launches not yet finished, in order (worker only)
  cudaEvent_t turn_done[8] = {};     // recorded after each turn's launches, used in rotation
  int next_turn_event = 0;
  int max_turns = 1;       // turns kept in flight
  size_t turn_bytes = 0;   // field bytes one turn copies in (at least one request)
};

// One copy, in pieces of OGS_SERVER_COPY_CHUNK bytes when that is set.
int copy_async(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind, cudaStream_t st) {
  const size_t piece = OGS_SERVER_COPY_CHUNK ? size_t(OGS_SERVER_COPY_CHUNK) : bytes;
  for (size_t at = 0; at < bytes; at += piece) {
    const size_t len = std::min(piece, bytes - at);
    const int e = cudaMemcpyAsync(static_cast<char*>(dst) + at, static_cast<const char*>(src) + at, len, kind, st);
    if (e) return e;
  }
  return 0;
}

}  // namespace
}  // namespace ogsgb

using namespace ogsgb;

struct ogs_server_s {
  ogs_server_config cfg{};
  int device = 0;
  std::vector<ogs_handle> meshes;
  char* pool_base = nullptr;
  char* d_tables = nullptr;  // every slot's device tables, one allocation
  char* h_tables = nullptr;  // and their pinned staging
  Pool pool;
  Lane lanes[2];  // [0] small fields, [1] large fields
  std::vector<TableSlot> slots;
  size_t next_slot = 0;

  std::mutex mu;
  std::condition_variable cv;
  std::deque<Req*> pending;
  std::vector<std::unique_ptr<Req>> all;  // by id
  std::vector<cudaEvent_t> spare_events;  // recycled completion events (worker only)
  std::atomic<int64_t> inflight{0}, completed{0}, submitted{0};
  std::atomic<int64_t> launches{0}, batched_requests{0};
  std::thread worker;
  std::atomic<bool> stop{false};
  std::string error;
  ogs_server_stats stats{};  // the worker's own timing (s->mu held to read or write)
};

namespace ogsgb {
namespace {

int batch_launch(int type, const BatchEntry* E, const int64_t* starts, int n, int64_t nitems, int plain,
                 cudaStream_t st) {
  switch (type) {
    case OGS_FLOAT: return launch_batch_f32(E, starts, n, nitems, 0, 256, 2, 0, plain, st);
    case OGS_DOUBLE: return launch_batch_f64(E, starts, n, nitems, 0, 256, 2, 0, plain, st);
    case OGS_INT32: return launch_batch_i32(E, starts, n, nitems, 0, 256, 2, 0, plain, st);
    default: return launch_batch_i64(E, starts, n, nitems, 0, 256, 2, 0, plain, st);
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

// Free table slots (their previous launch is over), without waiting; at most
// `want` of them.  A failed query is recorded as the server's error.
std::vector<TableSlot*> free_slots(ogs_server_s* s, int want) {
  std::vector<TableSlot*> got;
  const size_t n = s->slots.size();
  for (size_t j = 0; j < n && static_cast<int>(got.size()) < want; ++j) {
    TableSlot& t = s->slots[(s->next_slot + j) % n];
    if (t.used) {
      const cudaError_t e = cudaEventQuery(t.done);
      if (e == cudaErrorNotReady) continue;
      if (e != cudaSuccess) {
        std::lock_guard<std::mutex> g(s->mu);
        if (s->error.empty()) s->error = cudaGetErrorString(e);
        continue;
      }
      t.used = false;
    }
    got.push_back(&t);
  }
  if (!got.empty()) s->next_slot = (static_cast<size_t>(got.back() - s->slots.data()) + 1) % n;
  return got;
}

// Launch one group of a lane's requests of one value type on the lane's
// compute stream, after the lane's copies in; queue their copies out.
int launch_group(ogs_server_s* s, Lane& lane, TableSlot& slot, const std::vector<Req*>& grp, int type) {
  TraceRange trace(&lane == &s->lanes[0] ? "ogs_server: small-field batch" : "ogs_server: large-field batch");
  const int n = static_cast<int>(grp.size());
  slot.h_starts[0] = 0;
  int plain = 1;
  for (int i = 0; i < n; ++i) {
    const Req* q = grp[i];
    const ogs_handle_s* h = s->meshes[q->r.mesh];
    BatchEntry& e = slot.h_entries[i];
    e = BatchEntry{};
    e.recs = h->dmaps.wrecs;
    e.wemask = h->dmaps.wemask;
    e.v = s->pool_base + q->off;
    e.K = q->r.k;
    e.kmagic = batch_kmagic(q->r.k);
    e.op = q->r.op;
    const Pattern p = pattern_for(h, kModeGS, q->r.trans);
    e.gather_n = p.gather_n;
    e.scatter_n = p.scatter_n;
    e.limit_n = p.limit_n;
    e.use_mask = (e.gather_n || e.scatter_n) && h->kind == OGS_SIGNED;
    if (!batch_plain(e)) plain = 0;
    slot.h_starts[i + 1] = slot.h_starts[i] + static_cast<int64_t>(h->dmaps.nwtiles) * q->r.k;
  }
  cudaStream_t st = lane.compute;
  int e = cudaMemcpyAsync(slot.d_entries, slot.h_entries, sizeof(BatchEntry) * n, cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(slot.d_starts, slot.h_starts, sizeof(int64_t) * (n + 1), cudaMemcpyHostToDevice, st);
  if (!e) e = cudaStreamWaitEvent(st, lane.copied, 0);
  if (!e) e = batch_launch(type, slot.d_entries, slot.d_starts, n, slot.h_starts[n], plain, st);
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
  const double t = now_s();
  if (!e) e = cudaStreamWaitEvent(lane.out, slot.done, 0);
  for (int i = 0; !e && i < n; ++i) {
    Req* q = grp[i];
    q->t_launch = t;
    e = copy_async(q->r.host, s->pool_base + q->off, q->bytes, cudaMemcpyDeviceToHost, lane.out);
    if (!e && s->spare_events.empty()) {
      cudaEvent_t ev = nullptr;
      e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
      if (!e) s->spare_events.push_back(ev);
    }
    if (!e) {
      q->copied_out = s->spare_events.back();
      s->spare_events.pop_back();
      e = cudaEventRecord(q->copied_out, lane.out);
      lane.outstanding.push_back(q);
    }
  }
  s->launches.fetch_add(1);
  s->batched_requests.fetch_add(n);
  return e;
}

// Launch what a lane has ready, when enough table slots are free.
int launch_lane(ogs_server_s* s, Lane& lane) {
  if (lane.ready.empty()) return 0;
  while (!lane.running.empty()) {
    const cudaError_t q = cudaEventQuery(lane.running.front());
    if (q == cudaErrorNotReady) break;
    lane.running.pop_front();
  }
  if (static_cast<int>(lane.running.size()) >= lane.max_turns) return 0;  // next turn, a larger batch
  // this turn: the oldest ready requests up to the turn's byte budget
  size_t take = 0, bytes = 0;
  while (take < lane.ready.size() && (take == 0 || bytes + lane.ready[take]->bytes <= lane.turn_bytes))
    bytes += lane.ready[take++]->bytes;
  std::vector<Req*> grp[4];
  int groups = 0;
  for (size_t j = 0; j < take; ++j) {
    Req* q = lane.ready[j];
    if (grp[q->r.type].empty()) groups++;
    grp[q->r.type].push_back(q);
  }
  std::vector<TableSlot*> slots = free_slots(s, groups);
  if (static_cast<int>(slots.size()) < groups) return 0;  // next turn
  int e = 0;
  for (size_t j = 0; j < take; ++j) {
    Req* q = lane.ready[j];
    if (!e) e = copy_async(s->pool_base + q->off, q->r.host, q->bytes, cudaMemcpyHostToDevice, lane.in);
  }
  if (!e) e = cudaEventRecord(lane.copied, lane.in);
  int j = 0;
  for (int type = OGS_FLOAT; !e && type <= OGS_INT64; ++type)
    if (!grp[type].empty()) e = launch_group(s, lane, *slots[j++], grp[type], type);
  if (!e) {
    cudaEvent_t ev = lane.turn_done[lane.next_turn_event];
    lane.next_turn_event = (lane.next_turn_event + 1) % 8;
    e = cudaEventRecord(ev, lane.compute);
    if (!e) lane.running.push_back(ev);
  }
  lane.ready.erase(lane.ready.begin(), lane.ready.begin() + static_cast<std::ptrdiff_t>(take));
  return e;
}

// Completions arrive in copy-out order within a lane: poll from the oldest.
void retire(ogs_server_s* s, Lane& lane) {
  int n = 0;
  while (!lane.outstanding.empty()) {
    Req* q = lane.outstanding.front();
    const cudaError_t e = cudaEventQuery(q->copied_out);
    if (e == cudaErrorNotReady) break;
    const double t = now_s();
    lane.outstanding.pop_front();
    s->spare_events.push_back(q->copied_out);
    q->copied_out = nullptr;
    {
      std::lock_guard<std::mutex> g(s->mu);
      if (e != cudaSuccess && s->error.empty()) s->error = cudaGetErrorString(e);
      s->pool.release(q->off, q->bytes);
      q->t_done = t;
      q->state.store(kDone);
      s->inflight.fetch_sub(1);
    }
    s->completed.fetch_add(1);
    n++;
  }
  if (n) s->cv.notify_all();
}

// Admission pass (s->mu held): requests that have arrived and fit, in
// submission order, within the window.  Every admission counts as a
// pass-over for each earlier request of the pass that did not fit; one passed
// over kMaxPassOvers times stops the scan at itself, so it is the next to be
// admitted once memory frees up.  Returns the earliest arrival still in the
// future (0 if none was seen).
double admit(ogs_server_s* s, double now) {
  int looked = 0;
  double next = 0;
  std::vector<Req*> blocked;
  for (auto it = s->pending.begin(); it != s->pending.end() && looked < kAdmitWindow;) {
    if (s->inflight.load() >= s->cfg.max_inflight) break;
    Req* q = *it;
    looked++;
    if (q->t_arrival > now) {  // scheduled, not arrived yet
      if (next == 0 || q->t_arrival < next) next = q->t_arrival;
      ++it;
      continue;
    }
    Lane& lane = s->lanes[q->bytes <= kSmallBytes ? 0 : 1];
    if (static_cast<int>(lane.ready.size()) < s->cfg.max_batch && s->pool.alloc(q->bytes, &q->off)) {
      it = s->pending.erase(it);
      q->state.store(kInFlight);
      s->inflight.fetch_add(1);
      lane.ready.push_back(q);
      for (Req* b : blocked) b->passed_over++;
      continue;
    }
    if (q->passed_over >= kMaxPassOvers) break;  // nothing later may pass it any more
    blocked.push_back(q);
    ++it;
  }
  return next;
}

void worker_loop(ogs_server_s* s) {
  cudaSetDevice(s->device);
  double t_prev = now_s();
  while (true) {
    // the worker's timing: gaps between passes (sleeping or descheduled) and
    // the time spent in CUDA calls
    const double t_pass = now_s();
    for (Lane& l : s->lanes) retire(s, l);
    const double t_retired = now_s();
    {
      std::lock_guard<std::mutex> g(s->mu);
      ogs_server_stats& w = s->stats;
      w.passes++;
      w.max_gap_ms = std::max(w.max_gap_ms, (t_pass - t_prev) * 1e3);
      w.max_retire_ms = std::max(w.max_retire_ms, (t_retired - t_pass) * 1e3);
      if (t_pass - t_prev > 1e-3) w.gaps_over_1ms++;
    }
    t_prev = t_pass;
    bool idle;
    {
      std::unique_lock<std::mutex> lk(s->mu);
      const bool nothing_out = s->lanes[0].outstanding.empty() && s->lanes[1].outstanding.empty();
      const bool nothing_ready = s->lanes[0].ready.empty() && s->lanes[1].ready.empty();
      if (s->pending.empty() && nothing_ready && s->stop.load() && s->inflight.load() == 0) break;
      const double now = now_s();
      const double next = admit(s, now);
      idle = s->lanes[0].ready.empty() && s->lanes[1].ready.empty();
      if (idle) {
        // nothing to launch: wait for a submission or the next scheduled
        // arrival, or come back soon to retire what is in flight (which may
        // free budget for the pending); an arrival due within 100 us is
        // waited for by polling, for its admission time
        double wait_us = nothing_out ? 500 : 20;
        if (next > 0) wait_us = std::min(wait_us, (next - now) * 1e6);
        if (wait_us > 100) {
          s->cv.wait_for(lk, std::chrono::microseconds(static_cast<int64_t>(wait_us)));
        } else if (next > 0 && wait_us > 0) {
          lk.unlock();
          std::this_thread::yield();
        }
        continue;
      }
    }
    for (Lane& l : s->lanes) {
      const double t0 = now_s();
      const int e = launch_lane(s, l);
      const double dt = now_s() - t0;
      std::lock_guard<std::mutex> g(s->mu);
      s->stats.max_launch_ms = std::max(s->stats.max_launch_ms, dt * 1e3);
      if (dt > 1e-3) s->stats.launches_over_1ms++;
      if (e && s->error.empty()) s->error = cudaGetErrorString(static_cast<cudaError_t>(e));
    }
    {
      // a lane left waiting for a table slot: let launches finish
      std::unique_lock<std::mutex> lk(s->mu);
      if (!s->lanes[0].ready.empty() || !s->lanes[1].ready.empty())
        s->cv.wait_for(lk, std::chrono::microseconds(10));
    }
  }
}

void destroy(ogs_server_s* s) {
  for (cudaEvent_t ev : s->spare_events) cudaEventDestroy(ev);
  for (auto& q : s->all)
    if (q->copied_out) cudaEventDestroy(q->copied_out);
  for (TableSlot& t : s->slots)
    if (t.done) cudaEventDestroy(t.done);
  dev_free(s->d_tables);
  host_free(s->h_tables);
  for (Lane& l : s->lanes) {
    for (cudaStream_t st : {l.in, l.compute, l.out})
      if (st) cudaStreamDestroy(st);
    if (l.copied) cudaEventDestroy(l.copied);
    for (cudaEvent_t ev : l.turn_done)
      if (ev) cudaEventDestroy(ev);
  }
  dev_free(s->pool_base);
  delete s;
}

Req* find_req(ogs_server_s* s, int64_t id) {  // s->mu held
  if (id < 0 || id >= static_cast<int64_t>(s->all.size())) return nullptr;
  return s->all[id].get();
}

bool final_state(int st) { return st == kDone || st == kCancelled; }

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
  cudaError_t e = cudaGetDevice(&s->device);
  if (e == cudaSuccess) e = dev_malloc(&s->pool_base, static_cast<size_t>(cfg->field_budget_bytes));
  if (e == cudaSuccess) s->pool.reset(static_cast<size_t>(cfg->field_budget_bytes));
  s->lanes[0].max_turns = OGS_SERVER_SMALL_TURNS;
  s->lanes[0].turn_bytes = OGS_SERVER_SMALL_TURN_BYTES;
  s->lanes[1].max_turns = OGS_SERVER_LARGE_TURNS;
  s->lanes[1].turn_bytes = OGS_SERVER_LARGE_TURN_BYTES;
  for (Lane& l : s->lanes) {
    for (cudaStream_t* st : {&l.in, &l.compute, &l.out})
      if (e == cudaSuccess) e = cudaStreamCreateWithFlags(st, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&l.copied, cudaEventDisableTiming);
    for (cudaEvent_t& ev : l.turn_done)
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
  }
  // the launch tables of all slots: entries then starts, 256-byte aligned
  const size_t eb = (sizeof(BatchEntry) * cfg->max_batch + 255) / 256 * 256;
  const size_t sb = (sizeof(int64_t) * (cfg->max_batch + 1) + 255) / 256 * 256;
  if (e == cudaSuccess) e = dev_malloc(&s->d_tables, kTableSlots * (eb + sb));
  if (e == cudaSuccess) e = host_malloc(&s->h_tables, kTableSlots * (eb + sb));
  if (e == cudaSuccess) s->slots.resize(kTableSlots);
  for (size_t j = 0; j < s->slots.size(); ++j) {
    TableSlot& t = s->slots[j];
    t.d_entries = reinterpret_cast<BatchEntry*>(s->d_tables + j * (eb + sb));
    t.d_starts = reinterpret_cast<int64_t*>(s->d_tables + j * (eb + sb) + eb);
    t.h_entries = reinterpret_cast<BatchEntry*>(s->h_tables + j * (eb + sb));
    t.h_starts = reinterpret_cast<int64_t*>(s->h_tables + j * (eb + sb) + eb);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&t.done, cudaEventDisableTiming);
  }
  // Everything a first request would otherwise set up on the worker's path:
  // the batched kernels' modules (loaded lazily by the runtime on first use,
  // milliseconds each, during which every request waits), the completion
  // events, and each stream's first operation.
  if (e == cudaSuccess) e = static_cast<cudaError_t>(preload_batch_f32());
  if (e == cudaSuccess) e = static_cast<cudaError_t>(preload_batch_f64());
  if (e == cudaSuccess) e = static_cast<cudaError_t>(preload_batch_i32());
  if (e == cudaSuccess) e = static_cast<cudaError_t>(preload_batch_i64());
  for (int j = 0; e == cudaSuccess && j < kSpareEvents; ++j) {
    cudaEvent_t ev = nullptr;
    e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
    if (e == cudaSuccess) s->spare_events.push_back(ev);
  }
  for (Lane& l : s->lanes)
    for (cudaStream_t st : {l.in, l.compute, l.out}) {
      if (e == cudaSuccess) e = cudaEventRecord(l.copied, st);
      if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    }
  if (e != cudaSuccess) {
    cudaGetLastError();
    destroy(s);
    return set_error(e == cudaErrorMemoryAllocation ? OGS_ENOMEM : OGS_EDEVICE,
                     std::string("ogs_server_create: ") + cudaGetErrorString(e));
  }
  try {
    s->worker = std::thread(worker_loop, s);
  } catch (const std::exception&) {
    destroy(s);
    return set_error(OGS_ENOMEM, "ogs_server_create: cannot start the worker thread");
  }
  *out = s;
  return OGS_OK;
}

ogs_status ogs_server_add_mesh(ogs_server s, ogs_handle h, int* mesh_id) {
  if (!s || !h || !mesh_id) return set_error(OGS_EINVAL, "ogs_server_add_mesh: NULL argument");
  if (h->host_only || h->device != s->device)
    return set_error(OGS_EINVAL, "ogs_server_add_mesh: the handle must live on the server's device");
  if (h->gslib) return set_error(OGS_EINVAL, "ogs_server_add_mesh: handle was made by ogs_gslib_setup");
  if (!h->distinct_cols)
    return set_error(OGS_EINVAL, "ogs_server_add_mesh: a local node appears in two rows of this operator's map");
  std::lock_guard<std::mutex> g(s->mu);
  s->meshes.push_back(h);
  *mesh_id = static_cast<int>(s->meshes.size()) - 1;
  return OGS_OK;
}

ogs_status ogs_server_submit_many(ogs_server s, const ogs_server_request* rs, const double* arrivals, int64_t n,
                                  int64_t* first_id) {
  const char* fn = "ogs_server_submit";
  if (!s || (!rs && n > 0)) return set_error(OGS_EINVAL, std::string(fn) + ": NULL argument");
  if (n < 0) return set_error(OGS_EINVAL, std::string(fn) + ": n must be >= 0");
  std::vector<std::unique_ptr<Req>> qs;
  try {
    qs.reserve(static_cast<size_t>(n));
    for (int64_t i = 0; i < n; ++i) qs.emplace_back(new Req());
  } catch (const std::bad_alloc&) {
    return set_error(OGS_ENOMEM, std::string(fn) + ": out of host memory");
  }
  {
    std::lock_guard<std::mutex> g(s->mu);
    if (s->stop.load()) return set_error(OGS_EINVAL, std::string(fn) + ": the server is shutting down");
    // every request is checked before any is queued
    for (int64_t i = 0; i < n; ++i) {
      const ogs_server_request* r = &rs[i];
      if (r->mesh < 0 || r->mesh >= static_cast<int>(s->meshes.size()))
        return set_error(OGS_EINVAL, std::string(fn) + ": unknown mesh");
      if (r->type < OGS_FLOAT || r->type > OGS_INT64 || r->op < OGS_ADD || r->op > OGS_MIN || r->k < 1 ||
          r->trans < OGS_SYM || r->trans > OGS_TRANS || !r->host)
        return set_error(OGS_EINVAL, std::string(fn) + ": bad request");
      const size_t node_bytes = static_cast<size_t>(r->k) * type_size(r->type);
      const size_t nn = static_cast<size_t>(s->meshes[r->mesh]->N);
      if (nn > 0 && node_bytes > static_cast<size_t>(s->cfg.field_budget_bytes) / nn)
        return set_error(OGS_ERANGE, std::string(fn) + ": the field is larger than the whole budget");
      if (static_cast<int64_t>(s->meshes[r->mesh]->dmaps.nwtiles) * r->k > INT32_MAX)
        return set_error(OGS_ERANGE, std::string(fn) + ": more than 2^31 work items in one request");
    }
    try {
      s->all.reserve(s->all.size() + static_cast<size_t>(n));
    } catch (const std::bad_alloc&) {
      return set_error(OGS_ENOMEM, std::string(fn) + ": out of host memory");
    }
    const double now = now_s();
    if (first_id) *first_id = static_cast<int64_t>(s->all.size());
    for (int64_t i = 0; i < n; ++i) {
      Req* q = qs[i].get();
      q->r = rs[i];
      q->bytes = static_cast<size_t>(s->meshes[rs[i].mesh]->N) * static_cast<size_t>(rs[i].k) * type_size(rs[i].type);
      q->t_arrival = arrivals && arrivals[i] > 0 ? arrivals[i] : now;
      q->id = static_cast<int64_t>(s->all.size());
      s->pending.push_back(q);
      s->all.push_back(std::move(qs[i]));
    }
  }
  s->submitted.fetch_add(n);
  s->cv.notify_all();
  return OGS_OK;
}

ogs_status ogs_server_submit(ogs_server s, const ogs_server_request* r, double arrival, int64_t* id) {
  if (!r) return set_error(OGS_EINVAL, "ogs_server_submit: NULL argument");
  return ogs_server_submit_many(s, r, &arrival, 1, id);
}

double ogs_server_clock(void) { return now_s(); }

ogs_status ogs_server_wait_for(ogs_server s, int64_t id, double timeout_s) {
  if (!s) return set_error(OGS_EINVAL, "ogs_server_wait: NULL server");
  const auto deadline = std::chrono::steady_clock::now() +
                        std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                            std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 0.0));
  std::unique_lock<std::mutex> lk(s->mu);
  Req* q = find_req(s, id);
  if (!q) return set_error(OGS_EINVAL, "ogs_server_wait: unknown id");
  while (!final_state(q->state.load())) {
    if (!s->error.empty()) return set_error(OGS_EDEVICE, "ogs_server: " + s->error);
    if (timeout_s >= 0 && std::chrono::steady_clock::now() >= deadline)
      return set_error(OGS_ETIMEOUT, "ogs_server_wait: request " + std::to_string(id) + " still running");
    s->cv.wait_for(lk, std::chrono::milliseconds(1));
  }
  return OGS_OK;
}

ogs_status ogs_server_wait(ogs_server s, int64_t id) { return ogs_server_wait_for(s, id, -1.0); }

ogs_status ogs_server_cancel(ogs_server s, int64_t id, int* cancelled) {
  if (!s) return set_error(OGS_EINVAL, "ogs_server_cancel: NULL server");
  bool done_now = false;
  {
    std::lock_guard<std::mutex> g(s->mu);
    Req* q = find_req(s, id);
    if (!q) return set_error(OGS_EINVAL, "ogs_server_cancel: unknown id");
    if (q->state.load() == kPending) {
      s->pending.erase(std::find(s->pending.begin(), s->pending.end(), q));
      q->state.store(kCancelled);
      done_now = true;
    }
  }
  if (done_now) {
    s->completed.fetch_add(1);
    s->cv.notify_all();
  }
  if (cancelled) *cancelled = done_now ? 1 : 0;
  return OGS_OK;
}

ogs_status ogs_server_state(ogs_server s, int64_t id, int* state) {
  if (!s || !state) return set_error(OGS_EINVAL, "ogs_server_state: NULL argument");
  std::lock_guard<std::mutex> g(s->mu);
  Req* q = find_req(s, id);
  if (!q) return set_error(OGS_EINVAL, "ogs_server_state: unknown id");
  *state = q->state.load();
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

ogs_status ogs_server_times(ogs_server s, int64_t first, int64_t n, double* arrival, double* launched,
                            double* done) {
  if (!s) return set_error(OGS_EINVAL, "ogs_server_times: NULL server");
  std::lock_guard<std::mutex> g(s->mu);
  if (first < 0 || n < 0 || first + n > static_cast<int64_t>(s->all.size()))
    return set_error(OGS_EINVAL, "ogs_server_times: range out of bounds");
  for (int64_t i = 0; i < n; ++i) {
    const Req* q = s->all[first + i].get();
    const int st = q->state.load();
    if (arrival) arrival[i] = q->t_arrival;
    if (launched) launched[i] = st == kPending || st == kCancelled ? -1.0 : q->t_launch;
    if (done) done[i] = st == kDone ? q->t_done : -1.0;
  }
  return OGS_OK;
}

ogs_status ogs_server_latencies(ogs_server s, int64_t first, int64_t n, double* arrival, double* done) {
  return ogs_server_times(s, first, n, arrival, nullptr, done);
}

ogs_status ogs_server_get_stats(ogs_server s, ogs_server_stats* out) {
  if (!s || !out) return set_error(OGS_EINVAL, "ogs_server_get_stats: NULL argument");
  std::lock_guard<std::mutex> g(s->mu);
  *out = s->stats;
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
