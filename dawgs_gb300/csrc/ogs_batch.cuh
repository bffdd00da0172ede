// ogs_batch.cuh -- one persistent launch over many meshes' gather-scatters.
//
// A batch is a list of entries (mesh handle, field, k, op, transpose).  Each
// handle carries, from setup, one 32-byte record per warp tile (WarpRec:
// column and row arrays of its bucket, first row, degree and row count); the
// batch adds a prefix table `starts` over the entries' (record, component)
// items.  Warp w of the grid takes items w, w+W, ..., finds an item's entry
// by binary search (in shared memory for up to kBatchSmem entries), and runs
// the same per-warp pipeline as ogs_warp.cuh: the next item's column ids load
// while the current item's values are gathered, folded and stored.  The fold follows
// ogsOperator.cpp:311-360 with the entry's op chosen at run time
// (warp-uniform), so one launch serves entries with different ops.
#pragma once

#include "ogs_async.cuh"
#include "ogs_warp.cuh"

namespace ogsgb {

constexpr int kBatchSmem = 2048;

// The batched kernel comes in two register budgets, chosen per launch by the
// tuner: OCC 256-thread CTAs resident per SM (2: 107 registers, no spills;
// 3: 80 registers, a few spilled bytes, half as many warps again).

template <typename T, int D>
__device__ __forceinline__ void fold_store_rt(int op, const WarpState& s, T* dst, int64_t stride, int K, int k,
                                              bool gmask, int smode, int lane, const T (&V)[kWarpSlots]) {
  switch (op) {
    case OGS_ADD: warp_fold_store<T, OGS_ADD, kModeGS, D>(s, dst, nullptr, stride, K, k, gmask, smode, false, lane, V); break;
    case OGS_MUL: warp_fold_store<T, OGS_MUL, kModeGS, D>(s, dst, nullptr, stride, K, k, gmask, smode, false, lane, V); break;
    case OGS_MAX: warp_fold_store<T, OGS_MAX, kModeGS, D>(s, dst, nullptr, stride, K, k, gmask, smode, false, lane, V); break;
    default: warp_fold_store<T, OGS_MIN, kModeGS, D>(s, dst, nullptr, stride, K, k, gmask, smode, false, lane, V); break;
  }
}

__device__ __forceinline__ int batch_entry_of(const int64_t* starts, int n, int64_t item) {
  int lo = 0, hi = n - 1;  // largest e with starts[e] <= item
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (starts[mid] <= item) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// A thread's (row lane, component) in part `part` of an entry's record: as
// in the single-mesh kernel, a record's 32 row lanes x K components are split
// over its K items, so neighbouring threads read neighbouring components of
// one node.
__device__ __forceinline__ void batch_unit(int K, uint32_t kmagic, int part, int lane, int& rl, int& comp) {
  if (K == 1) {
    rl = lane;
    comp = 0;
    return;
  }
  const uint32_t u = static_cast<uint32_t>(part) * 32u + static_cast<uint32_t>(lane);
  rl = static_cast<int>(kmagic ? __umulhi(u, kmagic) : u / static_cast<uint32_t>(K));
  comp = static_cast<int>(u) - rl * K;
}

// One work item, (entry e, warp record r, part), reduced to what the fold
// needs: field, masks, column ids of the record's bucket and its tile, and
// the thread's component k and row lane.
struct BatchItem {
  const WarpRec* recs;
  const int32_t* cols;
  void* v;
  const uint8_t* wemask;
  int32_t K, flags;  // flags: op | gather_n << 4 | scatter_n << 5 | limit_n << 6 | use_mask << 7 | row lane << 8
  int32_t e, r, k;
  int32_t begin, bucket_count, stride, nP;
};

__device__ __forceinline__ int item_lane(const BatchItem& it) { return (it.flags >> 8) & 31; }

__device__ __forceinline__ void batch_load_entry(const BatchEntry* E, int e, BatchItem& it) {
  const BatchEntry& be = E[e];
  it.recs = be.recs;
  it.v = be.v;
  it.wemask = be.wemask;
  it.K = be.K;
  it.flags = be.op | (be.gather_n << 4) | (be.scatter_n << 5) | (be.limit_n << 6) | (be.use_mask << 7);
  it.e = e;
}

__device__ __forceinline__ void batch_load_rec(BatchItem& it) {
  const WarpRec& w = it.recs[it.r];
  it.cols = w.cols;
  it.begin = w.begin;
  it.bucket_count = w.bucket_count;
  it.stride = w.stride;
  it.nP = w.nP;
}

// The item at global index i: its entry by binary search over the prefix,
// then its record and component.
__device__ __forceinline__ void batch_item_at(const BatchEntry* E, const int64_t* st, int n, int64_t i, int lane,
                                              BatchItem& it) {
  batch_load_entry(E, batch_entry_of(st, n, i), it);
  const int32_t local = static_cast<int32_t>(i - st[it.e]);  // items of one entry fit 32 bits
  it.r = local / it.K;
  int rl, comp;
  batch_unit(it.K, E[it.e].kmagic, local - it.r * it.K, lane, rl, comp);
  it.k = comp;
  it.flags |= rl << 8;
  batch_load_rec(it);
}

template <bool PLAIN>
__device__ __forceinline__ void batch_load_state(const BatchItem& it, WarpState& s) {
  const int lane = item_lane(it);
  const Pattern pat = PLAIN ? Pattern{0, 0, 0} : Pattern{(it.flags >> 4) & 1, (it.flags >> 5) & 1, (it.flags >> 6) & 1};
  DevBucket b;
  b.cols = it.cols;
  b.rows = nullptr;
  b.nmask = nullptr;
  b.n = INT32_MAX;  // the records carry no bucket sizes: batched launches are not id-checked
  b.nP = it.nP;
  b.stride = it.stride;
  b.nnodes = INT32_MAX;
  b.nrows = INT32_MAX;
  b.err = nullptr;
  Tile t;
  t.begin = it.begin;
  t.count = it.bucket_count & 0xFFFF;
  t.first_row = 0;
  const bool use_mask = !PLAIN && ((it.flags >> 7) & 1);
#define OGS_B_LOAD(D) t.bucket = D; warp_load_state<kModeGS, D>(b, t, it.wemask, it.r, use_mask, pat, lane, s)
  OGS_DEGREE_SWITCH(it.bucket_count >> 16, OGS_B_LOAD)
#undef OGS_B_LOAD
}

// Warp w takes items w, w+W, ... of the (entry, record, component) items, so
// the grid sweeps every mesh front to back and the k components of a record
// run on neighbouring warps at once, sharing its column ids and the field's
// sectors through L1/L2 (a warp walking a contiguous run of items was much
// slower on large meshes, as for the single-mesh kernel).  The prefix
// `starts` is staged in shared memory (dynamic, (n+1) entries) when it fits.
// PLAIN: every entry folds and stores every member (no N masks, no limit on
// the rows): the mask and store-mode branches drop out at compile time.
template <typename T, int BLOCK, int OCC, bool PLAIN>
__global__ void __launch_bounds__(BLOCK, OCC * 256 / BLOCK)
    ogs_batch_kernel(const BatchEntry* __restrict__ E, const int64_t* __restrict__ starts, int n) {
  extern __shared__ int64_t s_starts[];
  const bool in_smem = n <= kBatchSmem;
  if (in_smem)
    for (int j = threadIdx.x; j <= n; j += BLOCK) s_starts[j] = starts[j];
  __syncthreads();
  const int64_t* st = in_smem ? s_starts : starts;
  const int64_t nitems = st[n];
  const int lane = static_cast<int>(threadIdx.x) & 31;
  const int64_t W = static_cast<int64_t>(gridDim.x) * (BLOCK / 32);
  int64_t i = static_cast<int64_t>(blockIdx.x) * (BLOCK / 32) + (threadIdx.x >> 5);
  if (i >= nitems) return;

  BatchItem cur, nxt;
  batch_item_at(E, st, n, i, lane, cur);
  WarpState scur;
  batch_load_state<PLAIN>(cur, scur);
  if (i + W < nitems) batch_item_at(E, st, n, i + W, lane, nxt);

  for (;;) {
    const bool more = i + W < nitems;
    const int K = cur.K, k = cur.k, d = cur.bucket_count >> 16, rl = item_lane(cur);
    const bool gmask = !PLAIN && ((cur.flags >> 4) & 1);
    const int smode = PLAIN ? 0 : (cur.flags >> 5) & 1;
    T* base = static_cast<T*>(cur.v) + k;
    T V[kWarpSlots];
#define OGS_B_VALS(D) warp_load_vals<T, kModeGS, D>(scur, base, nullptr, K, K, k, gmask, rl, V)
    OGS_DEGREE_SWITCH(d, OGS_B_VALS)
#undef OGS_B_VALS
    WarpState snxt;
    BatchItem nn;
    if (more) {
      batch_load_state<PLAIN>(nxt, snxt);
      if (i + 2 * W < nitems) batch_item_at(E, st, n, i + 2 * W, lane, nn);
    }
#define OGS_B_FOLD(D) fold_store_rt<T, D>(cur.flags & 15, scur, base, K, K, k, gmask, smode, rl, V)
    OGS_DEGREE_SWITCH(d, OGS_B_FOLD)
#undef OGS_B_FOLD
    if (!more) break;
    i += W;
    cur = nxt;
    scur = snxt;
    nxt = nn;
  }
}

template <typename T, int BLOCK, int OCC, bool PLAIN>
inline int batch_blocks_per_sm(int* sms) {
  static DeviceCache bps_cache, sms_cache;
  int dev = 0;
  cudaGetDevice(&dev);
  *sms = sms_cache.get(dev, [dev] {
    int s = 0;
    cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
    return s > 0 ? s : 1;
  });
  // occupancy with the largest starts table (the registers decide it)
  return bps_cache.get(dev, [] {
    int bps = 0;
    cudaFuncSetAttribute(ogs_batch_kernel<T, BLOCK, OCC, PLAIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>((kBatchSmem + 1) * sizeof(int64_t)));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ogs_batch_kernel<T, BLOCK, OCC, PLAIN>, BLOCK, 0);
    return bps > 0 ? bps : 1;
  });
}

template <typename T, int BLOCK, int OCC, bool PLAIN>
inline int launch_batch_shape(const BatchEntry* E, const int64_t* starts, int n, int64_t nitems, int grid,
                              cudaStream_t st) {
  int sms = 0;
  const int bps = batch_blocks_per_sm<T, BLOCK, OCC, PLAIN>(&sms);
  int64_t g = grid > 0 ? grid : static_cast<int64_t>(bps) * sms;
  const int64_t need = (nitems + (BLOCK / 32) - 1) / (BLOCK / 32);
  if (g > need) g = need;
  const size_t smem = n <= kBatchSmem ? static_cast<size_t>(n + 1) * sizeof(int64_t) : 0;
  ogs_batch_kernel<T, BLOCK, OCC, PLAIN><<<static_cast<unsigned>(g), BLOCK, smem, st>>>(E, starts, n);
  return static_cast<int>(cudaGetLastError());
}

// ---- the same batch on the cp.async ring (ogs_async.cuh) ----
// Each warp keeps two items' value gathers and a third item's column ids in
// flight, as the single-mesh kernel does.  To leave room for that in 80
// registers, a lookahead item is carried as its position only -- entry,
// record, component, degree -- and its field, op and record are read again
// from the entry table and the record (L1-resident) where they are needed.
struct BatchPos {
  int32_t e, r, k, d;  // k: the thread's component; d: degree | row lane << 8
};

__device__ __forceinline__ int pos_deg(const BatchPos& p) { return p.d & 0xFF; }
__device__ __forceinline__ int pos_lane(const BatchPos& p) { return p.d >> 8; }

__device__ __forceinline__ BatchPos batch_pos(const BatchEntry* E, const int64_t* st, int n, int64_t i, int lane) {
  BatchPos p;
  p.e = batch_entry_of(st, n, i);
  const int K = E[p.e].K;
  const int32_t local = static_cast<int32_t>(i - st[p.e]);  // items of one entry fit 32 bits
  p.r = local / K;
  int rl, comp;
  batch_unit(K, E[p.e].kmagic, local - p.r * K, lane, rl, comp);
  p.k = comp;
  p.d = (E[p.e].recs[p.r].bucket_count >> 16) | (rl << 8);
  return p;
}

template <int D, bool PLAIN>
__device__ __forceinline__ void batch_state_at(const BatchEntry* E, const BatchPos& p, WarpState& s) {
  const int lane = pos_lane(p);
  const BatchEntry& be = E[p.e];
  const WarpRec& w = be.recs[p.r];
  DevBucket b;
  b.cols = w.cols;
  b.rows = nullptr;
  b.nmask = nullptr;
  b.n = INT32_MAX;
  b.nP = w.nP;
  b.stride = w.stride;
  b.nnodes = INT32_MAX;
  b.nrows = INT32_MAX;
  b.err = nullptr;
  Tile t;
  t.bucket = D;
  t.begin = w.begin;
  t.count = w.bucket_count & 0xFFFF;
  t.first_row = 0;
  const Pattern pat = PLAIN ? Pattern{0, 0, 0} : Pattern{be.gather_n, be.scatter_n, be.limit_n};
  warp_load_state<kModeGS, D>(b, t, be.wemask, p.r, !PLAIN && be.use_mask != 0, pat, lane, s);
}

template <typename T>
OGS_HD constexpr size_t batch_ring_bytes() {  // 8 warps x 2 stages x kWarpSlots x 32 values
  return static_cast<size_t>(kBlock / 32) * kAsyncStages * kWarpSlots * 32 * sizeof(T);
}

template <typename T, int OCC, bool PLAIN>
__global__ void __launch_bounds__(kBlock, OCC)
    ogs_batch_async_kernel(const BatchEntry* __restrict__ E, const int64_t* __restrict__ starts, int n) {
  extern __shared__ __align__(16) unsigned char batch_smem[];
  const int lane = static_cast<int>(threadIdx.x) & 31;
  const int warp = static_cast<int>(threadIdx.x) >> 5;
  T* ring = reinterpret_cast<T*>(batch_smem) + static_cast<size_t>(warp) * kAsyncStages * kWarpSlots * 32;
  int64_t* s_starts = reinterpret_cast<int64_t*>(batch_smem + batch_ring_bytes<T>());
  const bool in_smem = n <= kBatchSmem;
  if (in_smem)
    for (int j = threadIdx.x; j <= n; j += kBlock) s_starts[j] = starts[j];
  __syncthreads();
  const int64_t* st = in_smem ? s_starts : starts;
  const int64_t nitems = st[n];
  const int64_t W = static_cast<int64_t>(gridDim.x) * (kBlock / 32);
  int64_t i = static_cast<int64_t>(blockIdx.x) * (kBlock / 32) + warp;
  if (i >= nitems) return;

  BatchPos cur = batch_pos(E, st, n, i, lane), nxt{}, nn{};
  const bool has1 = i + W < nitems;
  if (has1) nxt = batch_pos(E, st, n, i + W, lane);
  if (i + 2 * W < nitems) nn = batch_pos(E, st, n, i + 2 * W, lane);
  WarpState scur, snxt;
#define OGS_BA_STATE(D, P, S) batch_state_at<D, PLAIN>(E, P, S)
#define OGS_BA_CUR(D) OGS_BA_STATE(D, cur, scur)
  OGS_DEGREE_SWITCH(pos_deg(cur), OGS_BA_CUR)
#undef OGS_BA_CUR
  if (has1) {
#define OGS_BA_NXT(D) OGS_BA_STATE(D, nxt, snxt)
    OGS_DEGREE_SWITCH(pos_deg(nxt), OGS_BA_NXT)
#undef OGS_BA_NXT
  }
  {
    const BatchEntry& be = E[cur.e];
    const T* src = static_cast<const T*>(be.v) + cur.k;
    const bool gmask = !PLAIN && be.gather_n != 0;
#define OGS_BA_ISSUE0(D) \
  async_issue_vals<T, kModeGS, D>(scur, src, nullptr, be.K, be.K, cur.k, gmask, pos_lane(cur), lane, ring)
    OGS_DEGREE_SWITCH(pos_deg(cur), OGS_BA_ISSUE0)
#undef OGS_BA_ISSUE0
  }
  cp_async_commit();

  int stage = 0;
  for (;;) {
    const bool more1 = i + W < nitems;
    const bool more2 = i + 2 * W < nitems;
    const int nstage = stage == kAsyncStages - 1 ? 0 : stage + 1;
    if (more1) {
      const BatchEntry& be = E[nxt.e];
      const T* src1 = static_cast<const T*>(be.v) + nxt.k;
      const bool gmask1 = !PLAIN && be.gather_n != 0;
      T* st1 = ring + nstage * (kWarpSlots * 32);
#define OGS_BA_ISSUE1(D) \
  async_issue_vals<T, kModeGS, D>(snxt, src1, nullptr, be.K, be.K, nxt.k, gmask1, pos_lane(nxt), lane, st1)
      OGS_DEGREE_SWITCH(pos_deg(nxt), OGS_BA_ISSUE1)
#undef OGS_BA_ISSUE1
    }
    cp_async_commit();
    WarpState snn;
    BatchPos n3{};
    if (more2) {
#define OGS_BA_NN(D) OGS_BA_STATE(D, nn, snn)
      OGS_DEGREE_SWITCH(pos_deg(nn), OGS_BA_NN)
#undef OGS_BA_NN
      if (i + 3 * W < nitems) n3 = batch_pos(E, st, n, i + 3 * W, lane);
    }
    cp_async_wait<1>();  // the gathers of item i are in
    {
      const BatchEntry& be = E[cur.e];
      const int K = be.K;
      T* dst = static_cast<T*>(be.v) + cur.k;
      const bool gmask = !PLAIN && be.gather_n != 0;
      const int smode = PLAIN ? 0 : be.scatter_n;
      const int op = be.op;
      const T* st0 = ring + stage * (kWarpSlots * 32);
      T V[kWarpSlots];
#define OGS_BA_FOLD(D)                                                            \
  do {                                                                            \
    async_read_vals<T, kModeGS, D>(scur, gmask, pos_lane(cur), lane, st0, V);     \
    fold_store_rt<T, D>(op, scur, dst, K, K, cur.k, gmask, smode, pos_lane(cur), V); \
  } while (0)
      OGS_DEGREE_SWITCH(pos_deg(cur), OGS_BA_FOLD)
#undef OGS_BA_FOLD
    }
    if (!more1) break;
    i += W;
    stage = nstage;
    cur = nxt;
    scur = snxt;
    nxt = nn;
    snxt = snn;
    nn = n3;
  }
  cp_async_wait<0>();
#undef OGS_BA_STATE
}

template <typename T, int OCC, bool PLAIN>
inline int batch_async_blocks_per_sm(int* sms) {
  static DeviceCache bps_cache, sms_cache;
  int dev = 0;
  cudaGetDevice(&dev);
  *sms = sms_cache.get(dev, [dev] {
    int s = 0;
    cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
    return s > 0 ? s : 1;
  });
  return bps_cache.get(dev, [] {
    int bps = 0;
    const size_t smem = batch_ring_bytes<T>() + (kBatchSmem + 1) * sizeof(int64_t);
    cudaFuncSetAttribute(ogs_batch_async_kernel<T, OCC, PLAIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(smem));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ogs_batch_async_kernel<T, OCC, PLAIN>, kBlock,
                                                  batch_ring_bytes<T>() + 257 * sizeof(int64_t));
    return bps > 0 ? bps : 1;
  });
}

template <typename T, int OCC, bool PLAIN>
inline int launch_batch_async_shape(const BatchEntry* E, const int64_t* starts, int n, int64_t nitems, int grid,
                                    cudaStream_t st) {
  int sms = 0;
  const int bps = batch_async_blocks_per_sm<T, OCC, PLAIN>(&sms);
  int64_t g = grid > 0 ? grid : static_cast<int64_t>(bps) * sms;
  const int64_t need = (nitems + (kBlock / 32) - 1) / (kBlock / 32);
  if (g > need) g = need;
  const size_t smem = batch_ring_bytes<T>() + (n <= kBatchSmem ? static_cast<size_t>(n + 1) * sizeof(int64_t) : 0);
  ogs_batch_async_kernel<T, OCC, PLAIN><<<static_cast<unsigned>(g), kBlock, smem, st>>>(E, starts, n);
  return static_cast<int>(cudaGetLastError());
}

// Load the batched kernel of one launch shape and fill its occupancy cache
// now, so that a server's first request does not wait for the module load.
template <typename T, int BLOCK, int OCC>
inline int preload_batch_shape() {
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, ogs_batch_kernel<T, BLOCK, OCC, true>);
  if (e == cudaSuccess) e = cudaFuncGetAttributes(&a, ogs_batch_kernel<T, BLOCK, OCC, false>);
  int sms = 0;
  if (e == cudaSuccess) batch_blocks_per_sm<T, BLOCK, OCC, true>(&sms);
  if (e == cudaSuccess) batch_blocks_per_sm<T, BLOCK, OCC, false>(&sms);
  return static_cast<int>(e);
}

// grid <= 0: resident CTAs on every SM; grid > 0: that many CTAs.  block:
// 128 or 256 threads per CTA; occ: the register budget, 2 or 3 256-thread
// CTAs per SM; pipe 0: the register pipeline, 1: the cp.async ring.
// pipe 1: the cp.async ring (256-thread blocks; occ 2 or 3).
template <typename T, bool PLAIN>
inline int launch_batch_plain(const BatchEntry* E, const int64_t* starts, int n, int64_t nitems, int grid, int block,
                              int occ, int pipe, cudaStream_t st) {
  if (pipe == 1)
    return occ == 3 ? launch_batch_async_shape<T, 3, PLAIN>(E, starts, n, nitems, grid, st)
                    : launch_batch_async_shape<T, 2, PLAIN>(E, starts, n, nitems, grid, st);
  if (block == 128)
    return occ == 3 ? launch_batch_shape<T, 128, 3, PLAIN>(E, starts, n, nitems, grid, st)
                    : launch_batch_shape<T, 128, 2, PLAIN>(E, starts, n, nitems, grid, st);
  return occ == 3 ? launch_batch_shape<T, 256, 3, PLAIN>(E, starts, n, nitems, grid, st)
                  : launch_batch_shape<T, 256, 2, PLAIN>(E, starts, n, nitems, grid, st);
}

// plain: every entry has the plain pattern (Sym or no masks; see ogs_batch_kernel).
template <typename T>
inline int launch_batch_typed(const BatchEntry* E, const int64_t* starts, int n, int64_t nitems, int grid,
                              int block, int occ, int pipe, int plain, void* stream) {
  if (nitems <= 0) return 0;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  return plain ? launch_batch_plain<T, true>(E, starts, n, nitems, grid, block, occ, pipe, st)
               : launch_batch_plain<T, false>(E, starts, n, nitems, grid, block, occ, pipe, st);
}

}  // namespace ogsgb
