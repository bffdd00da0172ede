// ogs_batch.cuh -- one persistent launch over many meshes' gather-scatters.
//
// A batch is a list of entries (mesh handle, field, k, op, transpose).  Each
// handle carries, from setup, one 32-byte record per warp tile (WarpRec:
// column and row arrays of its bucket, first row, degree and row count); the
// batch adds a prefix table `starts` over the entries' record counts.  Warp w
// of the grid takes records w, w+W, ... of the concatenated list, finds the
// record's entry by binary search (in shared memory for up to kBatchSmem
// entries), and runs the same per-warp pipeline as ogs_warp.cuh: the next
// record's column ids load while the current record's k components are
// gathered, folded and stored.  The fold follows ogsOperator.cpp:311-360 with
// the entry's op chosen at run time (warp-uniform), so one launch serves
// entries with different ops.
#pragma once

#include "ogs_warp.cuh"

namespace ogsgb {

constexpr int kBatchSmem = 2048;

template <int D>
__device__ __forceinline__ void rec_to_tile(const WarpRec& r, DevBucket& b, Tile& t) {
  b.cols = r.cols;
  b.rows = r.rows;
  b.nmask = nullptr;
  b.n = 0;
  b.nP = r.nP;
  b.stride = r.stride;
  t.bucket = D;
  t.begin = r.begin;
  t.count = r.bucket_count & 0xFFFF;
  t.first_row = 0;
}

template <typename T, int D>
__device__ __forceinline__ void fold_store_rt(int op, const WarpState& s, T* dst, int64_t stride, int K, int k,
                                              bool gmask, bool smask, int lane, const T (&V)[kWarpSlots]) {
  switch (op) {
    case OGS_ADD: warp_fold_store<T, OGS_ADD, kModeGS, D>(s, dst, nullptr, stride, K, k, gmask, smask, lane, V); break;
    case OGS_MUL: warp_fold_store<T, OGS_MUL, kModeGS, D>(s, dst, nullptr, stride, K, k, gmask, smask, lane, V); break;
    case OGS_MAX: warp_fold_store<T, OGS_MAX, kModeGS, D>(s, dst, nullptr, stride, K, k, gmask, smask, lane, V); break;
    default: warp_fold_store<T, OGS_MIN, kModeGS, D>(s, dst, nullptr, stride, K, k, gmask, smask, lane, V); break;
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

template <typename T>
__global__ void __launch_bounds__(kBlock, OGS_WARP_MINB) ogs_batch_kernel(const BatchEntry* __restrict__ E,
                                                                          const int64_t* __restrict__ starts,
                                                                          int n) {
  __shared__ int64_t s_starts[kBatchSmem + 1];
  const bool in_smem = n <= kBatchSmem;
  if (in_smem)
    for (int j = threadIdx.x; j <= n; j += kBlock) s_starts[j] = starts[j];
  __syncthreads();
  const int64_t* st = in_smem ? s_starts : starts;
  const int64_t nitems = st[n];
  const int lane = static_cast<int>(threadIdx.x) & 31;
  const int64_t W = static_cast<int64_t>(gridDim.x) * (kBlock / 32);
  int64_t i = static_cast<int64_t>(blockIdx.x) * (kBlock / 32) + (threadIdx.x >> 5);
  if (i >= nitems) return;

  // current record: its entry, tile and column ids
  int ecur = batch_entry_of(st, n, i);
  BatchEntry bcur = E[ecur];
  int64_t rcur = i - st[ecur];
  WarpRec wcur = bcur.recs[rcur];
  WarpState scur;
  {
    const Pattern pat{bcur.gather_n, bcur.scatter_n, bcur.limit_n};
    DevBucket b;
    Tile t;
#define OGS_B_LOAD_CUR(D) \
  rec_to_tile<D>(wcur, b, t); \
  warp_load_state<kModeGS, D>(b, t, bcur.wemask, static_cast<int>(rcur), bcur.use_mask, pat, lane, scur)
    OGS_DEGREE_SWITCH(wcur.bucket_count >> 16, OGS_B_LOAD_CUR)
#undef OGS_B_LOAD_CUR
  }
  // next record's entry and descriptor
  int enxt = 0;
  BatchEntry bnxt{};
  int64_t rnxt = 0;
  WarpRec wnxt{};
  if (i + W < nitems) {
    enxt = batch_entry_of(st, n, i + W);
    bnxt = E[enxt];
    rnxt = i + W - st[enxt];
    wnxt = bnxt.recs[rnxt];
  }

  for (;;) {
    const bool more = i + W < nitems;
    const int K = bcur.K;
    if (lane == 0) {
      FieldArgs fa{};
      fa.v = bcur.v;
      prefetch_ahead<T>(fa, K, wcur.pf_lo, wcur.pf_hi, wcur.pf_cols, wcur.pf_stride, wcur.pf_begin,
                        wcur.pf_bucket_count);
    }
    const bool gmask = bcur.gather_n != 0, smask = bcur.scatter_n != 0;
    const int d = wcur.bucket_count >> 16;
    WarpState snxt;
    int enn = 0;
    BatchEntry bnn{};
    int64_t rnn = 0;
    WarpRec wnn{};
    for (int k = 0; k < K; ++k) {
      T* base = static_cast<T*>(bcur.v) + k;
      T V[kWarpSlots];
#define OGS_B_VALS(D) warp_load_vals<T, kModeGS, D>(scur, base, nullptr, K, K, k, gmask, lane, V)
      OGS_DEGREE_SWITCH(d, OGS_B_VALS)
#undef OGS_B_VALS
      if (k == 0 && more) {
        const Pattern pat{bnxt.gather_n, bnxt.scatter_n, bnxt.limit_n};
        DevBucket b;
        Tile t;
#define OGS_B_LOAD_NXT(D) \
  rec_to_tile<D>(wnxt, b, t); \
  warp_load_state<kModeGS, D>(b, t, bnxt.wemask, static_cast<int>(rnxt), bnxt.use_mask, pat, lane, snxt)
        OGS_DEGREE_SWITCH(wnxt.bucket_count >> 16, OGS_B_LOAD_NXT)
#undef OGS_B_LOAD_NXT
        if (i + 2 * W < nitems) {
          enn = batch_entry_of(st, n, i + 2 * W);
          bnn = E[enn];
          rnn = i + 2 * W - st[enn];
          wnn = bnn.recs[rnn];
        }
      }
#define OGS_B_FOLD(D) fold_store_rt<T, D>(bcur.op, scur, base, K, K, k, gmask, smask, lane, V)
      OGS_DEGREE_SWITCH(d, OGS_B_FOLD)
#undef OGS_B_FOLD
    }
    if (!more) break;
    i += W;
    bcur = bnxt;
    rcur = rnxt;
    wcur = wnxt;
    scur = snxt;
    bnxt = bnn;
    rnxt = rnn;
    wnxt = wnn;
  }
}

template <typename T>
inline int batch_blocks_per_sm(int* sms) {
  static int cached_dev = -1, cached_bps = 0, cached_sms = 0;
  int dev = 0;
  cudaGetDevice(&dev);
  if (dev != cached_dev) {
    int bps = 0, s = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ogs_batch_kernel<T>, kBlock, 0);
    cudaDeviceGetAttribute(&s, cudaDevAttrMultiProcessorCount, dev);
    cached_bps = bps > 0 ? bps : 1;
    cached_sms = s > 0 ? s : 1;
    cached_dev = dev;
  }
  *sms = cached_sms;
  return cached_bps;
}

// grid <= 0: resident CTAs on every SM.
template <typename T>
inline int launch_batch_typed(const BatchEntry* E, const int64_t* starts, int n, int64_t nitems, int grid,
                              void* stream) {
  if (nitems <= 0) return 0;
  int sms = 0;
  const int bps = batch_blocks_per_sm<T>(&sms);
  int64_t g = grid > 0 ? grid : static_cast<int64_t>(bps) * sms;
  const int64_t need = (nitems + (kBlock / 32) - 1) / (kBlock / 32);
  if (g > need) g = need;
  ogs_batch_kernel<T><<<static_cast<unsigned>(g), kBlock, 0, static_cast<cudaStream_t>(stream)>>>(E, starts, n);
  return static_cast<int>(cudaGetLastError());
}

}  // namespace ogsgb
