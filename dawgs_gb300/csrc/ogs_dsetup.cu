// ogs_dsetup.cu -- the N and T CSR maps of a handle, built on the GPU.
//
// Produces exactly what build_host_maps (ogs_setup.cpp) produces: the maps of
// ogsBase_t::Setup at one rank (libs/ogs/ogsSetup.cpp:69-190, 333-433,
// 569-776).  Rows are the distinct |id| groups, numbered by first appearance
// in local order with the groups that have a positive member first; each
// row's members are in ascending local index; zero ids take no part; with
// `unique` the lowest local index of each group keeps its positive id
// (ogsSetup.cpp:138-141 picks one member; this library always picks the
// first).  The host pass over a hash table becomes:
//   1. a stable radix sort of (|id|, local index) pairs over the key bits in
//      use, so each group is a run of ascending local indices and zero ids
//      form one run in front;
//   2. group heads, and inclusive/exclusive scans for group numbers and for
//      the positive members before each member;
//   3. per group: start, size, positive count, first (= lowest) member; a mark
//      at the first member, packed as (non-positive << 32 | positive), and one
//      exclusive scan over the local nodes that ranks positive and
//      non-positive groups by first appearance -- no second sort;
//   4. row degrees, scans for the row starts, and a scatter of every member
//      to its slot in the T map (and the N map for Signed handles).
// With `layout`, the degree buckets, tiles and the rest of the kernels'
// layout are built on the device too (build_device_layout), in the arena the
// host path would upload; the maps then go back to the host for
// ogs_get_maps.  Both paths give identical handles.
//
// Every buffer here is scratch of the setup call and is freed before it
// returns.  Device memory needed: about 70 bytes per local node.
#include <algorithm>
#include <cstdint>
#include <limits>
#include <string>
#include <vector>

#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include "ogs_internal.hpp"
#include "ogs_trace.hpp"

namespace ogsgb {
namespace {

constexpr int kT = 256;

inline unsigned nblocks(int64_t n) {
  const int64_t b = (n + kT - 1) / kT;
  return static_cast<unsigned>(b > 0 ? b : 1);
}

// flags[0]: an id equal to -2^63; flags[1]: a group without exactly one
// positive member; flags[2]: the largest group.
struct Counters {
  unsigned long long maxkey;
  unsigned long long zeros;
  int flags[3];
};

// Grid of the kernels that end in a global reduction: grid-stride loops, one
// atomic per block, so a few hundred atomics meet on each counter instead of
// one per warp.
constexpr int kReduceBlocks = 1024;

struct MaxOp {
  template <typename T>
  __device__ __forceinline__ T operator()(const T& a, const T& b) const {
    return a > b ? a : b;
  }
};

inline unsigned rblocks(int64_t n) {
  const unsigned b = nblocks(n);
  return b < kReduceBlocks ? b : kReduceBlocks;
}

// key = |id| (0 for zero ids), val = local index.
__global__ void k_keys(const int64_t* __restrict__ ids, int64_t n, uint64_t* __restrict__ key,
                       int32_t* __restrict__ val, Counters* c) {
  using RU = cub::BlockReduce<unsigned long long, kT>;
  __shared__ typename RU::TempStorage tmp;
  unsigned long long m = 0, zeros = 0;
  int bad = 0;
  for (int64_t i = static_cast<int64_t>(blockIdx.x) * kT + threadIdx.x; i < n;
       i += static_cast<int64_t>(gridDim.x) * kT) {
    const int64_t id = ids[i];
    bad |= (id == INT64_MIN);
    const uint64_t a = static_cast<uint64_t>(id < 0 ? -id : id);
    zeros += (id == 0);
    m = a > m ? a : m;
    key[i] = a;
    val[i] = static_cast<int32_t>(i);
  }
  const unsigned long long bm = RU(tmp).Reduce(m, MaxOp());
  __syncthreads();
  const unsigned long long bz = RU(tmp).Sum(zeros);
  const int bbad = __syncthreads_or(bad);
  if (threadIdx.x == 0) {
    if (bm) atomicMax(&c->maxkey, bm);
    if (bz) atomicAdd(&c->zeros, bz);
    if (bbad) atomicOr(&c->flags[0], 1);
  }
}

// Over the sorted nonzero pairs: head of a group, and whether the member is
// positive (Unsigned: all; Signed: id > 0; unique: the group's first member).
__global__ void k_heads(const uint64_t* __restrict__ key, const int32_t* __restrict__ val,
                        const int64_t* __restrict__ ids, int64_t nnz, int kind, int unique,
                        int32_t* __restrict__ head, int32_t* __restrict__ pos) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * kT + threadIdx.x;
  if (i >= nnz) return;
  const int h = (i == 0 || key[i] != key[i - 1]) ? 1 : 0;
  head[i] = h;
  int p;
  if (unique) p = h;
  else if (kind == OGS_UNSIGNED) p = 1;
  else p = ids[val[i]] > 0 ? 1 : 0;
  pos[i] = p;
}

// At each head: the group's start in sorted order and its first member.
__global__ void k_group_heads(const int32_t* __restrict__ head, const int32_t* __restrict__ gincl,
                              const int32_t* __restrict__ val, int64_t nnz, int32_t* __restrict__ gstart,
                              int32_t* __restrict__ gfirst) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * kT + threadIdx.x;
  if (i >= nnz || !head[i]) return;
  const int32_t g = gincl[i] - 1;
  gstart[g] = static_cast<int32_t>(i);
  gfirst[g] = val[i];
}

// Per group: size, positive count, and the first-appearance mark.
// gstart[ngroups] == nnz and pos_ex[nnz] == all positive members.
__global__ void k_group_stats(const int32_t* __restrict__ gstart, const int32_t* __restrict__ pos_ex,
                              const int32_t* __restrict__ gfirst, int64_t ngroups, int32_t* __restrict__ gsize,
                              int32_t* __restrict__ gpos, uint64_t* __restrict__ mark, Counters* c) {
  using RI = cub::BlockReduce<int, kT>;
  __shared__ typename RI::TempStorage tmp;
  int maxsize = 0, undefined = 0;
  for (int64_t g = static_cast<int64_t>(blockIdx.x) * kT + threadIdx.x; g < ngroups;
       g += static_cast<int64_t>(gridDim.x) * kT) {
    const int32_t s = gstart[g], e = gstart[g + 1];
    const int32_t size = e - s;
    const int32_t pc = pos_ex[e] - pos_ex[s];
    gsize[g] = size;
    gpos[g] = pc;
    undefined |= (pc != 1);
    maxsize = size > maxsize ? size : maxsize;
    mark[gfirst[g]] = pc > 0 ? uint64_t(1) : (uint64_t(1) << 32);
  }
  const int bm = RI(tmp).Reduce(maxsize, MaxOp());
  const int bu = __syncthreads_or(undefined);
  if (threadIdx.x == 0) {
    if (bm) atomicMax(&c->flags[2], bm);
    if (bu) atomicOr(&c->flags[1], 1);
  }
}

// Row of each group and the row degrees.  rank = exclusive scan of the
// marks: low word = positive groups before, high word = the others before.
__global__ void k_rows(const int32_t* __restrict__ gfirst, const int32_t* __restrict__ gsize,
                       const int32_t* __restrict__ gpos, const uint64_t* __restrict__ rank, int64_t ngroups,
                       int64_t nlocalP, int32_t* __restrict__ grow, int32_t* __restrict__ degT,
                       int32_t* __restrict__ degN) {
  const int64_t g = static_cast<int64_t>(blockIdx.x) * kT + threadIdx.x;
  if (g >= ngroups) return;
  const uint64_t rk = rank[gfirst[g]];
  const int32_t r = gpos[g] > 0 ? static_cast<int32_t>(rk & 0xffffffffu)
                                : static_cast<int32_t>(nlocalP + static_cast<int64_t>(rk >> 32));
  grow[g] = r;
  degT[r] = gsize[g];
  degN[r] = gpos[g];
}

// Each member to its slot: T map always, N map for positive members of a
// Signed handle.  Members of a group are in ascending local index already.
__global__ void k_fill(const int32_t* __restrict__ gincl, const int32_t* __restrict__ gstart,
                       const int32_t* __restrict__ grow, const int32_t* __restrict__ val,
                       const int32_t* __restrict__ pos, const int32_t* __restrict__ pos_ex,
                       const int32_t* __restrict__ rsT, const int32_t* __restrict__ rsN, int64_t nnz, int signed_maps,
                       int32_t* __restrict__ ciT, int32_t* __restrict__ ciN) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * kT + threadIdx.x;
  if (i >= nnz) return;
  const int32_t g = gincl[i] - 1;
  const int32_t s = gstart[g];
  const int32_t r = grow[g];
  ciT[rsT[r] + (static_cast<int32_t>(i) - s)] = val[i];
  if (signed_maps && pos[i]) ciN[rsN[r] + (pos_ex[i] - pos_ex[s])] = val[i];
}

// unique: the first member of each group keeps +|id|, the rest get -|id|.
__global__ void k_unique_ids(int64_t* __restrict__ ids, const int32_t* __restrict__ val,
                             const int32_t* __restrict__ head, int64_t nnz) {
  const int64_t i = static_cast<int64_t>(blockIdx.x) * kT + threadIdx.x;
  if (i >= nnz) return;
  const int32_t n = val[i];
  const int64_t id = ids[n];
  const int64_t a = id < 0 ? -id : id;
  ids[n] = head[i] ? a : -a;
}

// ---- layout kernels (the device form of build_layout, ogs_setup.cpp) ----

// Bucket of every row (1..kDmax: exact degree, 0: general) and row counts
// per bucket, all rows and rows below NlocalP (block histogram, one atomic
// per bucket and block).
__global__ void k_row_bucket(const int32_t* __restrict__ rsT, int64_t R, int64_t nlocalP, uint32_t* __restrict__ key,
                             int32_t* __restrict__ val, unsigned long long* counts) {
  __shared__ unsigned int hist[2 * (kDmax + 1)];
  if (threadIdx.x < 2 * (kDmax + 1)) hist[threadIdx.x] = 0;
  __syncthreads();
  for (int64_t r = static_cast<int64_t>(blockIdx.x) * kT + threadIdx.x; r < R;
       r += static_cast<int64_t>(gridDim.x) * kT) {
    const int d = rsT[r + 1] - rsT[r];
    const int b = (d >= 1 && d <= kDmax) ? d : 0;
    key[r] = static_cast<uint32_t>(b);
    val[r] = static_cast<int32_t>(r);
    atomicAdd(&hist[b], 1u);
    if (r < nlocalP) atomicAdd(&hist[kDmax + 1 + b], 1u);
  }
  __syncthreads();
  if (threadIdx.x < 2 * (kDmax + 1) && hist[threadIdx.x])
    atomicAdd(&counts[threadIdx.x], static_cast<unsigned long long>(hist[threadIdx.x]));
}

// Where the exact-degree buckets live in the arena.
struct BucketPtrs {
  int32_t* cols[kDmax + 1];
  int32_t* rows[kDmax + 1];
  uint8_t* nmask[kDmax + 1];
  int64_t stride[kDmax + 1];
  int64_t off[kDmax + 2];  // start of bucket d in the row order sorted by bucket (off[kDmax+1] = R)
};

// Rows of the exact-degree buckets, in bucket order: row ids, column ids in
// structure-of-arrays form, and for Signed maps the N-member mask.
__global__ void k_fill_exact(BucketPtrs B, const int32_t* __restrict__ srt, const int32_t* __restrict__ rsT,
                             const int32_t* __restrict__ ciT, const int32_t* __restrict__ rsN,
                             const int32_t* __restrict__ ciN, int sgn) {
  const int64_t lo = B.off[1], hi = B.off[kDmax + 1];
  for (int64_t pos = lo + static_cast<int64_t>(blockIdx.x) * kT + threadIdx.x; pos < hi;
       pos += static_cast<int64_t>(gridDim.x) * kT) {
    int d = 1;
#pragma unroll
    for (int e = 2; e <= kDmax; ++e)
      if (pos >= B.off[e]) d = e;
    const int64_t i = pos - B.off[d];
    const int32_t r = srt[pos];
    B.rows[d][i] = r;
    const int32_t s = rsT[r];
    int32_t q = sgn ? rsN[r] : 0;
    const int32_t qe = sgn ? rsN[r + 1] : 0;
    uint32_t mask = 0;
    for (int j = 0; j < d; ++j) {
      const int32_t c = ciT[s + j];
      B.cols[d][j * B.stride[d] + i] = c;
      // N members are a subsequence of the T members, both ascending
      if (sgn && q < qe && ciN[q] == c) { mask |= 1u << j; q++; }
    }
    if (sgn) B.nmask[d][i] = static_cast<uint8_t>(mask);
  }
}

// Degrees of the general rows (sorted first, bucket 0), for the row-start scans.
__global__ void k_general_deg(const int32_t* __restrict__ srt, int64_t ng, const int32_t* __restrict__ rs,
                              int32_t* __restrict__ deg) {
  const int64_t j = static_cast<int64_t>(blockIdx.x) * kT + threadIdx.x;
  if (j < ng) deg[j] = rs[srt[j] + 1] - rs[srt[j]];
  else if (j == ng) deg[j] = 0;
}

__global__ void k_fill_general(const int32_t* __restrict__ srt, int64_t ng, const int32_t* __restrict__ rs,
                               const int32_t* __restrict__ ci, const int32_t* __restrict__ gstarts,
                               int32_t* __restrict__ grows, int32_t* __restrict__ gcols) {
  const int64_t j = static_cast<int64_t>(blockIdx.x) * kT + threadIdx.x;
  if (j >= ng) return;
  const int32_t r = srt[j];
  if (grows) grows[j] = r;
  const int32_t s = rs[r], d = rs[r + 1] - s, o = gstarts[j];
  for (int32_t q = 0; q < d; ++q) gcols[o + q] = ci[s + q];
}

__global__ void k_gather_i32(const int32_t* __restrict__ src, const int64_t* __restrict__ pos, int64_t n,
                             int32_t* __restrict__ out) {
  const int64_t j = static_cast<int64_t>(blockIdx.x) * kT + threadIdx.x;
  if (j < n) out[j] = src[pos[j]];
}

// Lowest and highest node of every warp tile (one warp per tile) and of every
// general tile.
__global__ void k_tile_bounds(const Tile* __restrict__ wt, int64_t nw, BucketPtrs B, const Tile* __restrict__ gt,
                              int64_t ng, const int32_t* __restrict__ gstarts, const int32_t* __restrict__ gcols,
                              int64_t* __restrict__ lo, int64_t* __restrict__ hi) {
  const int64_t t = (static_cast<int64_t>(blockIdx.x) * kT + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (t >= nw + ng) return;
  int64_t a = INT64_MAX, z = -1;
  if (t < nw) {
    const Tile w = wt[t];
    const int d = w.bucket;
    for (int e = lane; e < d * w.count; e += 32) {
      const int j = e / w.count, r = e - j * w.count;
      const int64_t c = B.cols[d][j * B.stride[d] + w.begin + r];
      a = c < a ? c : a;
      z = c > z ? c : z;
    }
  } else {
    const Tile w = gt[t - nw];
    for (int32_t q = gstarts[w.begin] + lane; q < gstarts[w.begin + w.count]; q += 32) {
      const int64_t c = gcols[q];
      a = c < a ? c : a;
      z = c > z ? c : z;
    }
  }
  for (int o = 16; o > 0; o >>= 1) {
    const int64_t a2 = __shfl_down_sync(0xffffffffu, a, o), z2 = __shfl_down_sync(0xffffffffu, z, o);
    a = a2 < a ? a2 : a;
    z = z2 > z ? z2 : z;
  }
  if (lane == 0) {
    lo[t] = a;
    hi[t] = z;
  }
}

// Signed maps: each lane's N-member bits of its warp tile (bit j*d+q: member
// q of the lane's row j).
__global__ void k_wemask(const Tile* __restrict__ wt, int64_t nw, BucketPtrs B, uint8_t* __restrict__ wemask) {
  const int64_t x = static_cast<int64_t>(blockIdx.x) * kT + threadIdx.x;
  if (x >= nw * 32) return;
  const int64_t t = x >> 5;
  const int lane = static_cast<int>(x & 31);
  const Tile w = wt[t];
  const int d = w.bucket;
  uint32_t bits = 0;
  for (int j = 0; j < warp_rows_per_lane(d); ++j) {
    const int r = j * 32 + lane;
    if (r >= w.count) continue;
    const uint32_t mk = B.nmask[d][w.begin + r];
    for (int q = 0; q < d; ++q) bits |= ((mk >> q) & 1u) << (j * d + q);
  }
  wemask[x] = static_cast<uint8_t>(bits);
}

// Device scratch of one setup call, freed on every exit path.
struct Scratch {
  std::vector<void*> bufs;
  ~Scratch() {
    for (void* p : bufs) dev_free(p);
  }
  template <typename T>
  cudaError_t get(T** p, int64_t count) {
    void* q = nullptr;
    const size_t bytes = static_cast<size_t>(count > 0 ? count : 1) * sizeof(T);
    const cudaError_t e = dev_malloc(&q, bytes);
    if (e == cudaSuccess) bufs.push_back(q);
    *p = static_cast<T*>(q);
    return e;
  }
};

template <typename T>
cudaError_t exclusive_sum(Scratch& sc, const T* in, T* out, int64_t n, cudaStream_t st) {
  size_t bytes = 0;
  cudaError_t e = cub::DeviceScan::ExclusiveSum(nullptr, bytes, in, out, n, st);
  char* tmp = nullptr;
  if (e == cudaSuccess) e = sc.get(&tmp, static_cast<int64_t>(bytes));
  if (e == cudaSuccess) e = cub::DeviceScan::ExclusiveSum(tmp, bytes, in, out, n, st);
  return e;
}

template <typename T>
cudaError_t inclusive_sum(Scratch& sc, const T* in, T* out, int64_t n, cudaStream_t st) {
  size_t bytes = 0;
  cudaError_t e = cub::DeviceScan::InclusiveSum(nullptr, bytes, in, out, n, st);
  char* tmp = nullptr;
  if (e == cudaSuccess) e = sc.get(&tmp, static_cast<int64_t>(bytes));
  if (e == cudaSuccess) e = cub::DeviceScan::InclusiveSum(tmp, bytes, in, out, n, st);
  return e;
}

}  // namespace

ogs_status build_device_layout(ogs_handle_s* h, const int32_t* rsT, const int32_t* ciT, const int32_t* rsN,
                               const int32_t* ciN, void* stream) {
  TraceRange trace("ogs_setup: layout on the GPU");
  const cudaStream_t st = static_cast<cudaStream_t>(stream);
  HostLayout& L = h->lay;
  L = HostLayout{};
  const bool sgn = (h->kind == OGS_SIGNED);
  const int64_t R = h->NlocalT;
  if (!sgn) {
    rsN = rsT;
    ciN = ciT;
  }
  Scratch sc;
  auto fail = [&](cudaError_t e, const char* what) {
    cudaGetLastError();
    return set_error(e == cudaErrorMemoryAllocation ? OGS_ENOMEM : OGS_EDEVICE,
                     std::string("ogs_setup (device layout): ") + what + ": " + cudaGetErrorString(e));
  };
  // rows by bucket: a stable sort on the bucket number keeps them ascending
  uint32_t *key = nullptr, *key2 = nullptr;
  int32_t *val = nullptr, *srt = nullptr;
  unsigned long long* d_cnt = nullptr;
  cudaError_t e = sc.get(&key, R);
  if (!e) e = sc.get(&key2, R);
  if (!e) e = sc.get(&val, R);
  if (!e) e = sc.get(&srt, R);
  if (!e) e = sc.get(&d_cnt, 2 * (kDmax + 1));
  if (!e) e = cudaMemsetAsync(d_cnt, 0, 2 * (kDmax + 1) * sizeof(unsigned long long), st);
  if (e) return fail(e, "allocation");
  k_row_bucket<<<rblocks(R), kT, 0, st>>>(rsT, R, h->NlocalP, key, val, d_cnt);
  {
    size_t bytes = 0;
    e = cub::DeviceRadixSort::SortPairs(nullptr, bytes, key, key2, val, srt, R, 0, 4, st);
    char* tmp = nullptr;
    if (!e) e = sc.get(&tmp, static_cast<int64_t>(bytes));
    if (!e) e = cub::DeviceRadixSort::SortPairs(tmp, bytes, key, key2, val, srt, R, 0, 4, st);
    if (e) return fail(e, "sort");
  }
  unsigned long long cnt[2 * (kDmax + 1)];
  e = cudaMemcpyAsync(cnt, d_cnt, sizeof(cnt), cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaStreamSynchronize(st);
  if (e) return fail(e, "counts");
  const int64_t ng = static_cast<int64_t>(cnt[0]);
  int64_t stride[kDmax + 1] = {0}, off[kDmax + 2] = {0};
  off[1] = ng;
  for (int d = 1; d <= kDmax; ++d) {
    L.n[d] = static_cast<int32_t>(cnt[d]);
    L.nP[d] = static_cast<int32_t>(cnt[kDmax + 1 + d]);
    stride[d] = (static_cast<int64_t>(cnt[d]) + 3) / 4 * 4;
    off[d + 1] = off[d] + static_cast<int64_t>(cnt[d]);
  }
  L.g_nP = static_cast<int32_t>(cnt[kDmax + 1]);
  L.g_n = ng;
  // general row starts (T and N) by scans over the general rows' degrees
  int32_t *gdegT = nullptr, *gdegN = nullptr, *gsT = nullptr, *gsN = nullptr;
  e = sc.get(&gdegT, ng + 1);
  if (!e) e = sc.get(&gsT, ng + 1);
  if (!e && sgn) e = sc.get(&gdegN, ng + 1);
  if (!e && sgn) e = sc.get(&gsN, ng + 1);
  if (e) return fail(e, "allocation");
  k_general_deg<<<nblocks(ng + 1), kT, 0, st>>>(srt, ng, rsT, gdegT);
  if ((e = exclusive_sum(sc, gdegT, gsT, ng + 1, st))) return fail(e, "scan");
  if (sgn) {
    k_general_deg<<<nblocks(ng + 1), kT, 0, st>>>(srt, ng, rsN, gdegN);
    if ((e = exclusive_sum(sc, gdegN, gsN, ng + 1, st))) return fail(e, "scan");
  }
  std::vector<int32_t> g_startsT(static_cast<size_t>(ng) + 1);
  int32_t gnnzN = 0;
  e = cudaMemcpyAsync(g_startsT.data(), gsT, (ng + 1) * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (!e && sgn) e = cudaMemcpyAsync(&gnnzN, gsN + ng, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaStreamSynchronize(st);
  if (e) return fail(e, "general starts");
  const int64_t gnnzT = g_startsT[static_cast<size_t>(ng)];
  if (!sgn) gnnzN = static_cast<int32_t>(gnnzT);
  L.g_nnzT = gnnzT;
  // general tiles: greedy packing, as build_layout does
  {
    int32_t i = 0;
    const int32_t n = static_cast<int32_t>(ng);
    while (i < n) {
      int32_t j = i, nnz = 0;
      while (j < n && j - i < kGeneralRowsPerTile) {
        const int32_t dj = g_startsT[j + 1] - g_startsT[j];
        if (j > i && nnz + dj > kTileNnz) break;
        nnz += dj;
        j++;
      }
      L.gtiles.push_back(Tile{0, i, j - i, 0});
      i = j;
    }
  }
  // first rows of every tile, gathered from the sorted rows
  std::vector<int64_t> pos;
  std::vector<Tile> ctiles, wtiles;
  for (int d = 1; d <= kDmax; ++d) {
    const int32_t n = L.n[d], step = rows_per_tile(d);
    for (int32_t i = 0; i < n; i += step) {
      ctiles.push_back(Tile{d, i, std::min(step, n - i), 0});
      pos.push_back(off[d] + i);
    }
  }
  for (int d = 1; d <= kDmax; ++d) {
    const int32_t n = L.n[d], step = warp_rows_per_tile(d);
    for (int32_t i = 0; i < n; i += step) {
      wtiles.push_back(Tile{d, i, std::min(step, n - i), 0});
      pos.push_back(off[d] + i);
    }
  }
  for (const Tile& g : L.gtiles) pos.push_back(g.begin);  // bucket 0 starts the sorted order
  {
    int64_t* d_pos = nullptr;
    int32_t* d_first = nullptr;
    const int64_t np = static_cast<int64_t>(pos.size());
    std::vector<int32_t> first(pos.size());
    e = sc.get(&d_pos, np);
    if (!e) e = sc.get(&d_first, np);
    if (!e && np) e = cudaMemcpyAsync(d_pos, pos.data(), np * sizeof(int64_t), cudaMemcpyHostToDevice, st);
    if (e) return fail(e, "tile rows");
    if (np) k_gather_i32<<<nblocks(np), kT, 0, st>>>(srt, d_pos, np, d_first);
    if (!e && np) e = cudaMemcpyAsync(first.data(), d_first, np * sizeof(int32_t), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    if (e) return fail(e, "tile rows");
    size_t x = 0;
    for (Tile& t : ctiles) t.first_row = first[x++];
    for (Tile& t : wtiles) t.first_row = first[x++];
    for (Tile& t : L.gtiles) t.first_row = first[x++];
  }
  auto by_row = [](const Tile& a, const Tile& b) { return a.first_row < b.first_row; };
  std::stable_sort(wtiles.begin(), wtiles.end(), by_row);
  L.wtiles = wtiles;
  L.tiles = ctiles;
  L.tiles.insert(L.tiles.end(), L.gtiles.begin(), L.gtiles.end());
  std::stable_sort(L.tiles.begin(), L.tiles.end(), by_row);
  const int64_t nw = static_cast<int64_t>(L.wtiles.size());

  // the arena: the pieces and sizes of upload_layout (ogs_setup.cpp)
  size_t total = 0;
  auto add = [&](size_t bytes) {
    const size_t o = total;
    total = (total + std::max<size_t>(bytes, 1) + 255) / 256 * 256;
    return o;
  };
  size_t o_cols[kDmax + 1], o_rows[kDmax + 1], o_mask[kDmax + 1];
  for (int d = 1; d <= kDmax; ++d) {
    o_cols[d] = add(static_cast<size_t>(stride[d]) * d * 4);
    o_rows[d] = add(static_cast<size_t>(stride[d]) * 4);
    o_mask[d] = sgn ? add(static_cast<size_t>((L.n[d] + 15) / 16 * 16)) : 0;
  }
  const size_t o_grows = add(static_cast<size_t>(ng) * 4);
  const size_t o_gsT = add(static_cast<size_t>(ng + 1) * 4);
  const size_t o_gcT = add(static_cast<size_t>(gnnzT) * 4);
  const size_t o_gsN = sgn ? add(static_cast<size_t>(ng + 1) * 4) : o_gsT;
  const size_t o_gcN = sgn ? add(static_cast<size_t>(gnnzN) * 4) : o_gcT;
  const size_t o_tiles = add(L.tiles.size() * sizeof(Tile));
  const size_t o_gtiles = add(L.gtiles.size() * sizeof(Tile));
  const size_t o_wtiles = add(L.wtiles.size() * sizeof(Tile));
  const size_t o_wemask = add(sgn ? L.wtiles.size() * 32 : 0);
  const size_t o_wrecs = add(L.wtiles.size() * sizeof(WarpRec));
  const size_t o_err = add(sizeof(uint32_t));  // ids out of range (checked builds); zeroed with the arena
  int dev = 0;
  if ((e = cudaGetDevice(&dev))) return fail(e, "device");
  char* base = nullptr;
  if ((e = dev_malloc(reinterpret_cast<void**>(&base), total))) return fail(e, "arena");
  auto release = [&](cudaError_t err, const char* what) {
    dev_free(base);
    return fail(err, what);
  };
  if ((e = cudaMemsetAsync(base, 0, total, st))) return release(e, "arena");
  BucketPtrs B{};
  for (int d = 1; d <= kDmax; ++d) {
    B.cols[d] = reinterpret_cast<int32_t*>(base + o_cols[d]);
    B.rows[d] = reinterpret_cast<int32_t*>(base + o_rows[d]);
    B.nmask[d] = sgn ? reinterpret_cast<uint8_t*>(base + o_mask[d]) : nullptr;
    B.stride[d] = stride[d];
  }
  for (int d = 0; d <= kDmax + 1; ++d) B.off[d] = off[d];
  if (R > ng) k_fill_exact<<<rblocks(R - ng), kT, 0, st>>>(B, srt, rsT, ciT, rsN, ciN, sgn ? 1 : 0);
  int32_t* g_rows = reinterpret_cast<int32_t*>(base + o_grows);
  int32_t* g_sT = reinterpret_cast<int32_t*>(base + o_gsT);
  int32_t* g_cT = reinterpret_cast<int32_t*>(base + o_gcT);
  int32_t* g_sN = reinterpret_cast<int32_t*>(base + o_gsN);
  int32_t* g_cN = reinterpret_cast<int32_t*>(base + o_gcN);
  e = cudaMemcpyAsync(g_sT, gsT, (ng + 1) * sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
  if (!e && sgn) e = cudaMemcpyAsync(g_sN, gsN, (ng + 1) * sizeof(int32_t), cudaMemcpyDeviceToDevice, st);
  if (e) return release(e, "general starts");
  if (ng) {
    k_fill_general<<<nblocks(ng), kT, 0, st>>>(srt, ng, rsT, ciT, g_sT, g_rows, g_cT);
    if (sgn) k_fill_general<<<nblocks(ng), kT, 0, st>>>(srt, ng, rsN, ciN, g_sN, nullptr, g_cN);
  }
  // tiles, warp records; tile bounds and (Signed) lane masks on the device
  std::vector<WarpRec> wrecs(L.wtiles.size());
  for (size_t t = 0; t < L.wtiles.size(); ++t) {
    const Tile& w = L.wtiles[t];
    WarpRec& r = wrecs[t];
    r.cols = reinterpret_cast<const int32_t*>(base + o_cols[w.bucket]);
    r.rows = reinterpret_cast<const int32_t*>(base + o_rows[w.bucket]);
    r.begin = w.begin;
    r.bucket_count = (w.bucket << 16) | w.count;
    r.stride = static_cast<int32_t>(stride[w.bucket]);
    r.nP = L.nP[w.bucket];
  }
  const Tile* d_wt = reinterpret_cast<const Tile*>(base + o_wtiles);
  const Tile* d_gt = reinterpret_cast<const Tile*>(base + o_gtiles);
  e = cudaMemcpyAsync(base + o_tiles, L.tiles.data(), L.tiles.size() * sizeof(Tile), cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(base + o_gtiles, L.gtiles.data(), L.gtiles.size() * sizeof(Tile), cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(base + o_wtiles, L.wtiles.data(), L.wtiles.size() * sizeof(Tile), cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(base + o_wrecs, wrecs.data(), wrecs.size() * sizeof(WarpRec), cudaMemcpyHostToDevice, st);
  if (e) return release(e, "tiles");
  const int64_t ngt = static_cast<int64_t>(L.gtiles.size());
  int64_t *d_lo = nullptr, *d_hi = nullptr;
  e = sc.get(&d_lo, nw + ngt);
  if (!e) e = sc.get(&d_hi, nw + ngt);
  if (e) return release(e, "allocation");
  if (nw + ngt)
    k_tile_bounds<<<nblocks((nw + ngt) * 32), kT, 0, st>>>(d_wt, nw, B, d_gt, ngt, g_sT, g_cT, d_lo, d_hi);
  if (sgn && nw) k_wemask<<<nblocks(nw * 32), kT, 0, st>>>(d_wt, nw, B, reinterpret_cast<uint8_t*>(base + o_wemask));
  std::vector<int64_t> lo(static_cast<size_t>(nw + ngt)), hi(static_cast<size_t>(nw + ngt));
  if (nw + ngt) {
    e = cudaMemcpyAsync(lo.data(), d_lo, (nw + ngt) * sizeof(int64_t), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaMemcpyAsync(hi.data(), d_hi, (nw + ngt) * sizeof(int64_t), cudaMemcpyDeviceToHost, st);
  }
  if (!e) e = cudaGetLastError();
  if (!e) e = cudaStreamSynchronize(st);
  if (e) return release(e, "tile bounds");
  L.wlo.assign(lo.begin(), lo.begin() + nw);
  L.whi.assign(hi.begin(), hi.begin() + nw);
  L.glo.assign(lo.begin() + nw, lo.end());
  L.ghi.assign(hi.begin() + nw, hi.end());
  build_phases(h, OGS_HOST_PHASES);

  h->device = dev;
  h->arena = base;
  h->arena_bytes = total;
  DevMaps& m = h->dmaps;
  m = DevMaps{};
  for (int d = 1; d <= kDmax; ++d) {
    m.b[d].cols = B.cols[d];
    m.b[d].rows = B.rows[d];
    m.b[d].nmask = B.nmask[d];
    m.b[d].n = L.n[d];
    m.b[d].nP = L.nP[d];
    m.b[d].stride = static_cast<int32_t>(stride[d]);
  }
  m.g.rows = g_rows;
  m.g.startsT = g_sT;
  m.g.colsT = g_cT;
  m.g.startsN = g_sN;
  m.g.colsN = g_cN;
  m.g.n = static_cast<int32_t>(ng);
  m.g.nP = L.g_nP;
  m.tiles = reinterpret_cast<const Tile*>(base + o_tiles);
  m.ntiles = static_cast<int32_t>(L.tiles.size());
  m.gtiles = d_gt;
  m.ngtiles = static_cast<int32_t>(ngt);
  m.wtiles = d_wt;
  m.nwtiles = static_cast<int32_t>(nw);
  m.wemask = reinterpret_cast<const uint8_t*>(base + o_wemask);
  m.wrecs = reinterpret_cast<const WarpRec*>(base + o_wrecs);
  m.signed_maps = sgn ? 1 : 0;
  set_id_bounds(h, m, reinterpret_cast<unsigned int*>(base + o_err));
  return OGS_OK;
}

ogs_status build_device_maps(ogs_handle_s* h, int64_t N, int64_t* ids, int kind, int unique, bool layout) {
  TraceRange trace("ogs_setup: maps on the GPU");
  if (kind == OGS_HALO)
    return set_error(OGS_EINVAL, "ogs_setup: Halo handles are not part of the single-rank path");
  if (kind != OGS_UNSIGNED && kind != OGS_SIGNED) return set_error(OGS_EINVAL, "ogs_setup: unknown kind");
  if (kind == OGS_UNSIGNED && unique)  // ogsSetup.cpp:98-100
    return set_error(OGS_EINVAL, "Invalid ogs setup requested (Unsigned with unique)");
  if (N < 0) return set_error(OGS_EINVAL, "ogs_setup: N < 0");
  if (N > std::numeric_limits<int32_t>::max())
    return set_error(OGS_ERANGE, "ogs_setup: N exceeds 32-bit device indices");
  if (N > 0 && ids == nullptr) return set_error(OGS_EINVAL, "ogs_setup: ids is NULL");
  h->N = N;
  h->kind = kind;
  h->unique = unique ? 1 : 0;
  const bool sgn = (kind == OGS_SIGNED);
  auto empty_maps = [&]() {
    h->gather_defined = 1;
    h->NlocalP = h->NlocalT = h->Ngather = h->NgatherGlobal = 0;
    h->nnzT = h->nnzN = 0;
    h->max_degree = 0;
    h->rowStartsT.assign(1, 0);
    h->colIdsT.clear();
    if (sgn) h->rowStartsN.assign(1, 0);
    h->colIdsN.clear();
    h->covers_all = (N == 0);
    return OGS_OK;
  };
  if (N == 0) return empty_maps();

  const cudaStream_t st = nullptr;
  Scratch sc;
  auto fail = [&](cudaError_t e, const char* what) {
    cudaGetLastError();
    return set_error(e == cudaErrorMemoryAllocation ? OGS_ENOMEM : OGS_EDEVICE,
                     std::string("ogs_setup (device maps): ") + what + ": " + cudaGetErrorString(e));
  };

  // 1. keys and a stable sort by |id|
  int64_t* d_ids = nullptr;
  uint64_t *key = nullptr, *key2 = nullptr;
  int32_t *val = nullptr, *val2 = nullptr;
  Counters* d_c = nullptr;
  cudaError_t e = sc.get(&d_ids, N);
  if (!e) e = sc.get(&key, N);
  if (!e) e = sc.get(&key2, N);
  if (!e) e = sc.get(&val, N);
  if (!e) e = sc.get(&val2, N);
  if (!e) e = sc.get(&d_c, 1);
  if (e) return fail(e, "allocation");
  e = cudaMemcpyAsync(d_ids, ids, static_cast<size_t>(N) * sizeof(int64_t), cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemsetAsync(d_c, 0, sizeof(Counters), st);
  if (e) return fail(e, "copy in");
  k_keys<<<rblocks(N), kT, 0, st>>>(d_ids, N, key, val, d_c);
  Counters c{};
  e = cudaMemcpyAsync(&c, d_c, sizeof(Counters), cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaStreamSynchronize(st);
  if (e) return fail(e, "keys");
  if (c.flags[0]) return set_error(OGS_ERANGE, "ogs_setup: id -2^63 has no absolute value");
  const int64_t zeros = static_cast<int64_t>(c.zeros);
  const int64_t nnz = N - zeros;
  h->covers_all = (zeros == 0);
  if (nnz == 0) return empty_maps();
  int end_bit = 1;
  while (end_bit < 64 && (c.maxkey >> end_bit) != 0) end_bit++;
  {
    size_t bytes = 0;
    e = cub::DeviceRadixSort::SortPairs(nullptr, bytes, key, key2, val, val2, N, 0, end_bit, st);
    char* tmp = nullptr;
    if (!e) e = sc.get(&tmp, static_cast<int64_t>(bytes));
    if (!e) e = cub::DeviceRadixSort::SortPairs(tmp, bytes, key, key2, val, val2, N, 0, end_bit, st);
    if (e) return fail(e, "sort");
  }
  const uint64_t* skey = key2 + zeros;  // zero ids sort first
  const int32_t* sval = val2 + zeros;

  // 2. heads, group numbers, positive members before each member
  int32_t *head = nullptr, *gincl = nullptr, *pos = nullptr, *pos_ex = nullptr;
  e = sc.get(&head, nnz);
  if (!e) e = sc.get(&gincl, nnz);
  if (!e) e = sc.get(&pos, nnz + 1);
  if (!e) e = sc.get(&pos_ex, nnz + 1);
  if (e) return fail(e, "allocation");
  e = cudaMemsetAsync(pos + nnz, 0, sizeof(int32_t), st);
  if (e) return fail(e, "memset");
  k_heads<<<nblocks(nnz), kT, 0, st>>>(skey, sval, d_ids, nnz, kind, unique, head, pos);
  if ((e = inclusive_sum(sc, head, gincl, nnz, st))) return fail(e, "scan");
  if ((e = exclusive_sum(sc, pos, pos_ex, nnz + 1, st))) return fail(e, "scan");
  int32_t ngroups32 = 0;
  e = cudaMemcpyAsync(&ngroups32, gincl + nnz - 1, sizeof(int32_t), cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaStreamSynchronize(st);
  if (e) return fail(e, "groups");
  const int64_t ngroups = ngroups32;

  // 3. per-group figures and first-appearance ranks
  int32_t *gstart = nullptr, *gfirst = nullptr, *gsize = nullptr, *gpos = nullptr, *grow = nullptr;
  uint64_t *mark = nullptr, *rank = nullptr;
  e = sc.get(&gstart, ngroups + 1);
  if (!e) e = sc.get(&gfirst, ngroups);
  if (!e) e = sc.get(&gsize, ngroups);
  if (!e) e = sc.get(&gpos, ngroups);
  if (!e) e = sc.get(&grow, ngroups);
  if (!e) e = sc.get(&mark, N + 1);
  if (!e) e = sc.get(&rank, N + 1);
  if (e) return fail(e, "allocation");
  const int32_t nnz32 = static_cast<int32_t>(nnz);
  e = cudaMemcpyAsync(gstart + ngroups, &nnz32, sizeof(int32_t), cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemsetAsync(mark, 0, static_cast<size_t>(N + 1) * sizeof(uint64_t), st);
  if (e) return fail(e, "memset");
  k_group_heads<<<nblocks(nnz), kT, 0, st>>>(head, gincl, sval, nnz, gstart, gfirst);
  k_group_stats<<<rblocks(ngroups), kT, 0, st>>>(gstart, pos_ex, gfirst, ngroups, gsize, gpos, mark, d_c);
  if ((e = exclusive_sum(sc, mark, rank, N + 1, st))) return fail(e, "scan");
  uint64_t total = 0;
  e = cudaMemcpyAsync(&total, rank + N, sizeof(uint64_t), cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaMemcpyAsync(&c, d_c, sizeof(Counters), cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaStreamSynchronize(st);
  if (e) return fail(e, "ranks");
  const int64_t nlocalP = static_cast<int64_t>(total & 0xffffffffu);

  // 4. rows, row starts, members into place
  int32_t *degT = nullptr, *degN = nullptr, *rsT = nullptr, *rsN = nullptr, *ciT = nullptr, *ciN = nullptr;
  e = sc.get(&degT, ngroups + 1);
  if (!e) e = sc.get(&degN, ngroups + 1);
  if (!e) e = sc.get(&rsT, ngroups + 1);
  if (!e) e = sc.get(&rsN, ngroups + 1);
  if (!e) e = sc.get(&ciT, nnz);
  if (!e && sgn) e = sc.get(&ciN, nnz);
  if (e) return fail(e, "allocation");
  e = cudaMemsetAsync(degT + ngroups, 0, sizeof(int32_t), st);
  if (!e) e = cudaMemsetAsync(degN + ngroups, 0, sizeof(int32_t), st);
  if (e) return fail(e, "memset");
  k_rows<<<nblocks(ngroups), kT, 0, st>>>(gfirst, gsize, gpos, rank, ngroups, nlocalP, grow, degT, degN);
  if ((e = exclusive_sum(sc, degT, rsT, ngroups + 1, st))) return fail(e, "scan");
  if (sgn && (e = exclusive_sum(sc, degN, rsN, ngroups + 1, st))) return fail(e, "scan");
  k_fill<<<nblocks(nnz), kT, 0, st>>>(gincl, gstart, grow, sval, pos, pos_ex, rsT, rsN, nnz, sgn ? 1 : 0, ciT, ciN);
  if (unique) k_unique_ids<<<nblocks(nnz), kT, 0, st>>>(d_ids, sval, head, nnz);
  if ((e = cudaGetLastError())) return fail(e, "kernels");

  h->gather_defined = c.flags[1] ? 0 : 1;
  h->max_degree = c.flags[2];
  h->NlocalP = nlocalP;
  h->NlocalT = ngroups;
  h->Ngather = nlocalP;        // NlocalP + NhaloP with NhaloP = 0
  h->NgatherGlobal = nlocalP;  // single rank
  h->nnzT = nnz;
  // the kernels' layout, built from the maps while they are on the device
  if (layout) {
    ogs_status ls = build_device_layout(h, rsT, ciT, sgn ? rsN : nullptr, sgn ? ciN : nullptr, st);
    if (ls != OGS_OK) return ls;
  }
  // maps back to the host
  h->rowStartsT.resize(static_cast<size_t>(ngroups) + 1);
  h->colIdsT.resize(static_cast<size_t>(nnz));
  e = cudaMemcpyAsync(h->rowStartsT.data(), rsT, static_cast<size_t>(ngroups + 1) * 4, cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaMemcpyAsync(h->colIdsT.data(), ciT, static_cast<size_t>(nnz) * 4, cudaMemcpyDeviceToHost, st);
  if (sgn) {
    h->rowStartsN.resize(static_cast<size_t>(ngroups) + 1);
    if (!e)
      e = cudaMemcpyAsync(h->rowStartsN.data(), rsN, static_cast<size_t>(ngroups + 1) * 4, cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaStreamSynchronize(st);
    const int64_t nnzN = e ? 0 : h->rowStartsN[static_cast<size_t>(ngroups)];
    h->nnzN = nnzN;
    h->colIdsN.resize(static_cast<size_t>(nnzN));
    if (!e && nnzN)
      e = cudaMemcpyAsync(h->colIdsN.data(), ciN, static_cast<size_t>(nnzN) * 4, cudaMemcpyDeviceToHost, st);
  } else {
    h->nnzN = nnz;
    h->rowStartsN.clear();
    h->colIdsN.clear();
  }
  if (!e && unique)
    e = cudaMemcpyAsync(ids, d_ids, static_cast<size_t>(N) * sizeof(int64_t), cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaStreamSynchronize(st);
  if (e) return fail(e, "copy out");
  return OGS_OK;
}

}  // namespace ogsgb
