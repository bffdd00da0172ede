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
// The maps then go back to the host, where the degree buckets, tiles and the
// upload run as after a host setup, so both setups give identical handles.
//
// Every buffer here is scratch of the setup call and is freed before it
// returns.  Device memory needed: about 70 bytes per local node.
#include <cstdint>
#include <limits>
#include <string>
#include <vector>

#include <cub/cub.cuh>
#include <cuda_runtime.h>

#include "ogs_internal.hpp"

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

// Device scratch of one setup call, freed on every exit path.
struct Scratch {
  std::vector<void*> bufs;
  ~Scratch() {
    for (void* p : bufs) cudaFree(p);
  }
  template <typename T>
  cudaError_t get(T** p, int64_t count) {
    void* q = nullptr;
    const size_t bytes = static_cast<size_t>(count > 0 ? count : 1) * sizeof(T);
    const cudaError_t e = cudaMalloc(&q, bytes);
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

ogs_status build_device_maps(ogs_handle_s* h, int64_t N, int64_t* ids, int kind, int unique) {
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

  // maps back to the host
  h->gather_defined = c.flags[1] ? 0 : 1;
  h->max_degree = c.flags[2];
  h->NlocalP = nlocalP;
  h->NlocalT = ngroups;
  h->Ngather = nlocalP;        // NlocalP + NhaloP with NhaloP = 0
  h->NgatherGlobal = nlocalP;  // single rank
  h->nnzT = nnz;
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
