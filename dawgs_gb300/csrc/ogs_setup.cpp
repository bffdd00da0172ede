// ogs_setup.cpp -- host setup of one single-rank gather-scatter handle.
//
// Builds the same N and T CSR maps as the reference's ogsBase_t::Setup
// (libs/ogs/ogsSetup.cpp:69-190 -> 333-433 -> 569-776) at one rank, then
// re-lays them out for the GPU: rows bucketed by exact degree with
// structure-of-arrays column ids, plus a tile table ordered by row id.
//
// Ordering contract kept from the reference:
//  * zero ids do not take part (ogsSetup.cpp:103-121);
//  * Unsigned treats every id as positive (ogsSetup.cpp:114-115);
//  * rows are the distinct |id| groups numbered by first appearance in local
//    order, groups with a positive member first (rows [0,NlocalP)), the
//    others after (ogsSetup.cpp:406-433);
//  * each row lists its members in ascending local index (ogsSetup.cpp:637-663,
//    744-758), so a fold over a row runs in the reference's order.
// The reference sorts the nodes by |id| (a gnu-parallel sort); here one pass
// over the nodes with a hash table gives the groups already numbered by first
// appearance, which is the order the rows need.
#include <algorithm>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <limits>

#include <cuda_runtime.h>

#include "ogs_internal.hpp"

namespace ogsgb {
namespace {

inline uint64_t mix64(uint64_t z) {
  z ^= z >> 33;
  z *= 0xff51afd7ed558ccdULL;
  z ^= z >> 33;
  z *= 0xc4ceb9fe1a85ec53ULL;
  z ^= z >> 33;
  return z;
}

// Open-addressing map |id| -> group number; key 0 marks an empty slot (ids of
// 0 never enter the table).
class GroupTable {
 public:
  explicit GroupTable(int64_t n) {
    size_t cap = 16;
    while (cap < static_cast<size_t>(2 * n + 1)) cap <<= 1;
    keys_.assign(cap, 0);
    vals_.assign(cap, -1);
    mask_ = cap - 1;
  }
  // Returns the group of `key`, inserting it as group `next` if absent.
  int32_t find_or_insert(uint64_t key, int32_t next, bool* inserted) {
    size_t s = mix64(key) & mask_;
    while (true) {
      if (keys_[s] == key) { *inserted = false; return vals_[s]; }
      if (keys_[s] == 0) {
        keys_[s] = key;
        vals_[s] = next;
        *inserted = true;
        return next;
      }
      s = (s + 1) & mask_;
    }
  }
 private:
  std::vector<uint64_t> keys_;
  std::vector<int32_t> vals_;
  size_t mask_;
};

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

}  // namespace

ogs_status build_host_maps(ogs_handle_s* h, int64_t N, int64_t* ids, int kind, int unique) {
  if (kind == OGS_HALO)
    return set_error(OGS_EINVAL, "ogs_setup: Halo handles are not part of the single-rank path");
  if (kind != OGS_UNSIGNED && kind != OGS_SIGNED)
    return set_error(OGS_EINVAL, "ogs_setup: unknown kind");
  if (kind == OGS_UNSIGNED && unique)  // ogsSetup.cpp:98-100
    return set_error(OGS_EINVAL, "Invalid ogs setup requested (Unsigned with unique)");
  if (N < 0) return set_error(OGS_EINVAL, "ogs_setup: N < 0");
  if (N > std::numeric_limits<int32_t>::max())  // dlong = int (types.h:59-63)
    return set_error(OGS_ERANGE, "ogs_setup: N exceeds 32-bit device indices");
  if (N > 0 && ids == nullptr) return set_error(OGS_EINVAL, "ogs_setup: ids is NULL");

  h->N = N;
  h->kind = kind;
  h->unique = unique ? 1 : 0;

  std::vector<int32_t> group(static_cast<size_t>(N), -1);
  std::vector<uint8_t> positive(static_cast<size_t>(N), 0);
  std::vector<int32_t> deg, poscnt;
  GroupTable table(N);
  int32_t ngroups = 0;
  for (int64_t n = 0; n < N; ++n) {
    const int64_t id = ids[n];
    if (id == 0) continue;
    if (id == std::numeric_limits<int64_t>::min())
      return set_error(OGS_ERANGE, "ogs_setup: id -2^63 has no absolute value");
    const uint64_t a = static_cast<uint64_t>(id < 0 ? -id : id);
    bool fresh = false;
    const int32_t g = table.find_or_insert(a, ngroups, &fresh);
    if (fresh) {
      ngroups++;
      deg.push_back(0);
      poscnt.push_back(0);
    }
    group[n] = g;
    bool pos;
    if (unique) pos = fresh;  // first member in local order keeps its positive id
    else pos = (kind == OGS_UNSIGNED) || id > 0;
    positive[n] = pos;
    deg[g]++;
    poscnt[g] += pos;
  }

  // gather_defined: exactly one positive member per group (ogsSetup.cpp:276-282)
  int defined = 1;
  int64_t nlocalP = 0;
  for (int32_t g = 0; g < ngroups; ++g) {
    if (poscnt[g] != 1) defined = 0;
    nlocalP += poscnt[g] > 0;
  }
  h->gather_defined = defined;
  h->NlocalP = nlocalP;
  h->NlocalT = ngroups;
  h->Ngather = nlocalP;        // NlocalP + NhaloP with NhaloP = 0
  h->NgatherGlobal = nlocalP;  // single rank

  // rows: groups are numbered by first appearance already, so a row is the
  // group's rank among positive (or among non-positive) groups.
  std::vector<int32_t> row_of(ngroups);
  {
    int32_t cp = 0, cn = static_cast<int32_t>(nlocalP);
    for (int32_t g = 0; g < ngroups; ++g) row_of[g] = poscnt[g] > 0 ? cp++ : cn++;
  }

  if (unique) {  // ogsSetup.cpp:138-141
    for (int64_t n = 0; n < N; ++n) {
      if (ids[n] == 0) continue;
      const int64_t a = ids[n] < 0 ? -ids[n] : ids[n];
      ids[n] = positive[n] ? a : -a;
    }
  }

  const int64_t R = ngroups;
  h->rowStartsT.assign(R + 1, 0);
  int32_t maxd = 0;
  for (int32_t g = 0; g < ngroups; ++g) {
    h->rowStartsT[row_of[g] + 1] = deg[g];
    maxd = std::max(maxd, deg[g]);
  }
  h->max_degree = maxd;
  for (int64_t r = 0; r < R; ++r) h->rowStartsT[r + 1] += h->rowStartsT[r];
  h->nnzT = h->rowStartsT[R];
  h->colIdsT.resize(h->nnzT);
  {
    std::vector<int32_t> cursor(h->rowStartsT.begin(), h->rowStartsT.end() - 1);
    for (int64_t n = 0; n < N; ++n)
      if (group[n] >= 0) h->colIdsT[cursor[row_of[group[n]]]++] = static_cast<int32_t>(n);
  }
  if (kind == OGS_SIGNED) {
    h->rowStartsN.assign(R + 1, 0);
    for (int32_t g = 0; g < ngroups; ++g) h->rowStartsN[row_of[g] + 1] = poscnt[g];
    for (int64_t r = 0; r < R; ++r) h->rowStartsN[r + 1] += h->rowStartsN[r];
    h->nnzN = h->rowStartsN[R];
    h->colIdsN.resize(h->nnzN);
    std::vector<int32_t> cursor(h->rowStartsN.begin(), h->rowStartsN.end() - 1);
    for (int64_t n = 0; n < N; ++n)
      if (group[n] >= 0 && positive[n])
        h->colIdsN[cursor[row_of[group[n]]]++] = static_cast<int32_t>(n);
  } else {
    h->nnzN = h->nnzT;
  }
  h->covers_all = (h->nnzT == N);
  return OGS_OK;
}

void build_layout(ogs_handle_s* h) {
  HostLayout& L = h->lay;
  const bool sgn = (h->kind == OGS_SIGNED);
  const int64_t R = h->NlocalT;
  const std::vector<int32_t>& rsT = h->rowStartsT;
  const std::vector<int32_t>& ciT = h->colIdsT;
  const std::vector<int32_t>& rsN = sgn ? h->rowStartsN : h->rowStartsT;
  const std::vector<int32_t>& ciN = sgn ? h->colIdsN : h->colIdsT;

  int64_t cnt[kDmax + 1] = {0};
  int64_t gnnzT = 0, gnnzN = 0;
  for (int64_t r = 0; r < R; ++r) {
    const int d = rsT[r + 1] - rsT[r];
    if (d <= kDmax) cnt[d]++;
    else { cnt[0]++; gnnzT += d; gnnzN += rsN[r + 1] - rsN[r]; }
  }
  for (int d = 1; d <= kDmax; ++d) {
    L.cols[d].assign(static_cast<size_t>(cnt[d]) * d, 0);
    L.rows[d].assign(cnt[d], 0);
    L.nmask[d].assign(sgn ? cnt[d] : 0, 0);
    L.nP[d] = 0;
  }
  L.g_rows.clear(); L.g_startsT.assign(1, 0); L.g_colsT.clear();
  L.g_startsN.assign(1, 0); L.g_colsN.clear();
  L.g_rows.reserve(cnt[0]); L.g_colsT.reserve(gnnzT); L.g_colsN.reserve(gnnzN);
  L.g_nP = 0;

  int64_t fill[kDmax + 1] = {0};
  for (int64_t r = 0; r < R; ++r) {
    const int32_t s = rsT[r], d = rsT[r + 1] - s;
    const bool inP = r < h->NlocalP;
    if (d <= kDmax) {
      const int64_t i = fill[d]++;
      const int64_t n = cnt[d];
      L.rows[d][i] = static_cast<int32_t>(r);
      if (inP) L.nP[d]++;
      uint8_t mask = 0;
      int32_t q = rsN[r];
      for (int j = 0; j < d; ++j) {
        const int32_t c = ciT[s + j];
        L.cols[d][static_cast<size_t>(j) * n + i] = c;
        // N members are a subsequence of the T members, both ascending
        if (sgn && q < rsN[r + 1] && ciN[q] == c) { mask |= uint8_t(1u << j); q++; }
      }
      if (sgn) L.nmask[d][i] = mask;
    } else {
      L.g_rows.push_back(static_cast<int32_t>(r));
      if (inP) L.g_nP++;
      L.g_colsT.insert(L.g_colsT.end(), ciT.begin() + s, ciT.begin() + s + d);
      L.g_startsT.push_back(static_cast<int32_t>(L.g_colsT.size()));
      L.g_colsN.insert(L.g_colsN.end(), ciN.begin() + rsN[r], ciN.begin() + rsN[r + 1]);
      L.g_startsN.push_back(static_cast<int32_t>(L.g_colsN.size()));
    }
  }

  // Tiles: fixed row counts per exact-degree bucket, greedy packing of the
  // general bucket; then ordered by first row id.
  L.tiles.clear();
  for (int d = 1; d <= kDmax; ++d) {
    const int32_t n = static_cast<int32_t>(cnt[d]);
    const int32_t step = rows_per_tile(d);
    for (int32_t i = 0; i < n; i += step)
      L.tiles.push_back(Tile{d, i, std::min(step, n - i), L.rows[d][i]});
  }
  {
    const int32_t n = static_cast<int32_t>(L.g_rows.size());
    int32_t i = 0;
    while (i < n) {
      int32_t j = i, nnz = 0;
      while (j < n && j - i < kGeneralRowsPerTile) {
        const int32_t dj = L.g_startsT[j + 1] - L.g_startsT[j];
        if (j > i && nnz + dj > kTileNnz) break;
        nnz += dj;
        j++;
      }
      L.tiles.push_back(Tile{0, i, j - i, L.g_rows[i]});
      i = j;
    }
  }
  std::stable_sort(L.tiles.begin(), L.tiles.end(),
                   [](const Tile& a, const Tile& b) { return a.first_row < b.first_row; });
}

void release_device(ogs_handle_s* h) {
  if (h->arena) cudaFree(h->arena);
  if (h->stage) cudaFree(h->stage);
  h->arena = nullptr;
  h->stage = nullptr;
  h->arena_bytes = h->stage_bytes = 0;
  h->dmaps = DevMaps{};
}

ogs_status upload_layout(ogs_handle_s* h) {
  HostLayout& L = h->lay;
  const bool sgn = (h->kind == OGS_SIGNED);
  struct Piece { const void* src; size_t bytes; size_t off; };
  std::vector<Piece> pieces;
  size_t total = 0;
  auto add = [&](const void* src, size_t bytes) -> size_t {
    const size_t off = total;
    pieces.push_back(Piece{src, bytes, off});
    total = align_up(total + std::max<size_t>(bytes, 1), 256);
    return off;
  };
  size_t o_cols[kDmax + 1], o_rows[kDmax + 1], o_mask[kDmax + 1];
  for (int d = 1; d <= kDmax; ++d) {
    o_cols[d] = add(L.cols[d].data(), L.cols[d].size() * 4);
    o_rows[d] = add(L.rows[d].data(), L.rows[d].size() * 4);
    o_mask[d] = sgn ? add(L.nmask[d].data(), L.nmask[d].size()) : 0;
  }
  const size_t o_grows = add(L.g_rows.data(), L.g_rows.size() * 4);
  const size_t o_gsT = add(L.g_startsT.data(), L.g_startsT.size() * 4);
  const size_t o_gcT = add(L.g_colsT.data(), L.g_colsT.size() * 4);
  const size_t o_gsN = sgn ? add(L.g_startsN.data(), L.g_startsN.size() * 4) : o_gsT;
  const size_t o_gcN = sgn ? add(L.g_colsN.data(), L.g_colsN.size() * 4) : o_gcT;
  const size_t o_tiles = add(L.tiles.data(), L.tiles.size() * sizeof(Tile));

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(OGS_EDEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  char* base = nullptr;
  e = cudaMalloc(reinterpret_cast<void**>(&base), total);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(e == cudaErrorMemoryAllocation ? OGS_ENOMEM : OGS_EDEVICE,
                     std::string("cudaMalloc of maps: ") + cudaGetErrorString(e));
  }
  for (const Piece& p : pieces) {
    if (!p.bytes) continue;
    e = cudaMemcpy(base + p.off, p.src, p.bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      cudaFree(base);
      return set_error(OGS_EDEVICE, std::string("cudaMemcpy of maps: ") + cudaGetErrorString(e));
    }
  }
  h->device = dev;
  h->arena = base;
  h->arena_bytes = total;
  DevMaps& m = h->dmaps;
  m = DevMaps{};
  for (int d = 1; d <= kDmax; ++d) {
    m.b[d].cols = reinterpret_cast<const int32_t*>(base + o_cols[d]);
    m.b[d].rows = reinterpret_cast<const int32_t*>(base + o_rows[d]);
    m.b[d].nmask = sgn ? reinterpret_cast<const uint8_t*>(base + o_mask[d]) : nullptr;
    m.b[d].n = static_cast<int32_t>(L.rows[d].size());
    m.b[d].nP = L.nP[d];
  }
  m.g.rows = reinterpret_cast<const int32_t*>(base + o_grows);
  m.g.startsT = reinterpret_cast<const int32_t*>(base + o_gsT);
  m.g.colsT = reinterpret_cast<const int32_t*>(base + o_gcT);
  m.g.startsN = reinterpret_cast<const int32_t*>(base + o_gsN);
  m.g.colsN = reinterpret_cast<const int32_t*>(base + o_gcN);
  m.g.n = static_cast<int32_t>(L.g_rows.size());
  m.g.nP = L.g_nP;
  m.tiles = reinterpret_cast<const Tile*>(base + o_tiles);
  m.ntiles = static_cast<int32_t>(L.tiles.size());
  m.signed_maps = sgn ? 1 : 0;
  return OGS_OK;
}

}  // namespace ogsgb
