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
#include <climits>
#include <limits>

#include <cuda_runtime.h>

#include "ogs_internal.hpp"
#include "ogs_trace.hpp"

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
  TraceRange trace("ogs_setup: maps on the host");
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
  TraceRange trace("ogs_setup: layout on the host");
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
    // rows without members (possible in operators built from caller maps) go
    // to the general bucket: a Gather still writes the op identity there
    if (d >= 1 && d <= kDmax) cnt[d]++;
    else { cnt[0]++; gnnzT += d; gnnzN += rsN[r + 1] - rsN[r]; }
  }
  int64_t stride[kDmax + 1] = {0};
  for (int d = 1; d <= kDmax; ++d) {
    stride[d] = (cnt[d] + 3) / 4 * 4;
    L.cols[d].assign(static_cast<size_t>(stride[d]) * d, 0);
    L.rows[d].assign(stride[d], 0);
    L.nmask[d].assign(sgn ? (cnt[d] + 15) / 16 * 16 : 0, 0);
    L.nP[d] = 0;
    L.n[d] = static_cast<int32_t>(cnt[d]);
  }
  L.g_rows.clear(); L.g_startsT.assign(1, 0); L.g_colsT.clear();
  L.g_startsN.assign(1, 0); L.g_colsN.clear();
  L.g_rows.reserve(cnt[0]); L.g_colsT.reserve(gnnzT); L.g_colsN.reserve(gnnzN);
  L.g_nP = 0;

  int64_t fill[kDmax + 1] = {0};
  for (int64_t r = 0; r < R; ++r) {
    const int32_t s = rsT[r], d = rsT[r + 1] - s;
    const bool inP = r < h->NlocalP;
    if (d >= 1 && d <= kDmax) {
      const int64_t i = fill[d]++;
      const int64_t n = stride[d];
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
  L.gtiles.clear();
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
      L.gtiles.push_back(Tile{0, i, j - i, L.g_rows[i]});
      i = j;
    }
  }
  auto by_row = [](const Tile& a, const Tile& b) { return a.first_row < b.first_row; };
  // warp tiles and, for Signed maps, each lane's entry mask: bit j*d+q set
  // when member q of the lane's row j is in the N map
  L.wtiles.clear();
  for (int d = 1; d <= kDmax; ++d) {
    const int32_t n = static_cast<int32_t>(cnt[d]);
    const int32_t step = warp_rows_per_tile(d);
    for (int32_t i = 0; i < n; i += step)
      L.wtiles.push_back(Tile{d, i, std::min(step, n - i), L.rows[d][i]});
  }
  std::stable_sort(L.wtiles.begin(), L.wtiles.end(), by_row);
  L.wemask.assign(sgn ? L.wtiles.size() * 32 : 0, 0);
  if (sgn) {
    for (size_t t = 0; t < L.wtiles.size(); ++t) {
      const Tile& w = L.wtiles[t];
      const int d = w.bucket;
      for (int lane = 0; lane < 32; ++lane) {
        uint32_t bits = 0;
        for (int j = 0; j < warp_rows_per_lane(d); ++j) {
          const int r = j * 32 + lane;
          if (r >= w.count) continue;
          const uint32_t mk = L.nmask[d][w.begin + r];
          for (int q = 0; q < d; ++q) bits |= ((mk >> q) & 1u) << (j * d + q);
        }
        L.wemask[t * 32 + lane] = static_cast<uint8_t>(bits);
      }
    }
  }
  L.tiles.insert(L.tiles.end(), L.gtiles.begin(), L.gtiles.end());
  std::stable_sort(L.tiles.begin(), L.tiles.end(), by_row);
  L.g_n = static_cast<int64_t>(L.g_rows.size());
  L.g_nnzT = static_cast<int64_t>(L.g_colsT.size());
  // lowest and highest node of every tile (the host pipeline's slices)
  L.wlo.assign(L.wtiles.size(), INT64_MAX);
  L.whi.assign(L.wtiles.size(), -1);
  for (size_t t = 0; t < L.wtiles.size(); ++t) {
    const Tile& w = L.wtiles[t];
    const int d = w.bucket;
    const int64_t stride = static_cast<int64_t>(L.rows[d].size());
    for (int q = 0; q < d; ++q)
      for (int32_t r = 0; r < w.count; ++r) {
        const int64_t c = L.cols[d][q * stride + w.begin + r];
        L.wlo[t] = std::min(L.wlo[t], c);
        L.whi[t] = std::max(L.whi[t], c);
      }
  }
  L.glo.assign(L.gtiles.size(), INT64_MAX);
  L.ghi.assign(L.gtiles.size(), -1);
  for (size_t t = 0; t < L.gtiles.size(); ++t) {
    const Tile& w = L.gtiles[t];
    for (int32_t q = L.g_startsT[w.begin]; q < L.g_startsT[w.begin + w.count]; ++q) {
      L.glo[t] = std::min<int64_t>(L.glo[t], L.g_colsT[q]);
      L.ghi[t] = std::max<int64_t>(L.ghi[t], L.g_colsT[q]);
    }
  }
  build_phases(h, OGS_HOST_PHASES);
}

void build_phases(ogs_handle_s* h, int max_phases) {
  HostLayout& L = h->lay;
  L.phases.clear();
  const int32_t nw = static_cast<int32_t>(L.wtiles.size());
  const int32_t ng = static_cast<int32_t>(L.gtiles.size());
  if (nw + ng == 0) return;
  int P = nw / 256;
  if (P < 1) P = 1;
  if (P > max_phases) P = max_phases;
  // phase boundaries in warp tiles (in quarters of a share); general tiles
  // follow by first row
  std::vector<int64_t> cum(P + 1, 0);
  for (int p = 0; p < P; ++p) {
    int64_t w = 4;
    if (OGS_HOST_TAPER && P >= 6) {
      if (p == 0 || p == P - 1) w = 1;
      else if (p == 1 || p == P - 2) w = 2;
    }
    cum[p + 1] = cum[p] + w;
  }
  for (int p = 0; p < P; ++p) {
    Phase ph{};
    ph.w0 = static_cast<int32_t>(static_cast<int64_t>(nw) * cum[p] / cum[P]);
    ph.w1 = static_cast<int32_t>(static_cast<int64_t>(nw) * cum[p + 1] / cum[P]);
    L.phases.push_back(ph);
  }
  int32_t g = 0;
  for (int p = 0; p < P; ++p) {
    Phase& ph = L.phases[p];
    ph.g0 = g;
    const bool last = (p == P - 1);
    const int32_t row_end = last || ph.w1 >= nw ? INT32_MAX : L.wtiles[ph.w1].first_row;
    while (g < ng && (last || L.gtiles[g].first_row < row_end)) g++;
    ph.g1 = g;
    int64_t lo = INT64_MAX, hi = -1;
    for (int32_t t = ph.w0; t < ph.w1; ++t) {
      lo = std::min(lo, L.wlo[t]);
      hi = std::max(hi, L.whi[t]);
    }
    for (int32_t t = ph.g0; t < ph.g1; ++t) {
      lo = std::min(lo, L.glo[t]);
      hi = std::max(hi, L.ghi[t]);
    }
    ph.lo = lo;
    ph.hi = hi;
  }
  // Chunk boundaries sit on multiples of kCopyAlignNodes nodes (4 KiB and up
  // for any node size): copy engines move misaligned chunks much more slowly
  // (8 chunks each way at 8-byte offsets: 0.59 ms, at 4 KiB offsets: 0.43 ms
  // for 56.6 MB each way on GB300).  Copying a node in earlier or out later
  // than it must is always safe.
  constexpr int64_t kCopyAlignNodes = 1024;
  auto up = [&](int64_t x) { return std::min<int64_t>(h->N, (x + kCopyAlignNodes - 1) / kCopyAlignNodes * kCopyAlignNodes); };
  auto down = [&](int64_t x) { return x / kCopyAlignNodes * kCopyAlignNodes; };
  // host->device chunk p: up to the highest node phases <= p touch (all of N at the end)
  int64_t need = 0;
  for (int p = 0; p < P; ++p) {
    Phase& ph = L.phases[p];
    ph.h0 = need;
    need = std::max(need, up(ph.hi + 1));
    if (p == P - 1) need = h->N;
    ph.h1 = need;
  }
  // device->host chunk p: nodes below the lowest node any later phase touches
  int64_t fin = h->N;
  std::vector<int64_t> final_at(P);
  for (int p = P - 1; p >= 0; --p) {
    final_at[p] = p == P - 1 ? fin : down(fin);
    fin = std::min(fin, L.phases[p].lo);
  }
  // (never beyond the nodes already copied in: nodes that no row touches --
  // zero ids -- may leave a gap between one slice's nodes and the next's,
  // and their values must have come in before they go back out)
  int64_t prev = 0;
  for (int p = 0; p < P; ++p) {
    L.phases[p].d0 = prev;
    L.phases[p].d1 = std::max(prev, std::min(final_at[p], L.phases[p].h1));
    prev = L.phases[p].d1;
  }
  // Rows.  Each row belongs to one tile and a tile's rows are >= its first
  // row, so every row below the first row of the next slice's first tile is
  // written by this slice or an earlier one.  A tile's rows end before the
  // first row of the next tile of its bucket.
  const int64_t R = h->NlocalT;
  auto rup = [&](int64_t x) { return std::min<int64_t>(R, (x + kCopyAlignNodes - 1) / kCopyAlignNodes * kCopyAlignNodes); };
  auto rdown = [&](int64_t x) { return x / kCopyAlignNodes * kCopyAlignNodes; };
  std::vector<int64_t> wend(nw, R), gend(ng, R);  // one past each tile's last row
  {
    int32_t next_first[kDmax + 1];
    for (int d = 0; d <= kDmax; ++d) next_first[d] = static_cast<int32_t>(R);
    for (int32_t t = nw - 1; t >= 0; --t) {
      const Tile& w = L.wtiles[t];
      wend[t] = next_first[w.bucket];
      next_first[w.bucket] = w.first_row;
    }
    int32_t gnext = static_cast<int32_t>(R);
    for (int32_t t = ng - 1; t >= 0; --t) {
      gend[t] = gnext;
      gnext = L.gtiles[t].first_row;
    }
  }
  int64_t rprev = 0, rneed = 0;
  for (int p = 0; p < P; ++p) {
    Phase& ph = L.phases[p];
    int64_t later = R;  // lowest first row of any later slice's tile
    if (ph.w1 < nw) later = std::min<int64_t>(later, L.wtiles[ph.w1].first_row);
    if (ph.g1 < ng) later = std::min<int64_t>(later, L.gtiles[ph.g1].first_row);
    ph.r0 = rprev;
    ph.r1 = std::max(rprev, p == P - 1 ? R : rdown(later));
    rprev = ph.r1;
    for (int32_t t = ph.w0; t < ph.w1; ++t) rneed = std::max(rneed, rup(wend[t]));
    for (int32_t t = ph.g0; t < ph.g1; ++t) rneed = std::max(rneed, rup(gend[t]));
    ph.rn = p == P - 1 ? R : rneed;
  }
}

void set_id_bounds(const ogs_handle_s* h, DevMaps& m, unsigned int* err) {
  for (int d = 1; d <= kDmax; ++d) {
    m.b[d].nnodes = static_cast<int32_t>(h->N);
    m.b[d].nrows = static_cast<int32_t>(h->NlocalT);
    m.b[d].err = err;
  }
  m.g.nnodes = static_cast<int32_t>(h->N);
  m.g.nrows = static_cast<int32_t>(h->NlocalT);
  m.g.err = err;
}

DevMaps phase_maps(const DevMaps& m, const Phase& p) {
  DevMaps r = m;
  r.wtiles = m.wtiles + p.w0;
  r.nwtiles = p.w1 - p.w0;
  if (m.wemask) r.wemask = m.wemask + static_cast<int64_t>(p.w0) * 32;
  r.gtiles = m.gtiles + p.g0;
  r.ngtiles = p.g1 - p.g0;
  r.ntiles = r.nwtiles + r.ngtiles;
  return r;
}

void release_device(ogs_handle_s* h) {
  for (auto& g : h->host_graphs) cudaGraphExecDestroy(static_cast<cudaGraphExec_t>(g.exec));
  h->host_graphs.clear();
  if (h->capture) cudaStreamDestroy(static_cast<cudaStream_t>(h->capture));
  h->capture = nullptr;
  for (void* e : h->events) cudaEventDestroy(static_cast<cudaEvent_t>(e));
  h->events.clear();
  if (h->copy_in) cudaStreamDestroy(static_cast<cudaStream_t>(h->copy_in));
  if (h->copy_out) cudaStreamDestroy(static_cast<cudaStream_t>(h->copy_out));
  h->copy_in = h->copy_out = nullptr;
  if (h->arena) dev_free(h->arena);
  if (h->stage) dev_free(h->stage);
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
  const size_t o_gtiles = add(L.gtiles.data(), L.gtiles.size() * sizeof(Tile));
  const size_t o_wtiles = add(L.wtiles.data(), L.wtiles.size() * sizeof(Tile));
  const size_t o_wemask = add(L.wemask.data(), L.wemask.size());
  // warp records hold device pointers: filled in once the arena exists
  std::vector<WarpRec> wrecs(L.wtiles.size());
  const size_t o_wrecs = add(wrecs.data(), wrecs.size() * sizeof(WarpRec));
  const uint32_t zero = 0;
  const size_t o_err = add(&zero, sizeof(zero));  // ids out of range (checked builds)

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(OGS_EDEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  char* base = nullptr;
  e = dev_malloc(reinterpret_cast<void**>(&base), total);
  if (e != cudaSuccess) {
    cudaGetLastError();
    return set_error(e == cudaErrorMemoryAllocation ? OGS_ENOMEM : OGS_EDEVICE,
                     std::string("cudaMalloc of maps: ") + cudaGetErrorString(e));
  }
  for (size_t t = 0; t < L.wtiles.size(); ++t) {
    const Tile& w = L.wtiles[t];
    WarpRec& r = wrecs[t];
    r.cols = reinterpret_cast<const int32_t*>(base + o_cols[w.bucket]);
    r.rows = reinterpret_cast<const int32_t*>(base + o_rows[w.bucket]);
    r.begin = w.begin;
    r.bucket_count = (w.bucket << 16) | w.count;
    r.stride = static_cast<int32_t>(L.rows[w.bucket].size());
    r.nP = L.nP[w.bucket];
  }
  for (const Piece& p : pieces) {
    if (!p.bytes) continue;
    e = cudaMemcpy(base + p.off, p.src, p.bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
      dev_free(base);
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
    m.b[d].n = L.n[d];
    m.b[d].nP = L.nP[d];
    m.b[d].stride = static_cast<int32_t>(L.rows[d].size());
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
  m.gtiles = reinterpret_cast<const Tile*>(base + o_gtiles);
  m.ngtiles = static_cast<int32_t>(L.gtiles.size());
  m.wtiles = reinterpret_cast<const Tile*>(base + o_wtiles);
  m.nwtiles = static_cast<int32_t>(L.wtiles.size());
  m.wemask = reinterpret_cast<const uint8_t*>(base + o_wemask);
  m.wrecs = reinterpret_cast<const WarpRec*>(base + o_wrecs);
  set_id_bounds(h, m, reinterpret_cast<unsigned int*>(base + o_err));

  m.signed_maps = sgn ? 1 : 0;
  return OGS_OK;
}

}  // namespace ogsgb
