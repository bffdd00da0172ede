// ogs_warp.cuh -- persistent, warp-pipelined gather-scatter kernel with the
// gathered values in registers: the kernel of Gather and Scatter (a row
// writes or reads one gathered value, and holding a second tile's gathers in
// the shared-memory ring of ogs_async.cuh costs more there than it hides),
// and the fold and state helpers the cp.async pipeline shares.
//
// Arithmetic as in ogs_kernels.cuh (one fold per row from the op identity
// over the members in ascending local index: ogsOperator.cpp:60-97, 206-238,
// 311-360).  The data movement is organised per warp, with no block-level
// synchronisation at all:
//
//  * Work items are warp tiles (for k > 1 interleaved, a tile's parts; for
//    separate arrays, the array; see KLayout).  A warp tile holds 32 lanes x
//    kWarpEntries member entries of one exact-degree bucket: lane l owns rows
//    l, l+32, ... of the tile, each with its d members.  Tiles are ordered by
//    first row; warp w of the grid takes items w, w+W, w+2W, ... so the grid
//    sweeps the mesh front to back and the nodes that neighbouring tiles share
//    are served from L2.
//  * Every iteration issues, back to back and without waiting: the value
//    gathers of the current item, the column ids (and row ids / N masks) of
//    the next item, and the descriptor of the item after that.  Only then does
//    it fold the current rows and store the results.  One memory round trip
//    per item instead of three (descriptor -> column ids -> values).
//
// Stores to the field never alias a later item's loads (every local node
// belongs to one row), so loads and stores of different items may be in
// flight together.
#pragma once

#include <cstdint>

#include "ogs_kernels.cuh"

// Minimum resident CTAs per SM the register allocation must allow.
#ifndef OGS_WARP_MINB
#define OGS_WARP_MINB 3
#endif

namespace ogsgb {

// GatherScatter skips the store to a member whose value already has the
// result's bits: degree-1 rows under Add (x + 0 == x), the member holding the
// maximum under Max, and so on.  Memory ends bit-identical to storing every
// member; the store traffic of those members disappears.  OGS_SILENT_STORE=0
// stores every member (for comparisons).
#ifndef OGS_SILENT_STORE
#define OGS_SILENT_STORE 1
#endif

template <typename T>
__device__ __forceinline__ bool same_bits(const T a, const T b) {
  using U = typename std::conditional<sizeof(T) == 8, unsigned long long, unsigned int>::type;
  U x, y;
  memcpy(&x, &a, sizeof(T));
  memcpy(&y, &b, sizeof(T));
  return x == y;
}

// Column ids, row ids and the per-lane entry mask of one warp tile.
struct WarpState {
  int32_t I[kWarpSlots];  // entry e = j*D + q: member q of the lane's row j
  int32_t R[kWarpSlots];  // row ids (Gather / Scatter only)
  uint32_t emask;           // bit e: entry e is in the N map (Signed only)
  int32_t cnt;              // rows of the tile this call processes
};

template <int MODE, int D>
__device__ __forceinline__ void warp_load_state(const DevBucket& b, const Tile& t, const uint8_t* wemask,
                                                int tile_index, bool use_mask, const Pattern& pat, int lane,
                                                WarpState& s) {
  constexpr int RPT = warp_rows_per_lane(D);
  s.cnt = pat.limit_n ? min(t.count, b.nP - t.begin) : t.count;
  s.emask = use_mask ? __ldg(wemask + static_cast<int64_t>(tile_index) * 32 + lane) : 0xFFu;
#pragma unroll
  for (int j = 0; j < RPT; ++j) {
    const int r = j * 32 + lane;
    if (r < s.cnt) {
      // (checked builds) a tile reaching past its bucket reads bucket row 0
      const int idx = OGS_CHECK_BOUNDS ? checked_id(t.begin + r, b.n, b.err) : t.begin + r;
#pragma unroll
      for (int q = 0; q < D; ++q)
        s.I[j * D + q] = checked_id(__ldg(b.cols + static_cast<int64_t>(q) * b.stride + idx), b.nnodes, b.err);
      if (MODE != kModeGS) s.R[j] = checked_id(__ldg(b.rows + idx), b.nrows, b.err);
    }
  }
}

template <typename T, int MODE, int D>
__device__ __forceinline__ void warp_load_vals(const WarpState& s, const T* src, const T* gv, int64_t stride,
                                               int K, int k, bool gmask, int lane, T (&V)[kWarpSlots]) {
  constexpr int RPT = warp_rows_per_lane(D);
#pragma unroll
  for (int j = 0; j < RPT; ++j) {
    if (j * 32 + lane < s.cnt) {
      if (MODE == kModeScatter) {
        V[j] = gv[static_cast<int64_t>(s.R[j]) * K + k];
      } else {
#pragma unroll
        for (int q = 0; q < D; ++q)
          if (!gmask || ((s.emask >> (j * D + q)) & 1u)) V[j * D + q] = src[static_cast<int64_t>(s.I[j * D + q]) * stride];
      }
    }
  }
}

// smode: 0 write every member, 1 only N members, 2 N members or, in a row
// without any, member 0 (gslib transpose 1).  gslib: fold from the first
// member taking part instead of from the identity (gs_local.c:58-72).
template <typename T, int OP, int MODE, int D>
__device__ __forceinline__ void warp_fold_store(const WarpState& s, T* dst, T* gv, int64_t stride, int K, int k,
                                                bool gmask, int smode, bool gslib, int lane,
                                                const T (&V)[kWarpSlots]) {
  constexpr int RPT = warp_rows_per_lane(D);
#pragma unroll
  for (int j = 0; j < RPT; ++j) {
    if (j * 32 + lane < s.cnt) {
      T a;
      if (MODE == kModeScatter) {
        a = V[j];
      } else if (gslib) {
        // members are stored unflagged first, so member 0 takes part whenever any does
        a = (!gmask || (s.emask >> (j * D)) & 1u) ? V[j * D] : op_init_gs<T, OP>();
#pragma unroll
        for (int q = 1; q < D; ++q)
          if (!gmask || ((s.emask >> (j * D + q)) & 1u)) op_apply<T, OP>(a, V[j * D + q]);
      } else if ((OP == OGS_ADD || OP == OGS_MUL) && !gmask) {
        a = fold_from_first<T, OP, D>(V, j * D);
      } else {
        a = op_init<T, OP>();
#pragma unroll
        for (int q = 0; q < D; ++q)
          if (!gmask || ((s.emask >> (j * D + q)) & 1u)) op_apply<T, OP>(a, V[j * D + q]);
      }
      if (MODE == kModeGather) {
        gv[static_cast<int64_t>(s.R[j]) * K + k] = a;
      } else {
        const uint32_t row_n = (s.emask >> (j * D)) & ((1u << D) - 1u);
#pragma unroll
        for (int q = 0; q < D; ++q) {
          const bool in_n = (s.emask >> (j * D + q)) & 1u;
          if (smode == 1 && !in_n) continue;
          if (smode == 2 && !(row_n ? in_n : q == 0)) continue;
          // a member that took part in the fold still holds its value in V
          if (OGS_SILENT_STORE && MODE == kModeGS && (!gmask || in_n) && same_bits(a, V[j * D + q])) continue;
          dst[static_cast<int64_t>(s.I[j * D + q]) * stride] = a;
        }
      }
    }
  }
}

#define OGS_DEGREE_SWITCH(bucket, CALL) \
  switch (bucket) {                     \
    case 1: CALL(1); break;             \
    case 2: CALL(2); break;             \
    case 3: CALL(3); break;             \
    case 4: CALL(4); break;             \
    case 5: CALL(5); break;             \
    case 6: CALL(6); break;             \
    case 7: CALL(7); break;             \
    default: CALL(8); break;            \
  }

// How the k components of a field map onto work items.
enum KLayout : int {
  kK1 = 0,          // k = 1: item = tile
  kKInterleaved = 1,  // v[c + n*k], k > 1: item = (tile, part), tile-major;
                      // part j takes the tile's (row lane, component) units
                      // 32j .. 32j+31, so neighbouring threads read the k
                      // values of one node in one instruction.  (One item per
                      // tile looping over the components was slower: 86 vs
                      // 66 us for k = 3 on 3.5 M permuted nodes.)
  kKMany = 2,       // k separate arrays: item = (array, tile), array-major, so
                    // one array and the column ids stay resident in L2 while
                    // the grid sweeps that array
};

template <typename T, int OP, int MODE, int KL, bool PLAIN>
__global__ void __launch_bounds__(kBlock, OGS_WARP_MINB) ogs_warp_kernel(const DevMaps m, const FieldArgs f,
                                                                         const Pattern pat_in) {
  const Pattern pat = PLAIN ? Pattern{0, 0, 0, 0} : pat_in;
  const int lane = static_cast<int>(threadIdx.x) & 31;
  const int64_t W = static_cast<int64_t>(gridDim.x) * (kBlock / 32);
  const int K = KL == kK1 ? 1 : f.K;
  const int64_t nw = m.nwtiles;
  const int64_t nitems = nw * K;
  int64_t i = static_cast<int64_t>(blockIdx.x) * (kBlock / 32) + (threadIdx.x >> 5);
  if (i >= nitems) return;
  const bool use_mask = !PLAIN && (pat.gather_n || pat.scatter_n) && m.signed_maps;
  const bool gmask = !PLAIN && pat.gather_n != 0;
  const int smode = PLAIN ? 0 : pat.scatter_n;
  const bool gslib = !PLAIN && pat.gslib != 0;
  const int64_t stride = KL == kKInterleaved ? K : 1;
  auto tile_of = [&](int64_t item) {
    return static_cast<int>(KL == kKMany ? item % nw : (KL == kKInterleaved ? item / K : item));
  };
  // k > 1 interleaved: item (tile, part j); thread t works row lane
  // (32j + t) / k, component (32j + t) % k, as in the cp.async pipeline
  const uint32_t kmagic = KL == kKInterleaved && K > 1 ? 0xFFFFFFFFu / static_cast<uint32_t>(K) + 1u : 0u;
  auto row_lane = [&](int64_t item, int& comp) {
    if (KL != kKInterleaved) {
      comp = KL == kKMany ? static_cast<int>(item / nw) : 0;
      return lane;
    }
    const uint32_t u = static_cast<uint32_t>(item % K) * 32u + static_cast<uint32_t>(lane);
    const int rl = static_cast<int>(K < 11585 ? __umulhi(u, kmagic) : u / static_cast<uint32_t>(K));
    comp = static_cast<int>(u) - rl * K;
    return rl;
  };

  int tcur = tile_of(i);
  Tile cur = m.wtiles[tcur];
  WarpState scur;
  int ccur;
  int rcur = row_lane(i, ccur);
#define OGS_LOAD_CUR(D) warp_load_state<MODE, D>(m.b[D], cur, m.wemask, tcur, use_mask, pat, rcur, scur)
  OGS_DEGREE_SWITCH(cur.bucket, OGS_LOAD_CUR)
#undef OGS_LOAD_CUR
  Tile nxt{};
  if (i + W < nitems) nxt = m.wtiles[tile_of(i + W)];

  T* gv = static_cast<T*>(f.gv);
  for (;;) {
    const int k0 = ccur;
    const T* src = (MODE == kModeScatter) ? nullptr : field_base<T>(f, k0);
    T* dst = (MODE == kModeGather) ? nullptr : field_base<T>(f, k0);
    T V[kWarpSlots];
#define OGS_VALS(D) warp_load_vals<T, MODE, D>(scur, src, gv, stride, K, k0, gmask, rcur, V)
    OGS_DEGREE_SWITCH(cur.bucket, OGS_VALS)
#undef OGS_VALS
    const bool more = i + W < nitems;
    WarpState snxt;
    Tile nn{};
    int tnxt = 0, cnxt = 0, rnxt = lane;
    if (more) {
      tnxt = tile_of(i + W);
      rnxt = row_lane(i + W, cnxt);
#define OGS_LOAD_NXT(D) warp_load_state<MODE, D>(m.b[D], nxt, m.wemask, tnxt, use_mask, pat, rnxt, snxt)
      OGS_DEGREE_SWITCH(nxt.bucket, OGS_LOAD_NXT)
#undef OGS_LOAD_NXT
      if (i + 2 * W < nitems) nn = m.wtiles[tile_of(i + 2 * W)];
    }
#define OGS_FOLD(D) warp_fold_store<T, OP, MODE, D>(scur, dst, gv, stride, K, k0, gmask, smode, gslib, rcur, V)
    OGS_DEGREE_SWITCH(cur.bucket, OGS_FOLD)
#undef OGS_FOLD
    if (!more) break;
    i += W;
    cur = nxt;
    scur = snxt;
    nxt = nn;
    tcur = tnxt;
    ccur = cnxt;
    rcur = rnxt;
  }
}


// CTAs of the warp kernel resident per SM, once per instantiation and device.
template <typename T, int OP, int MODE, int KL, bool PLAIN>
inline int warp_grid(int64_t nitems) {
  static DeviceCache cache;
  int dev = 0;
  cudaGetDevice(&dev);
  const int cached = cache.get(dev, [dev] {
    int bps = 0, sms = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ogs_warp_kernel<T, OP, MODE, KL, PLAIN>, kBlock, 0);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return (bps > 0 ? bps : 1) * (sms > 0 ? sms : 1);
  });
  const int64_t need = (nitems + (kBlock / 32) - 1) / (kBlock / 32);
  return static_cast<int>(need < cached ? need : cached);
}

template <typename T, int OP, int MODE, int KL, bool PLAIN>
inline void launch_warp_kl(const DevMaps& m, const FieldArgs& f, Pattern pat, cudaStream_t s) {
  const int64_t nitems = static_cast<int64_t>(m.nwtiles) * (KL == kK1 ? 1 : f.K);
  const int grid = warp_grid<T, OP, MODE, KL, PLAIN>(nitems);
  ogs_warp_kernel<T, OP, MODE, KL, PLAIN><<<grid, kBlock, 0, s>>>(m, f, pat);
}

template <typename T, int OP, int MODE, bool PLAIN>
inline void launch_warp_plain(const DevMaps& m, const FieldArgs& f, Pattern pat, cudaStream_t s) {
  if (f.is_many) launch_warp_kl<T, OP, MODE, kKMany, PLAIN>(m, f, pat, s);
  else if (f.K == 1) launch_warp_kl<T, OP, MODE, kK1, PLAIN>(m, f, pat, s);
  else launch_warp_kl<T, OP, MODE, kKInterleaved, PLAIN>(m, f, pat, s);
}

template <typename T, int OP, int MODE>
inline cudaError_t launch_warp(const DevMaps& m, const FieldArgs& f, Pattern pat, cudaStream_t s) {
  if (m.nwtiles > 0) {
    const bool plain = !pat.gather_n && !pat.scatter_n && !pat.limit_n && !pat.gslib;
    if (plain) launch_warp_plain<T, OP, MODE, true>(m, f, pat, s);
    else launch_warp_plain<T, OP, MODE, false>(m, f, pat, s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  if (m.ngtiles > 0) {
    DevMaps g = m;
    g.tiles = m.gtiles;
    g.ntiles = m.ngtiles;
    return launch_direct<T, OP, MODE>(g, f, pat, s);
  }
  return cudaSuccess;
}

}  // namespace ogsgb
