// ogs_async.cuh -- the warp pipeline with its value gathers staged through
// shared memory by cp.async.
//
// Same work items, arithmetic and stores as ogs_warp_kernel (ogs_warp.cuh;
// the reference fold is ogsOperator.cpp:60-97, 206-238, 311-360).  What
// changes is how many loads a warp keeps in flight.  The register pipeline
// holds one item's values and the next item's column ids; its registers cap
// it there, and the kernel is latency-bound (ncu: DRAM well under half busy,
// long-scoreboard stalls first).  Here the value gathers of an item are
// cp.async copies into a per-warp ring of shared memory, which hold no
// registers while in flight, so each warp keeps two items' values and a
// third item's column ids in flight:
//
//   iteration for item i:  issue gathers of item i+W into stage (s+1) % 2
//                          issue column-id loads of item i+2W (registers)
//                          wait for the gathers of item i (stage s)
//                          fold item i from shared memory, store
//
// Every lane gathers and later folds its own entries only, so no barrier of
// any kind is needed: cp.async.wait_group makes a thread's own completed
// copies visible to it.  Two stages suffice: the stage an iteration refills
// is the one the previous iteration read, and every value read there was
// consumed by the fold (in-order issue, and the asm's memory clobber keeps
// the compiler from moving the reads) before this iteration's cp.async
// issues.  A third stage only takes shared memory from L1 (measured slower).
#pragma once

#include <cstdint>

#include "ogs_warp.cuh"

#ifndef OGS_ASYNC
#define OGS_ASYNC 1
#endif

namespace ogsgb {

#ifndef OGS_ASYNC_STAGES
#define OGS_ASYNC_STAGES 2
#endif
constexpr int kAsyncStages = OGS_ASYNC_STAGES;
// k > 1 interleaved: split a tile's (row lane, component) units across its k
// parts so neighbouring threads take one node's neighbouring values (1), or
// give part j component j of every row lane (0).
// Resident CTAs per SM of the grid (0: as many as fit).
#ifndef OGS_ASYNC_CTAS
#define OGS_ASYNC_CTAS 0
#endif
#ifndef OGS_KI_SPLIT
#define OGS_KI_SPLIT 1
#endif

template <typename T>
__device__ __forceinline__ void cp_async_elem(T* smem, const T* gmem) {
  const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
  if (sizeof(T) == 8)
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(s), "l"(gmem) : "memory");
  else
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}

__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }

template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// `lane` picks the tile rows (rows lane, lane + 32, ...); entry e of the
// thread lives at stage[e * 32 + slot], slot = the thread's own lane.
template <typename T, int MODE, int D>
__device__ __forceinline__ void async_issue_vals(const WarpState& s, const T* src, const T* gv, int64_t stride, int K,
                                                 int k, bool gmask, int lane, int slot, T* stage) {
  constexpr int RPT = warp_rows_per_lane(D);
#pragma unroll
  for (int j = 0; j < RPT; ++j) {
    if (j * 32 + lane < s.cnt) {
      if (MODE == kModeScatter) {
        cp_async_elem(stage + j * 32 + slot, gv + static_cast<int64_t>(s.R[j]) * K + k);
      } else {
#pragma unroll
        for (int q = 0; q < D; ++q)
          if (!gmask || ((s.emask >> (j * D + q)) & 1u))
            cp_async_elem(stage + (j * D + q) * 32 + slot, src + static_cast<int64_t>(s.I[j * D + q]) * stride);
      }
    }
  }
}

template <typename T, int MODE, int D>
__device__ __forceinline__ void async_read_vals(const WarpState& s, bool gmask, int lane, int slot, const T* stage,
                                                T (&V)[kWarpSlots]) {
  constexpr int RPT = warp_rows_per_lane(D);
#pragma unroll
  for (int j = 0; j < RPT; ++j) {
    if (j * 32 + lane < s.cnt) {
      if (MODE == kModeScatter) {
        V[j] = stage[j * 32 + slot];
      } else {
#pragma unroll
        for (int q = 0; q < D; ++q)
          if (!gmask || ((s.emask >> (j * D + q)) & 1u)) V[j * D + q] = stage[(j * D + q) * 32 + slot];
      }
    }
  }
}

template <typename T>
constexpr size_t async_smem_bytes() {
  return static_cast<size_t>(kBlock / 32) * kAsyncStages * kWarpSlots * 32 * sizeof(T);
}

// PLAIN: every member takes part and receives the result (Pattern all zero:
// GatherScatter Sym, Gather/Scatter through the T map) -- the member-mask,
// store-mode and gslib branches drop out at compile time.
template <typename T, int OP, int MODE, int KL, bool PLAIN>
__global__ void __launch_bounds__(kBlock, OGS_WARP_MINB) ogs_async_kernel(const DevMaps m, const FieldArgs f,
                                                                          const Pattern pat_in) {
  const Pattern pat = PLAIN ? Pattern{0, 0, 0, 0} : pat_in;
  extern __shared__ __align__(16) unsigned char async_smem[];
  const int lane = static_cast<int>(threadIdx.x) & 31;
  const int warp = static_cast<int>(threadIdx.x) >> 5;
  T* ring = reinterpret_cast<T*>(async_smem) + static_cast<size_t>(warp) * kAsyncStages * kWarpSlots * 32;
  const int64_t W = static_cast<int64_t>(gridDim.x) * (kBlock / 32);
  const int K = KL == kK1 ? 1 : f.K;
  const int64_t nw = m.nwtiles;
  const int64_t nitems = nw * K;
  const int64_t wid = static_cast<int64_t>(blockIdx.x) * (kBlock / 32) + warp;
  // Warp w takes items w, w+W, w+2W, ...: the grid sweeps the mesh front to
  // back.  k > 1 interleaved: item = (tile, part), tile-major, parts 0..k-1.
  // A tile's 32 row lanes times k components are 32k (row lane, component)
  // units, and part j takes units 32j .. 32j+31: thread t of part j works row
  // lane (32j+t) / k, component (32j+t) % k.  Neighbouring threads then read
  // the k neighbouring values of one node in the same instruction, so a
  // gather touches the sectors of about 32/k nodes instead of 32 (with OGS_KI_SPLIT
  // = 0, part j is component j for all 32 row lanes, and the k warps of a
  // tile meet each node's sectors only through L1).  Separate arrays: item =
  // (array, tile), array-major, so one array and the column ids stay in L2
  // while the grid sweeps it.  (A warp running a contiguous run of (tile,
  // component) items, loading each tile's column ids once, was measured much
  // slower: 83 vs 62 us for k = 3 on 3.5 M permuted nodes.)  Items are
  // followed as (tile, part) pairs, advanced by W without division.
  const int64_t i0 = wid;
  if (i0 >= nitems) return;
  int64_t i = i0;
  const int64_t step = W, iend = nitems;
  // item = outer * M + inner; interleaved: (tile, comp), M = K; many: (comp, tile), M = nw
  const int M = KL == kKMany ? static_cast<int>(nw) : (KL == kKInterleaved ? K : 1);
  const int Wi = static_cast<int>(W);
  const int Wq = KL == kK1 ? Wi : Wi / M, Wr = KL == kK1 ? 0 : Wi % M;
  const int o0 = KL == kK1 ? static_cast<int>(i0) : static_cast<int>(i0 / M);
  const int n0 = KL == kK1 ? 0 : static_cast<int>(i0 - static_cast<int64_t>(o0) * M);
  int tcur = KL == kKMany ? n0 : o0;
  int ccur = KL == kKMany ? o0 : n0;
  const bool use_mask = !PLAIN && (pat.gather_n || pat.scatter_n) && m.signed_maps;
  const bool gmask = !PLAIN && pat.gather_n != 0;
  const int smode = PLAIN ? 0 : pat.scatter_n;
  const bool gslib = !PLAIN && pat.gslib != 0;
  const int64_t stride = KL == kKInterleaved ? K : 1;
  // the item W after (t, c)
  auto advance = [&](int t, int c, int& tn, int& cn) {
    if (KL == kK1) {
      tn = t + Wi;
      cn = 0;
    } else if (KL == kKInterleaved) {
      cn = c + Wr;
      tn = t + Wq;
      if (cn >= M) { cn -= M; tn += 1; }
    } else {
      tn = t + Wr;
      cn = c + Wq;
      if (tn >= M) { tn -= M; cn += 1; }
    }
  };
  T* gv = static_cast<T*>(f.gv);
  // The thread's row lane and component in item part c, recomputed where
  // needed rather than carried through the pipeline (registers).  Division by
  // k as a multiply-high by ceil(2^32 / k), exact while (32k) * k < 2^32.
  const bool split = KL == kKInterleaved && OGS_KI_SPLIT;
  const uint32_t kmagic = split && K > 1 ? 0xFFFFFFFFu / static_cast<uint32_t>(K) + 1u : 0u;
  const bool kmagic_ok = K < 11585;
  auto unit = [&](int c, int& rl, int& comp) {
    if (split) {
      const uint32_t u = static_cast<uint32_t>(c) * 32u + static_cast<uint32_t>(lane);
      rl = static_cast<int>(kmagic_ok ? __umulhi(u, kmagic) : u / static_cast<uint32_t>(K));
      comp = static_cast<int>(u) - rl * K;
    } else {
      rl = lane;
      comp = c;
    }
  };
  int rcur, kcur;
  unit(ccur, rcur, kcur);

  // prologue: the descriptors of items i, i+1 step, i+2 steps in one round
  // trip, the column ids of the first two in the next, then the gathers of
  // item i; the loop's first pass issues the gathers of the next item at once
  int tnxt = 0, cnxt = 0, tnn = 0, cnn = 0;
  const bool has1 = i + step < iend;
  Tile cur = m.wtiles[tcur];
  Tile nxt{}, nn{};
  if (has1) {
    advance(tcur, ccur, tnxt, cnxt);
    nxt = m.wtiles[tnxt];
    if (i + 2 * step < iend) {
      advance(tnxt, cnxt, tnn, cnn);
      nn = m.wtiles[tnn];
    }
  }
  WarpState scur, snxt;
#define OGS_A_LOAD(D, TILE, TI, RL, S) warp_load_state<MODE, D>(m.b[D], TILE, m.wemask, TI, use_mask, pat, RL, S)
#define OGS_A_LOAD_CUR(D) OGS_A_LOAD(D, cur, tcur, rcur, scur)
  OGS_DEGREE_SWITCH(cur.bucket, OGS_A_LOAD_CUR)
#undef OGS_A_LOAD_CUR
  if (has1) {
    int rnxt, knxt;
    unit(cnxt, rnxt, knxt);
#define OGS_A_LOAD_NXT(D) OGS_A_LOAD(D, nxt, tnxt, rnxt, snxt)
    OGS_DEGREE_SWITCH(nxt.bucket, OGS_A_LOAD_NXT)
#undef OGS_A_LOAD_NXT
  }
  {
    const T* src = (MODE == kModeScatter) ? nullptr : field_base<T>(f, kcur);
#define OGS_A_ISSUE0(D) async_issue_vals<T, MODE, D>(scur, src, gv, stride, K, kcur, gmask, rcur, lane, ring)
    OGS_DEGREE_SWITCH(cur.bucket, OGS_A_ISSUE0)
#undef OGS_A_ISSUE0
  }
  cp_async_commit();

  int stage = 0;
  for (;;) {
    const bool more1 = i + step < iend;
    const bool more2 = i + 2 * step < iend;
    const int nstage = stage == kAsyncStages - 1 ? 0 : stage + 1;
    if (more1) {
      int rnxt, knxt;
      unit(cnxt, rnxt, knxt);
      const T* src1 = (MODE == kModeScatter) ? nullptr : field_base<T>(f, knxt);
      T* st1 = ring + nstage * (kWarpSlots * 32);
#define OGS_A_ISSUE1(D) async_issue_vals<T, MODE, D>(snxt, src1, gv, stride, K, knxt, gmask, rnxt, lane, st1)
      OGS_DEGREE_SWITCH(nxt.bucket, OGS_A_ISSUE1)
#undef OGS_A_ISSUE1
    }
    cp_async_commit();
    WarpState snn;
    Tile n3{};
    int tn3 = 0, cn3 = 0;
    if (more2) {
      int rnn, knn;
      unit(cnn, rnn, knn);
#define OGS_A_LOAD_NN(D) OGS_A_LOAD(D, nn, tnn, rnn, snn)
      OGS_DEGREE_SWITCH(nn.bucket, OGS_A_LOAD_NN)
#undef OGS_A_LOAD_NN
      if (i + 3 * step < iend) {
        advance(tnn, cnn, tn3, cn3);
        n3 = m.wtiles[tn3];
      }
    }
    cp_async_wait<1>();  // the gathers of item i are in
    {
      unit(ccur, rcur, kcur);
      T* dst = (MODE == kModeGather) ? nullptr : field_base<T>(f, kcur);
      const T* st0 = ring + stage * (kWarpSlots * 32);
      T V[kWarpSlots];
#define OGS_A_FOLD(D)                                                                              \
  do {                                                                                             \
    async_read_vals<T, MODE, D>(scur, gmask, rcur, lane, st0, V);                                  \
    warp_fold_store<T, OP, MODE, D>(scur, dst, gv, stride, K, kcur, gmask, smode, gslib, rcur, V); \
  } while (0)
      OGS_DEGREE_SWITCH(cur.bucket, OGS_A_FOLD)
#undef OGS_A_FOLD
    }
    if (!more1) break;
    i += step;
    stage = nstage;
    cur = nxt;
    scur = snxt;
    tcur = tnxt;
    ccur = cnxt;
    nxt = nn;
    snxt = snn;
    tnxt = tnn;
    cnxt = cnn;
    nn = n3;
    tnn = tn3;
    cnn = cn3;
  }
  cp_async_wait<0>();
#undef OGS_A_LOAD
}

template <typename T, int OP, int MODE, int KL, bool PLAIN>
inline int async_grid(int64_t nitems) {
  static DeviceCache cache;
  int dev = 0;
  cudaGetDevice(&dev);
  const int cached = cache.get(dev, [dev] {
    int bps = 0, sms = 0;
    // above 48 KB (more entries per lane) the dynamic shared memory must be opted into
    if (async_smem_bytes<T>() > 48 * 1024)
      cudaFuncSetAttribute(ogs_async_kernel<T, OP, MODE, KL, PLAIN>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                           static_cast<int>(async_smem_bytes<T>()));
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, ogs_async_kernel<T, OP, MODE, KL, PLAIN>, kBlock,
                                                  async_smem_bytes<T>());
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
#if OGS_ASYNC_CTAS > 0
    if (bps > OGS_ASYNC_CTAS) bps = OGS_ASYNC_CTAS;
#endif
    return (bps > 0 ? bps : 1) * (sms > 0 ? sms : 1);
  });
  const int64_t need = (nitems + (kBlock / 32) - 1) / (kBlock / 32);
  return static_cast<int>(need < cached ? need : cached);
}

template <typename T, int OP, int MODE, int KL>
inline void launch_async_kl(const DevMaps& m, const FieldArgs& f, Pattern pat, cudaStream_t s) {
  const int64_t nitems = static_cast<int64_t>(m.nwtiles) * (KL == kK1 ? 1 : f.K);
  const bool plain = !pat.gather_n && !pat.scatter_n && !pat.limit_n && !pat.gslib;
  if (plain) {
    const int grid = async_grid<T, OP, MODE, KL, true>(nitems);
    ogs_async_kernel<T, OP, MODE, KL, true><<<grid, kBlock, async_smem_bytes<T>(), s>>>(m, f, pat);
  } else {
    const int grid = async_grid<T, OP, MODE, KL, false>(nitems);
    ogs_async_kernel<T, OP, MODE, KL, false><<<grid, kBlock, async_smem_bytes<T>(), s>>>(m, f, pat);
  }
}

// Exact-degree tiles on the async pipeline, general tiles on the direct kernel.
template <typename T, int OP, int MODE>
inline cudaError_t launch_async(const DevMaps& m, const FieldArgs& f, Pattern pat, cudaStream_t s) {
  if (m.nwtiles > 0) {
    if (f.is_many) launch_async_kl<T, OP, MODE, kKMany>(m, f, pat, s);
    else if (f.K == 1) launch_async_kl<T, OP, MODE, kK1>(m, f, pat, s);
    else launch_async_kl<T, OP, MODE, kKInterleaved>(m, f, pat, s);
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
