// ogs_internal.hpp -- shared definitions of the GB300 gather-scatter library:
// the device layout of one mesh's maps, the work tiles, and the launch
// interface between the C ABI (ogs_capi.cpp) and the per-type kernel units
// (ogs_kern_*.cu).
#pragma once

#include <atomic>
#include <cstdint>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime_api.h>

#include "ogs_c.h"

#ifdef __CUDACC__
#define OGS_HD __host__ __device__
#else
#define OGS_HD
#endif

namespace ogsgb {

// A launch figure per device (CTAs per SM, SM count), computed on first use.
// Concurrent first uses compute the same value, so filling it without a lock
// is safe; the atomics keep the sharing well defined.
struct DeviceCache {
  static constexpr int kDevices = 64;
  std::atomic<int> v[kDevices];
  template <typename F>
  int get(int dev, F compute) {
    if (dev < 0 || dev >= kDevices) return compute();
    int x = v[dev].load(std::memory_order_acquire);
    if (x == 0) {
      x = compute();
      v[dev].store(x, std::memory_order_release);
    }
    return x;
  }
};

// Checked builds (-DOGS_CHECK_BOUNDS=1, for tests): every column id and row
// id a kernel loads from the maps is compared with the handle's node and row
// counts before a value is read or written through it; an id out of range
// is counted in the handle's error word and replaced by 0, so the access
// stays inside the field.  Default builds compile the checks out.
#ifndef OGS_CHECK_BOUNDS
#define OGS_CHECK_BOUNDS 0
#endif

// Rows of exact degree 1..kDmax are stored in fixed-width buckets; rows of a
// larger degree go to one general CSR bucket.
constexpr int kDmax = 8;
// Entries (row members) per work tile.  A 256-thread CTA handles one tile:
// every thread owns kTileNnz/256 = 8 entries, i.e. 8/d rows of degree d.
constexpr int kBlock = 256;
constexpr int kTileNnz = 2048;
constexpr int kEntriesPerThread = kTileNnz / kBlock;
// General-bucket tiles hold at most one row per thread.
constexpr int kGeneralRowsPerTile = kBlock;
// Slices of the host-buffer pipeline (ogs_gather_scatter_host) and whether
// the pipeline is captured into a CUDA graph and replayed on later calls with
// the same host buffer.
#ifndef OGS_HOST_PHASES
#define OGS_HOST_PHASES 8
#endif
#ifndef OGS_HOST_GRAPH
#define OGS_HOST_GRAPH 0
#endif
// With 6 or more slices, the first and last two take 1/4 and 1/2 of the
// others' share of tiles: the first copy in and the last copy out run with
// nothing beside them, so they are kept short.
#ifndef OGS_HOST_TAPER
#define OGS_HOST_TAPER 1
#endif
// Separate arrays handled by one launch of the *_many entry points.
constexpr int kMaxMany = 16;
// Member entries per lane of a warp tile (ogs_warp.cuh): lane l owns
// kWarpEntries/d rows of degree d (at least one); the per-lane arrays hold up
// to kWarpSlots entries.
#ifndef OGS_WARP_ENTRIES
#define OGS_WARP_ENTRIES 8
#endif
constexpr int kWarpEntries = OGS_WARP_ENTRIES;
constexpr int kWarpSlots = kWarpEntries > kDmax ? kWarpEntries : kDmax;

// Rows of degree d that one thread handles in a tile (at least one).
OGS_HD inline constexpr int rows_per_thread(int d) {
  return (kEntriesPerThread / d) > 0 ? (kEntriesPerThread / d) : 1;
}
OGS_HD inline constexpr int rows_per_tile(int d) {
  return d >= 1 && d <= kDmax ? kBlock * rows_per_thread(d) : kGeneralRowsPerTile;
}
OGS_HD inline constexpr int warp_rows_per_lane(int d) {
  return (kWarpEntries / d) > 0 ? (kWarpEntries / d) : 1;
}
OGS_HD inline constexpr int warp_rows_per_tile(int d) { return 32 * warp_rows_per_lane(d); }

// One bucket of rows of exact degree d, rows in ascending row order.
// Arrays are padded (stride = n rounded up to 4 rows, masks to 16 bytes) so
// that every tile's chunk starts on a 16-byte boundary and may be copied with
// its length rounded up, as the bulk (TMA) copies require.
struct DevBucket {
  const int32_t* cols;   // [d][stride]: member j of bucket row i at cols[j*stride + i]
  const int32_t* rows;   // [stride] row ids (ascending)
  const uint8_t* nmask;  // [stride rounded to 16] bit j: member j is in the N map (Signed only)
  int32_t n;             // rows in the bucket
  int32_t nP;            // rows with row id < NrowsN, a prefix of the bucket
  int32_t stride;        // n rounded up to a multiple of 4
  int32_t nnodes;        // local nodes: column ids lie in [0, nnodes)
  int32_t nrows;         // rows of the T map: row ids lie in [0, nrows)
  unsigned int* err;     // ids found out of range (checked builds); may be null
};

// Rows of degree > kDmax, CSR relative to the bucket.
struct DevGeneral {
  const int32_t* rows;     // [n]
  const int32_t* startsT;  // [n+1]
  const int32_t* colsT;
  const int32_t* startsN;  // [n+1] (alias startsT when Unsigned)
  const int32_t* colsN;
  int32_t n, nP;
  int32_t nnodes, nrows;   // as in DevBucket
  unsigned int* err;
};

// A tile: `count` consecutive rows of one bucket, starting at `begin`.
// bucket 0 = general, 1..kDmax = exact degree.  Tiles are ordered by the row
// id of their first row so that concurrently running CTAs touch nearby nodes.
struct Tile {
  int32_t bucket;
  int32_t begin;
  int32_t count;
  int32_t first_row;
};

// One warp tile as a self-contained 32-byte record, for launches that walk
// the tiles of several meshes (ogs_batch.cuh).
struct WarpRec {
  const int32_t* cols;   // the bucket's column ids (member q of row i at cols[q*stride + i])
  const int32_t* rows;   // the bucket's row ids
  int32_t begin;         // first bucket row of the tile
  int32_t bucket_count;  // degree << 16 | rows in the tile
  int32_t stride;        // the bucket's stride
  int32_t nP;            // bucket rows below NrowsN
};
static_assert(sizeof(WarpRec) == 32, "WarpRec is 32 bytes");

// One entry of a batched launch, in device memory.
struct BatchEntry {
  const WarpRec* recs;     // the handle's warp records
  const uint8_t* wemask;   // the handle's per-lane N masks (Signed only)
  void* v;                 // field, K interleaved components per node
  int32_t K, op;
  int32_t gather_n, scatter_n, limit_n, use_mask;
  uint32_t kmagic;         // ceil(2^32 / K) for 1 < K < 11585 (division by K as a multiply-high), else 0
  int32_t reserved;
};
// The multiply-high divisor of a batch entry's K: floor(u / K) ==
// umulhi(u, ceil(2^32 / K)) for every u < 32 K when (32 K) K < 2^32.
inline bool batch_plain(const BatchEntry& e) {
  return !e.gather_n && !e.scatter_n && !e.limit_n && !e.use_mask;
}
inline uint32_t batch_kmagic(int K) { return K > 1 && K < 11585 ? 0xFFFFFFFFu / static_cast<uint32_t>(K) + 1u : 0u; }
// Work items of a batched launch: each (warp record, component) pair of each
// entry; starts[e] = first item of entry e, records of an entry in order with
// their K components adjacent.


struct DevMaps {
  DevBucket b[kDmax + 1];  // b[0] unused
  DevGeneral g;
  const Tile* tiles;       // CTA tiles of every bucket, ordered by first row (direct kernel)
  int32_t ntiles;
  int32_t signed_maps;     // N maps differ from T maps
  int32_t ngtiles;         // general-bucket CTA tiles, ordered by first row
  const Tile* gtiles;
  const Tile* wtiles;      // exact-degree warp tiles (ogs_warp.cuh), ordered by first row
  const uint8_t* wemask;   // [nwtiles][32] per-lane entry masks of the N map (Signed only)
  int32_t nwtiles;
  const WarpRec* wrecs;    // [nwtiles] the warp tiles as records (batched launches)
};

// Which members take part, per ogsOperator.cpp:60-97, 206-238, 311-360.
struct Pattern {
  int32_t gather_n;   // fold only members of the N map
  int32_t scatter_n;  // 1: write only members of the N map; 2: those, or member 0
                      //    when the row has none (gslib transpose 1)
  int32_t limit_n;    // process rows < NrowsN only
  int32_t gslib = 0;  // gslib rules: fold from the first member taking part,
                      //    integer Max starting at INT_MIN (gs_defs.h:44-52)
};

enum Mode : int { kModeGS = 0, kModeGather = 1, kModeScatter = 2 };

// Field operands of one launch.  Interleaved: component c of node n at
// base[0][c + n*K].  Many: component c of node n at base[c][n].
struct FieldArgs {
  void* v;                  // interleaved local vector (GS, Gather input, Scatter output)
  void* gv;                 // interleaved gathered vector (Gather output, Scatter input)
  void* many[kMaxMany];     // separate arrays (GS many)
  int32_t K;
  int32_t is_many;
};

// A slice of the warp and general tiles for the host-buffer pipeline: its
// kernels read and write local nodes in [lo, hi]; its host->device chunk is
// [h0, h1) and once it has run, local nodes [d0, d1) are final and go back.
struct Phase {
  int32_t w0, w1;  // warp tiles
  int32_t g0, g1;  // general tiles
  int64_t lo, hi;
  int64_t h0, h1, d0, d1;
  // rows: the gathered vector's rows [r0, r1) are final once this slice has
  // run (no later slice writes a row below r1); rows [0, rn) hold every row
  // this slice or an earlier one reads (host-buffer Gather and Scatter)
  int64_t r0, r1, rn;
};

// Host-side copy of everything built at setup.
struct HostLayout {
  std::vector<int32_t> cols[kDmax + 1];
  std::vector<int32_t> rows[kDmax + 1];
  std::vector<uint8_t> nmask[kDmax + 1];
  int32_t nP[kDmax + 1] = {0};
  int32_t n[kDmax + 1] = {0};
  std::vector<int32_t> g_rows, g_startsT, g_colsT, g_startsN, g_colsN;
  int32_t g_nP = 0;
  std::vector<Tile> tiles;   // CTA tiles, all buckets, by first row
  std::vector<Tile> gtiles;  // general CTA tiles, by first row
  std::vector<Tile> wtiles;  // exact-degree warp tiles, by first row
  std::vector<uint8_t> wemask;
  std::vector<Phase> phases;
  int64_t g_n = 0, g_nnzT = 0;  // general-bucket rows and T entries
  // lowest and highest local node each warp tile / general tile touches
  std::vector<int64_t> wlo, whi, glo, ghi;
};

}  // namespace ogsgb

struct ogs_handle_s {
  int64_t N = 0;
  int kind = 0;
  int unique = 0;
  int gather_defined = 0;
  int64_t NlocalP = 0, NlocalT = 0, Ngather = 0, NgatherGlobal = 0;
  int64_t nnzT = 0, nnzN = 0;
  int32_t max_degree = 0;
  bool host_only = false;
  bool covers_all = false;  // every local node is in the T map (no zero ids)
  bool gslib = false;       // maps in gslib's member order (ogs_gslib.cpp)
  bool from_maps = false;   // an operator over caller-built maps (ogs_maps.cpp)
  bool distinct_cols = true;  // no local node in two rows (GatherScatter/Scatter need it)

  std::vector<int32_t> rowStartsT, colIdsT, rowStartsN, colIdsN;  // N empty when Unsigned
  ogsgb::HostLayout lay;

  int device = -1;
  void* arena = nullptr;  // one device allocation for all maps
  size_t arena_bytes = 0;
  ogsgb::DevMaps dmaps{};

  std::mutex host_mu;     // serialises the _host entry points (they share `stage`)
  void* stage = nullptr;  // device staging for the _host entry points
  size_t stage_bytes = 0;
  void* copy_in = nullptr;   // cudaStream_t: host->device chunks of the host pipeline
  void* copy_out = nullptr;  // cudaStream_t: device->host chunks
  void* capture = nullptr;   // cudaStream_t: the pipeline is captured on it
  std::vector<void*> events; // cudaEvent_t: [0] start, 2 per phase, then 2 joins
  struct HostGraph {         // captured host-buffer pipelines, most recent first
    void* host;
    int k, type, op, trans;
    void* exec;              // cudaGraphExec_t
  };
  std::vector<HostGraph> host_graphs;
};

namespace ogsgb {

// Host setup (ogs_setup.cpp).
ogs_status build_host_maps(ogs_handle_s* h, int64_t N, int64_t* ids, int kind, int unique);
// The same maps built on the current device (ogs_dsetup.cu).
ogs_status build_device_maps(ogs_handle_s* h, int64_t N, int64_t* ids, int kind, int unique, bool layout);
void build_layout(ogs_handle_s* h);
ogs_status upload_layout(ogs_handle_s* h);
void release_device(ogs_handle_s* h);
void build_phases(ogs_handle_s* h, int max_phases);  // needs the tiles and their lo/hi
// The maps' layout built on the current device from device CSR maps
// (ogs_dsetup.cu): the arena, DevMaps and the host-side tile lists and phases.
ogs_status build_device_layout(ogs_handle_s* h, const int32_t* d_rsT, const int32_t* d_ciT, const int32_t* d_rsN,
                               const int32_t* d_ciN, void* stream);
// DevMaps restricted to the tiles of one phase.
DevMaps phase_maps(const DevMaps& m, const Phase& p);
// The id ranges and error word of every bucket (both setup paths).
void set_id_bounds(const ogs_handle_s* h, DevMaps& m, unsigned int* err);

// Per-type launchers (ogs_kern_*.cu).  Return a cudaError_t value.  k = 1
// interleaved fields take the pipelined kernel over the exact-degree tiles
// plus the direct kernel over the general tiles; every other case runs the
// direct kernel over all tiles.
int launch_f32(const DevMaps& m, const FieldArgs& f, int mode, int op, Pattern pat, void* stream);
int launch_f64(const DevMaps& m, const FieldArgs& f, int mode, int op, Pattern pat, void* stream);
int launch_i32(const DevMaps& m, const FieldArgs& f, int mode, int op, Pattern pat, void* stream);
int launch_i64(const DevMaps& m, const FieldArgs& f, int mode, int op, Pattern pat, void* stream);

// Batched launch over `n` entries (ogs_batch.cuh); grid <= 0 = one full wave;
// block = 128 or 256 threads per CTA; occ = 2 or 3 (register budget: 256-thread
// CTAs per SM); pipe = 0 register pipeline, 1 cp.async ring (256 threads);
// plain = 1 when no entry has N masks, a store mode or a row limit
// (batch_plain), which selects kernels without those branches.
int launch_batch_f32(const BatchEntry* E, const int64_t* starts, int n, int64_t nitems, int grid, int block,
                     int occ, int pipe, int plain, void* stream);
int launch_batch_f64(const BatchEntry* E, const int64_t* starts, int n, int64_t nitems, int grid, int block,
                     int occ, int pipe, int plain, void* stream);
int launch_batch_i32(const BatchEntry* E, const int64_t* starts, int n, int64_t nitems, int grid, int block,
                     int occ, int pipe, int plain, void* stream);
int launch_batch_i64(const BatchEntry* E, const int64_t* starts, int n, int64_t nitems, int grid, int block,
                     int occ, int pipe, int plain, void* stream);

// Device and page-locked host allocations (ogs_alloc.cpp): counted, and made
// to fail on demand by ogs_debug_fail_alloc.  Every allocation of the library
// goes through these.
cudaError_t dev_malloc_raw(void** p, size_t bytes);
void dev_free(void* p);
cudaError_t host_malloc_raw(void** p, size_t bytes);
void host_free(void* p);
template <typename T>
inline cudaError_t dev_malloc(T** p, size_t bytes) {
  return dev_malloc_raw(reinterpret_cast<void**>(p), bytes);
}
template <typename T>
inline cudaError_t host_malloc(T** p, size_t bytes) {
  return host_malloc_raw(reinterpret_cast<void**>(p), bytes);
}

// Load the batched kernel the server launches (256 threads, 2 CTAs per SM)
// ahead of its first use.
int preload_batch_f32();
int preload_batch_f64();
int preload_batch_i32();
int preload_batch_i64();

// Thread-local error message (ogs_capi.cpp).
ogs_status set_error(ogs_status s, const std::string& msg);

// Argument checks and member patterns shared by the entry points (ogs_capi.cpp).
size_t type_size(int type);
// handle usable on the current device, k >= 1, known type and transpose; refuses
// host-only handles and handles made by ogs_gslib_setup
ogs_status check_common(ogs_handle h, int k, int type, int trans, const char* fn);
// GatherScatter and Scatter write every member: no local node in two rows
ogs_status check_writes(ogs_handle h, const char* fn);
ogs_status check_op(int op, const char* fn);
// members read and written for (kind, mode, transpose), ogsOperator.cpp:71-79, 214-222, 321-339
Pattern pattern_for(const ogs_handle_s* h, int mode, int trans);

}  // namespace ogsgb
