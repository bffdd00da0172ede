// ogs_internal.hpp -- shared definitions of the GB300 gather-scatter library:
// the device layout of one mesh's maps, the work tiles, and the launch
// interface between the C ABI (ogs_capi.cpp) and the per-type kernel units
// (ogs_kern_*.cu).
#pragma once

#include <cstdint>
#include <string>
#include <vector>

#include "ogs_c.h"

#ifdef __CUDACC__
#define OGS_HD __host__ __device__
#else
#define OGS_HD
#endif

namespace ogsgb {

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
// Separate arrays handled by one launch of the *_many entry points.
constexpr int kMaxMany = 16;

// Rows of degree d that one thread handles in a tile (at least one).
OGS_HD inline constexpr int rows_per_thread(int d) {
  return (kEntriesPerThread / d) > 0 ? (kEntriesPerThread / d) : 1;
}
OGS_HD inline constexpr int rows_per_tile(int d) {
  return d >= 1 && d <= kDmax ? kBlock * rows_per_thread(d) : kGeneralRowsPerTile;
}

// One bucket of rows of exact degree d, rows in ascending row order.
struct DevBucket {
  const int32_t* cols;   // [d][n]: member j of bucket row i at cols[j*n + i]
  const int32_t* rows;   // [n] row ids (ascending)
  const uint8_t* nmask;  // [n] bit j set when member j is in the N map (Signed only)
  int32_t n;             // rows in the bucket
  int32_t nP;            // rows with row id < NrowsN, a prefix of the bucket
};

// Rows of degree > kDmax, CSR relative to the bucket.
struct DevGeneral {
  const int32_t* rows;     // [n]
  const int32_t* startsT;  // [n+1]
  const int32_t* colsT;
  const int32_t* startsN;  // [n+1] (alias startsT when Unsigned)
  const int32_t* colsN;
  int32_t n, nP;
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

struct DevMaps {
  DevBucket b[kDmax + 1];  // b[0] unused
  DevGeneral g;
  const Tile* tiles;
  int32_t ntiles;
  int32_t signed_maps;     // N maps differ from T maps
};

// Which members take part, per ogsOperator.cpp:60-97, 206-238, 311-360.
struct Pattern {
  int32_t gather_n;   // fold only members of the N map
  int32_t scatter_n;  // write only members of the N map
  int32_t limit_n;    // process rows < NrowsN only
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

// Host-side copy of everything built at setup.
struct HostLayout {
  std::vector<int32_t> cols[kDmax + 1];
  std::vector<int32_t> rows[kDmax + 1];
  std::vector<uint8_t> nmask[kDmax + 1];
  int32_t nP[kDmax + 1] = {0};
  std::vector<int32_t> g_rows, g_startsT, g_colsT, g_startsN, g_colsN;
  int32_t g_nP = 0;
  std::vector<Tile> tiles;
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

  std::vector<int32_t> rowStartsT, colIdsT, rowStartsN, colIdsN;  // N empty when Unsigned
  ogsgb::HostLayout lay;

  int device = -1;
  void* arena = nullptr;  // one device allocation for all maps
  size_t arena_bytes = 0;
  ogsgb::DevMaps dmaps{};

  void* stage = nullptr;  // device staging for the _host entry points
  size_t stage_bytes = 0;
};

namespace ogsgb {

// Host setup (ogs_setup.cpp).
ogs_status build_host_maps(ogs_handle_s* h, int64_t N, int64_t* ids, int kind, int unique);
void build_layout(ogs_handle_s* h);
ogs_status upload_layout(ogs_handle_s* h);
void release_device(ogs_handle_s* h);

// Per-type launchers (ogs_kern_*.cu).  Return a cudaError_t value.
int launch_f32(const DevMaps& m, const FieldArgs& f, int mode, int op, Pattern pat, void* stream);
int launch_f64(const DevMaps& m, const FieldArgs& f, int mode, int op, Pattern pat, void* stream);
int launch_i32(const DevMaps& m, const FieldArgs& f, int mode, int op, Pattern pat, void* stream);
int launch_i64(const DevMaps& m, const FieldArgs& f, int mode, int op, Pattern pat, void* stream);

// Thread-local error message (ogs_capi.cpp).
ogs_status set_error(ogs_status s, const std::string& msg);

}  // namespace ogsgb
