// ogs_maps.cpp -- operators over caller-built CSR maps.
//
// The reference builds three operators of one class from its maps:
// gatherLocal, gatherHalo and the exchange's postmpi (ogsOperator_t,
// libs/ogs/ogsOperator.hpp:40-120; postmpi in ogsAllToAll.cpp:255-331).  The
// multi-rank setup that produces the halo and postmpi maps is the MPI layer;
// ogs_setup_maps takes such maps from the caller and returns a handle whose
// Gather, Scatter and GatherScatter run on the library's kernels.
//
// The T map is required.  An N map, when given, has a row-start entry for
// every T row; rows at and above NrowsN must be empty, and each row's N
// members are a subsequence of its T members in the same order (true of the
// reference's local and halo maps, and of postmpi's when every received
// entry is positive; a caller with other N maps makes a second operator with
// them as its T map).  NULL N maps make N = T.
#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "ogs_internal.hpp"

using namespace ogsgb;

namespace {

ogs_status check_map(const char* which, int64_t N, int64_t rows, const int32_t* rs, const int32_t* ci) {
  const std::string fn = std::string("ogs_setup_maps: ") + which;
  if (!rs) return set_error(OGS_EINVAL, fn + " rowStarts is NULL");
  if (rs[0] != 0) return set_error(OGS_EINVAL, fn + " rowStarts[0] != 0");
  for (int64_t r = 0; r < rows; ++r)
    if (rs[r + 1] < rs[r]) return set_error(OGS_EINVAL, fn + " rowStarts decreases at row " + std::to_string(r));
  const int64_t nnz = rs[rows];
  if (nnz > 0 && !ci) return set_error(OGS_EINVAL, fn + " colIds is NULL");
  for (int64_t e = 0; e < nnz; ++e)
    if (ci[e] < 0 || ci[e] >= N)
      return set_error(OGS_ERANGE, fn + " colIds[" + std::to_string(e) + "] = " + std::to_string(ci[e]) +
                                       " is outside [0, N)");
  return OGS_OK;
}

}  // namespace

extern "C" ogs_status ogs_setup_maps(ogs_handle* out, int64_t N, int64_t NrowsN, int64_t NrowsT,
                                     const int32_t* rowStartsN, const int32_t* colIdsN, const int32_t* rowStartsT,
                                     const int32_t* colIdsT, unsigned flags) {
  if (!out) return set_error(OGS_EINVAL, "ogs_setup_maps: out is NULL");
  *out = nullptr;
  if (N < 0 || NrowsT < 0) return set_error(OGS_EINVAL, "ogs_setup_maps: N and NrowsT must be >= 0");
  if (N > INT32_MAX || NrowsT > INT32_MAX)
    return set_error(OGS_ERANGE, "ogs_setup_maps: sizes exceed 32-bit device indices");
  if (flags & OGS_SETUP_DEVICE_MAPS) return set_error(OGS_EINVAL, "ogs_setup_maps: the maps are given, not built");
  const bool sgn = rowStartsN != nullptr;
  if (!sgn) NrowsN = NrowsT;
  if (NrowsN < 0 || NrowsN > NrowsT) return set_error(OGS_EINVAL, "ogs_setup_maps: NrowsN must lie in [0, NrowsT]");
  ogs_status s = check_map("T map", N, NrowsT, rowStartsT, colIdsT);
  if (s != OGS_OK) return s;
  if (sgn && (s = check_map("N map", N, NrowsT, rowStartsN, colIdsN)) != OGS_OK) return s;
  ogs_handle_s* h = new (std::nothrow) ogs_handle_s();
  if (!h) return set_error(OGS_ENOMEM, "ogs_setup_maps: out of host memory");
  try {
    h->N = N;
    h->kind = sgn ? OGS_SIGNED : OGS_UNSIGNED;
    h->unique = 0;
    h->from_maps = true;
    h->gather_defined = 1;  // an operator has no well-definedness check (ogs_t has, ogsSetup.cpp:861-864)
    h->NlocalT = NrowsT;
    h->NlocalP = NrowsN;
    h->Ngather = h->NgatherGlobal = NrowsN;
    h->rowStartsT.assign(rowStartsT, rowStartsT + NrowsT + 1);
    h->nnzT = h->rowStartsT[NrowsT];
    h->colIdsT.assign(colIdsT, colIdsT + h->nnzT);
    int32_t maxd = 0;
    for (int64_t r = 0; r < NrowsT; ++r) maxd = std::max(maxd, h->rowStartsT[r + 1] - h->rowStartsT[r]);
    h->max_degree = maxd;
    // every column at most once: GatherScatter and Scatter write each member
    std::vector<uint8_t> seen(static_cast<size_t>(N), 0);
    bool distinct = true;
    for (int32_t c : h->colIdsT) {
      if (seen[c]) { distinct = false; break; }
      seen[c] = 1;
    }
    h->distinct_cols = distinct;
    h->covers_all = distinct && h->nnzT == N;
    if (sgn) {
      h->rowStartsN.assign(rowStartsN, rowStartsN + NrowsT + 1);
      h->nnzN = h->rowStartsN[NrowsT];
      h->colIdsN.assign(colIdsN, colIdsN + h->nnzN);
      for (int64_t r = 0; r < NrowsT; ++r) {
        const int32_t n0 = h->rowStartsN[r], n1 = h->rowStartsN[r + 1];
        if (r >= NrowsN && n1 > n0) {
          delete h;
          return set_error(OGS_EINVAL, "ogs_setup_maps: N map row " + std::to_string(r) + " at or above NrowsN is not empty");
        }
        int32_t q = n0;
        for (int32_t t = h->rowStartsT[r]; t < h->rowStartsT[r + 1] && q < n1; ++t)
          if (h->colIdsT[t] == h->colIdsN[q]) q++;
        if (q != n1) {
          delete h;
          return set_error(OGS_EINVAL, "ogs_setup_maps: N map row " + std::to_string(r) +
                                           " is not a subsequence of T map row " + std::to_string(r));
        }
      }
    } else {
      h->nnzN = h->nnzT;
    }
    build_layout(h);
    h->host_only = (flags & OGS_SETUP_HOST_ONLY) != 0;
    if (!h->host_only) {
      s = upload_layout(h);
      if (s != OGS_OK) { release_device(h); delete h; return s; }
      const cudaError_t e = cudaDeviceSynchronize();
      if (e != cudaSuccess) {
        release_device(h);
        delete h;
        return set_error(OGS_EDEVICE, std::string("ogs_setup_maps: synchronize: ") + cudaGetErrorString(e));
      }
    }
  } catch (const std::bad_alloc&) {
    release_device(h);
    delete h;
    return set_error(OGS_ENOMEM, "ogs_setup_maps: out of host memory");
  }
  *out = h;
  return OGS_OK;
}
