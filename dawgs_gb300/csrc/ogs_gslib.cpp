// ogs_gslib.cpp -- gslib-compatible entry points (C ABI part of ogs_c.h).
//
// gslib is the gather-scatter library that dawgs vendors (3rdParty/gslib) and
// uses as its correctness reference (dawgsGS.cpp:34-105).  Its single-rank
// local step (gs.c:1172-1188 with the maps of gs.c:85-125, 333-375) differs
// from ogs in a few rules, all reproduced here on the same kernels:
//  * ids < 0 are "flagged"; each id group lists its unflagged members first,
//    then the flagged ones, each in ascending local index, and folds in that
//    order starting from the first member's own value (gs_local.c:58-72), not
//    from an identity;
//  * transpose 0: fold the unflagged members; a group with none gets the
//    identity (integer Max: INT_MIN, gs_defs.h:48-52); every member receives
//    the result;
//  * transpose 1: fold all members; the first member and the other unflagged
//    members receive the result, flagged ones keep their values;
//  * a lone unflagged member is left as it is.
// Setup stores each row's members in gslib's order; the kernels' gslib mode
// folds from the first member and, for transpose 1, writes the unflagged
// members or, in a row without any, member 0.
#include <algorithm>
#include <new>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "ogs_internal.hpp"

using namespace ogsgb;

namespace ogsgb {
namespace {

// Reorder every T row to [N members ascending, other members ascending].
void gslib_order(ogs_handle_s* h) {
  std::vector<int32_t> out(h->colIdsT.size());
  for (int64_t r = 0; r < h->NlocalT; ++r) {
    const int32_t t0 = h->rowStartsT[r], t1 = h->rowStartsT[r + 1];
    const int32_t n0 = h->rowStartsN[r], n1 = h->rowStartsN[r + 1];
    int32_t w = t0, q = n0;
    for (int32_t i = n0; i < n1; ++i) out[w++] = h->colIdsN[i];
    for (int32_t i = t0; i < t1; ++i) {
      if (q < n1 && h->colIdsN[q] == h->colIdsT[i]) { q++; continue; }
      out[w++] = h->colIdsT[i];
    }
  }
  h->colIdsT.swap(out);
}

ogs_status check_gs(ogs_handle h, int vn, int dom, int op, int transpose, const char* fn) {
  if (!h) return set_error(OGS_EINVAL, std::string(fn) + ": handle is NULL");
  if (!h->gslib) return set_error(OGS_EINVAL, std::string(fn) + ": handle was not made by ogs_gslib_setup");
  if (h->host_only) return set_error(OGS_EINVAL, std::string(fn) + ": handle was set up host-only");
  if (vn < 1) return set_error(OGS_EINVAL, std::string(fn) + ": vn must be >= 1");
  if (dom < OGS_FLOAT || dom > OGS_INT64) return set_error(OGS_EINVAL, std::string(fn) + ": unknown domain");
  if (op < OGS_ADD || op > OGS_MIN) return set_error(OGS_EINVAL, std::string(fn) + ": unknown op");
  if (transpose != 0 && transpose != 1) return set_error(OGS_EINVAL, std::string(fn) + ": transpose must be 0 or 1");
  int dev = -1;
  const cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return set_error(OGS_EDEVICE, std::string(fn) + ": " + cudaGetErrorString(e));
  if (h->N > 0 && dev != h->device) return set_error(OGS_EINVAL, std::string(fn) + ": handle lives on another device");
  return OGS_OK;
}

Pattern gs_pattern(int transpose) {
  Pattern p{0, 0, 0};
  if (transpose == 0) p = Pattern{1, 0, 0};
  else p = Pattern{0, 2, 0};
  p.gslib = 1;
  return p;
}

ogs_status run(ogs_handle h, const FieldArgs& f, int dom, int op, int transpose, void* stream, const char* fn) {
  int e = 0;
  const Pattern pat = gs_pattern(transpose);
  switch (dom) {
    case OGS_FLOAT: e = launch_f32(h->dmaps, f, kModeGS, op, pat, stream); break;
    case OGS_DOUBLE: e = launch_f64(h->dmaps, f, kModeGS, op, pat, stream); break;
    case OGS_INT32: e = launch_i32(h->dmaps, f, kModeGS, op, pat, stream); break;
    default: e = launch_i64(h->dmaps, f, kModeGS, op, pat, stream); break;
  }
  if (e) return set_error(OGS_EDEVICE, std::string(fn) + ": kernel launch failed: " +
                                         cudaGetErrorString(static_cast<cudaError_t>(e)));
  return OGS_OK;
}

}  // namespace
}  // namespace ogsgb

extern "C" {

ogs_status ogs_gslib_setup(ogs_handle* out, const int64_t* ids, int64_t n, unsigned flags) {
  if (!out) return set_error(OGS_EINVAL, "ogs_gslib_setup: out is NULL");
  *out = nullptr;
  if (n > 0 && !ids) return set_error(OGS_EINVAL, "ogs_gslib_setup: ids is NULL");
  ogs_handle_s* h = new (std::nothrow) ogs_handle_s();
  if (!h) return set_error(OGS_ENOMEM, "ogs_gslib_setup: out of host memory");
  try {
    std::vector<int64_t> copy(ids, ids + (n > 0 ? n : 0));
    ogs_status s = build_host_maps(h, n, copy.data(), OGS_SIGNED, 0);
    if (s != OGS_OK) { delete h; return s; }
    gslib_order(h);
    h->gslib = true;
    build_layout(h);
    h->host_only = (flags & OGS_SETUP_HOST_ONLY) != 0;
    if (!h->host_only) {
      s = upload_layout(h);
      if (s != OGS_OK) { release_device(h); delete h; return s; }
    }
  } catch (const std::bad_alloc&) {
    release_device(h);
    delete h;
    return set_error(OGS_ENOMEM, "ogs_gslib_setup: out of host memory");
  }
  *out = h;
  return OGS_OK;
}

ogs_status ogs_gslib_gs_vec(ogs_handle h, void* d_u, int vn, int dom, int op, int transpose, void* stream) {
  const char* fn = "ogs_gslib_gs_vec";
  ogs_status s = check_gs(h, vn, dom, op, transpose, fn);
  if (s != OGS_OK) return s;
  if (h->N == 0) return OGS_OK;
  if (!d_u) return set_error(OGS_EINVAL, "ogs_gslib_gs_vec: u is NULL");
  FieldArgs f{};
  f.v = d_u;
  f.K = vn;
  return run(h, f, dom, op, transpose, stream, fn);
}

ogs_status ogs_gslib_gs(ogs_handle h, void* d_u, int dom, int op, int transpose, void* stream) {
  return ogs_gslib_gs_vec(h, d_u, 1, dom, op, transpose, stream);
}

ogs_status ogs_gslib_gs_many(ogs_handle h, void* const* d_us, int vn, int dom, int op, int transpose, void* stream) {
  const char* fn = "ogs_gslib_gs_many";
  ogs_status s = check_gs(h, vn, dom, op, transpose, fn);
  if (s != OGS_OK) return s;
  if (h->N == 0) return OGS_OK;
  if (!d_us) return set_error(OGS_EINVAL, "ogs_gslib_gs_many: us is NULL");
  for (int k0 = 0; k0 < vn; k0 += kMaxMany) {
    FieldArgs f{};
    f.is_many = 1;
    f.K = (vn - k0 < kMaxMany) ? (vn - k0) : kMaxMany;
    for (int j = 0; j < f.K; ++j) {
      if (!d_us[k0 + j]) return set_error(OGS_EINVAL, "ogs_gslib_gs_many: a field pointer is NULL");
      f.many[j] = d_us[k0 + j];
    }
    if ((s = run(h, f, dom, op, transpose, stream, fn)) != OGS_OK) return s;
  }
  return OGS_OK;
}

}  // extern "C"
