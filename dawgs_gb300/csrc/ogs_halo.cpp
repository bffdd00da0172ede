// ogs_halo.cpp -- halo_t: Exchange and Combine of the halo rows (ogs_c.h).
//
// The reference's halo_t (include/ogs.hpp:346-397, libs/ogs/ogsHalo.cpp:39-359)
// runs, around its MPI exchange object:
//   ExchangeStart   haloBuf[0, NhaloP) <- Gather(v, Add, NoTrans) over the
//                   gatherHalo maps (or, for a halo made from a gather, a copy
//                   of the gathered vector's rows NlocalT..NlocalT+NhaloP);
//                   exchange->Start(haloBuf, k, Add, NoTrans)
//   ExchangeFinish  exchange->Finish(...), then v <- Scatter(haloBuf, NoTrans)
//                   (or a copy of rows NhaloP..NhaloT back behind the owned rows)
//   CombineStart    haloBuf[0, NhaloT) <- Gather(v, Add, Trans); exchange->Start(.., Trans)
//   CombineFinish   exchange->Finish(.., Trans); v <- Scatter(haloBuf, Trans)
// The gathers, scatters and copies run here on the library's kernels, on the
// caller's stream.  The exchange object -- MPI, or anything that moves the
// halo buffer between ranks -- is the caller's, passed in as start/finish
// callbacks; the device packing and post-exchange folding it needs are
// ogs_extract and operators from ogs_setup_maps.  At one rank a halo has no
// rows and the exchange has nothing to move, as in the reference.
//
// The halo buffer is reserved once per (k, type) size and owned by the handle
// (the reference allocates it in every Start, ogsHalo.cpp:47); a lock in the
// handle serialises the calls that use it.
#include <mutex>
#include <new>
#include <string>
#include <unordered_map>

#include <cuda_runtime.h>

#include "ogs_internal.hpp"
#include "ogs_trace.hpp"

using namespace ogsgb;

struct ogs_halo_s {
  int64_t N = 0, NlocalT = 0, NhaloP = 0, NhaloT = 0, Nrecv = 0;
  bool gathered = false;
  ogs_handle op = nullptr;  // gatherHalo (halos from maps with rows)
  std::mutex mu;
  void* buf = nullptr;      // k * (NhaloT + Nrecv) values
  size_t buf_bytes = 0;
  void* stage = nullptr;    // the field, for the host-buffer forms
  size_t stage_bytes = 0;
};

namespace {

ogs_status cuda_st(cudaError_t e, const char* fn, const char* what) {
  if (e == cudaSuccess) return OGS_OK;
  cudaGetLastError();
  return set_error(e == cudaErrorMemoryAllocation ? OGS_ENOMEM : OGS_EDEVICE,
                   std::string(fn) + ": " + what + ": " + cudaGetErrorString(e));
}

ogs_status check_args(ogs_halo h, int k, int type, const char* fn) {
  if (!h) return set_error(OGS_EINVAL, std::string(fn) + ": halo is NULL");
  if (k < 1) return set_error(OGS_EINVAL, std::string(fn) + ": k must be >= 1");
  if (type < OGS_FLOAT || type > OGS_INT64) return set_error(OGS_EINVAL, std::string(fn) + ": unknown type");
  return OGS_OK;
}

// (re)allocate a device block of at least `bytes` (h->mu held)
ogs_status grow(void** p, size_t* have, size_t bytes, const char* fn, const char* what) {
  if (bytes <= *have) return OGS_OK;
  dev_free(*p);
  *p = nullptr;
  *have = 0;
  ogs_status s = cuda_st(dev_malloc(p, bytes), fn, what);
  if (s == OGS_OK) *have = bytes;
  return s;
}

ogs_status reserve_locked(ogs_halo h, int k, int type, const char* fn) {
  const size_t rows = static_cast<size_t>(h->NhaloT + h->Nrecv);
  if (rows == 0) return OGS_OK;
  return grow(&h->buf, &h->buf_bytes, rows * static_cast<size_t>(k) * type_size(type), fn, "halo buffer");
}

ogs_status run_exchange(const ogs_exchange* x, bool start, ogs_halo h, int k, int type, int trans, void* stream,
                        const char* fn) {
  if (!x) return OGS_OK;
  ogs_exchange_fn f = start ? x->start : x->finish;
  if (!f) return OGS_OK;
  const ogs_status s = f(x->user, h->buf, k, type, trans, stream);
  if (s != OGS_OK)
    return set_error(s, std::string(fn) + ": the exchange's " + (start ? "start" : "finish") + " returned " +
                            std::to_string(static_cast<int>(s)));
  return OGS_OK;
}

// The halo steps on a device field v (h->mu held).  trans: OGS_NOTRANS
// (Exchange) or OGS_TRANS (Combine).
ogs_status start_locked(ogs_halo h, void* v, int k, int type, int trans, const ogs_exchange* x, void* stream,
                        const char* fn) {
  ogs_status s = reserve_locked(h, k, type, fn);
  if (s != OGS_OK) return s;
  const size_t nb = static_cast<size_t>(k) * type_size(type);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (h->gathered) {
    const int64_t rows = trans == OGS_NOTRANS ? h->NhaloP : h->NhaloT;
    if (rows > 0 &&
        (s = cuda_st(cudaMemcpyAsync(h->buf, static_cast<char*>(v) + h->NlocalT * nb, rows * nb,
                                     cudaMemcpyDeviceToDevice, st), fn, "copy of the halo rows")) != OGS_OK)
      return s;
  } else if (h->op && (s = ogs_gather(h->op, h->buf, v, k, type, OGS_ADD, trans, stream)) != OGS_OK) {
    return s;
  }
  return run_exchange(x, true, h, k, type, trans, stream, fn);
}

ogs_status finish_locked(ogs_halo h, void* v, int k, int type, int trans, const ogs_exchange* x, void* stream,
                         const char* fn) {
  ogs_status s = reserve_locked(h, k, type, fn);
  if (s != OGS_OK) return s;
  if ((s = run_exchange(x, false, h, k, type, trans, stream, fn)) != OGS_OK) return s;
  const size_t nb = static_cast<size_t>(k) * type_size(type);
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (h->gathered) {
    // Exchange: the rows this rank does not own get their owners' values;
    // Combine: the owned rows get the sums
    char* dst = static_cast<char*>(v) + (trans == OGS_NOTRANS ? h->NlocalT + h->NhaloP : h->NlocalT) * nb;
    const char* src = static_cast<char*>(h->buf) + (trans == OGS_NOTRANS ? h->NhaloP : 0) * nb;
    const int64_t rows = trans == OGS_NOTRANS ? h->NhaloT - h->NhaloP : h->NhaloP;
    if (rows > 0)
      return cuda_st(cudaMemcpyAsync(dst, src, rows * nb, cudaMemcpyDeviceToDevice, st), fn, "copy of the halo rows");
    return OGS_OK;
  }
  if (h->op) return ogs_scatter(h->op, v, h->buf, k, type, trans, stream);
  return OGS_OK;
}

ogs_status device_call(ogs_halo h, void* d_v, int k, int type, int trans, const ogs_exchange* x, void* stream,
                       int which, const char* fn) {
  TraceRange trace(fn);
  ogs_status s = check_args(h, k, type, fn);
  if (s != OGS_OK) return s;
  if (!d_v && h->N > 0 && (h->NhaloT > 0)) return set_error(OGS_EINVAL, std::string(fn) + ": field is NULL");
  std::lock_guard<std::mutex> g(h->mu);
  if (which & 1) s = start_locked(h, d_v, k, type, trans, x, stream, fn);
  if (s == OGS_OK && (which & 2)) s = finish_locked(h, d_v, k, type, trans, x, stream, fn);
  return s;
}

// Host field: staged through the device, the whole step, copied back.
ogs_status host_call(ogs_halo h, void* v, int k, int type, int trans, const ogs_exchange* x, void* stream,
                     const char* fn) {
  TraceRange trace(fn);
  ogs_status s = check_args(h, k, type, fn);
  if (s != OGS_OK) return s;
  if (h->NhaloT == 0) {  // nothing of v is read or written; the exchange still runs
    std::lock_guard<std::mutex> g(h->mu);
    if ((s = run_exchange(x, true, h, k, type, trans, stream, fn)) != OGS_OK) return s;
    return run_exchange(x, false, h, k, type, trans, stream, fn);
  }
  if (!v) return set_error(OGS_EINVAL, std::string(fn) + ": field is NULL");
  std::lock_guard<std::mutex> g(h->mu);
  const size_t bytes = static_cast<size_t>(h->N) * static_cast<size_t>(k) * type_size(type);
  if ((s = grow(&h->stage, &h->stage_bytes, bytes, fn, "staging")) != OGS_OK) return s;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if ((s = cuda_st(cudaMemcpyAsync(h->stage, v, bytes, cudaMemcpyHostToDevice, st), fn, "copy in")) != OGS_OK)
    return s;
  if ((s = start_locked(h, h->stage, k, type, trans, x, stream, fn)) != OGS_OK) return s;
  if ((s = finish_locked(h, h->stage, k, type, trans, x, stream, fn)) != OGS_OK) return s;
  if ((s = cuda_st(cudaMemcpyAsync(v, h->stage, bytes, cudaMemcpyDeviceToHost, st), fn, "copy out")) != OGS_OK)
    return s;
  return cuda_st(cudaStreamSynchronize(st), fn, "synchronize");
}

}  // namespace

extern "C" {

ogs_status ogs_halo_setup(ogs_halo* out, int64_t N, const int64_t* ids, int method, int verbose) {
  (void)verbose;
  if (!out) return set_error(OGS_EINVAL, "ogs_halo_setup: out is NULL");
  *out = nullptr;
  if (N < 0 || (N > 0 && !ids)) return set_error(OGS_EINVAL, "ogs_halo_setup: bad N or ids");
  if (N > INT32_MAX) return set_error(OGS_ERANGE, "ogs_halo_setup: N exceeds 32-bit device indices");
  if (method < OGS_AUTO || method > OGS_ALLTOALL) return set_error(OGS_EINVAL, "ogs_halo_setup: unknown method");
  // every id group needs exactly one positive member (ogsSetup.cpp:276-288);
  // at one rank no group is shared with another rank, so the halo has no rows
  try {
    std::unordered_map<int64_t, int32_t> positives;
    positives.reserve(static_cast<size_t>(N));
    for (int64_t n = 0; n < N; ++n) {
      const int64_t id = ids[n];
      if (id == 0) continue;
      if (id == INT64_MIN) return set_error(OGS_ERANGE, "ogs_halo_setup: id -2^63 has no magnitude");
      int32_t& c = positives[id < 0 ? -id : id];
      if (id > 0) c++;
    }
    for (const auto& kv : positives)
      if (kv.second != 1)
        return set_error(OGS_EINVAL, "ogs_halo_setup: found " + std::to_string(kv.second) +
                                         " positive Ids for baseId: " + std::to_string(kv.first) + ".");
  } catch (const std::bad_alloc&) {
    return set_error(OGS_ENOMEM, "ogs_halo_setup: out of host memory");
  }
  ogs_halo h = new (std::nothrow) ogs_halo_s();
  if (!h) return set_error(OGS_ENOMEM, "ogs_halo_setup: out of host memory");
  h->N = N;
  *out = h;
  return OGS_OK;
}

ogs_status ogs_halo_setup_maps(ogs_halo* out, int64_t N, int64_t NhaloP, int64_t NhaloT, const int32_t* rowStartsN,
                               const int32_t* colIdsN, const int32_t* rowStartsT, const int32_t* colIdsT,
                               int64_t Nrecv, unsigned flags) {
  if (!out) return set_error(OGS_EINVAL, "ogs_halo_setup_maps: out is NULL");
  *out = nullptr;
  if (NhaloT < 0 || NhaloP < 0 || NhaloP > NhaloT || Nrecv < 0)
    return set_error(OGS_EINVAL, "ogs_halo_setup_maps: need 0 <= NhaloP <= NhaloT and Nrecv >= 0");
  if (NhaloT + Nrecv > INT32_MAX) return set_error(OGS_ERANGE, "ogs_halo_setup_maps: halo buffer beyond 32-bit rows");
  ogs_handle op = nullptr;
  if (NhaloT > 0) {
    const ogs_status s =
        ogs_setup_maps(&op, N, NhaloP, NhaloT, rowStartsN, colIdsN, rowStartsT, colIdsT, flags);
    if (s != OGS_OK) return s;
  } else if (N < 0) {
    return set_error(OGS_EINVAL, "ogs_halo_setup_maps: N must be >= 0");
  }
  ogs_halo h = new (std::nothrow) ogs_halo_s();
  if (!h) {
    ogs_free(op);
    return set_error(OGS_ENOMEM, "ogs_halo_setup_maps: out of host memory");
  }
  h->N = N;
  h->NhaloP = NhaloP;
  h->NhaloT = NhaloT;
  h->Nrecv = Nrecv;
  h->op = op;
  *out = h;
  return OGS_OK;
}

ogs_status ogs_halo_setup_from_gather(ogs_halo* out, int64_t NlocalT, int64_t NhaloP, int64_t NhaloT,
                                      int64_t Nrecv) {
  if (!out) return set_error(OGS_EINVAL, "ogs_halo_setup_from_gather: out is NULL");
  *out = nullptr;
  if (NlocalT < 0 || NhaloT < 0 || NhaloP < 0 || NhaloP > NhaloT || Nrecv < 0)
    return set_error(OGS_EINVAL, "ogs_halo_setup_from_gather: need counts >= 0 and NhaloP <= NhaloT");
  if (NlocalT + NhaloT > INT32_MAX || NhaloT + Nrecv > INT32_MAX)
    return set_error(OGS_ERANGE, "ogs_halo_setup_from_gather: sizes exceed 32-bit device indices");
  ogs_halo h = new (std::nothrow) ogs_halo_s();
  if (!h) return set_error(OGS_ENOMEM, "ogs_halo_setup_from_gather: out of host memory");
  h->N = NlocalT + NhaloT;  // ogsSetup.cpp:892
  h->NlocalT = NlocalT;
  h->NhaloP = NhaloP;
  h->NhaloT = NhaloT;
  h->Nrecv = Nrecv;
  h->gathered = true;
  *out = h;
  return OGS_OK;
}

ogs_status ogs_halo_free(ogs_halo h) {
  if (!h) return OGS_OK;
  ogs_free(h->op);
  dev_free(h->buf);
  dev_free(h->stage);
  delete h;
  return OGS_OK;
}

ogs_status ogs_halo_get_counts(ogs_halo h, ogs_halo_counts* out) {
  if (!h || !out) return set_error(OGS_EINVAL, "ogs_halo_get_counts: NULL argument");
  out->N = h->N;
  out->NlocalT = h->NlocalT;
  out->NhaloP = h->NhaloP;
  out->NhaloT = h->NhaloT;
  out->Nhalo = h->NhaloT - h->NhaloP;  // ogsSetup.cpp:63, 895
  out->Nrecv = h->Nrecv;
  out->gathered = h->gathered ? 1 : 0;
  return OGS_OK;
}

ogs_status ogs_halo_reserve(ogs_halo h, int k, int type, void** d_buf) {
  ogs_status s = check_args(h, k, type, "ogs_halo_reserve");
  if (s != OGS_OK) return s;
  std::lock_guard<std::mutex> g(h->mu);
  if ((s = reserve_locked(h, k, type, "ogs_halo_reserve")) != OGS_OK) return s;
  if (d_buf) *d_buf = h->buf;
  return OGS_OK;
}

ogs_status ogs_halo_exchange_start(ogs_halo h, void* d_v, int k, int type, const ogs_exchange* x, void* stream) {
  return device_call(h, d_v, k, type, OGS_NOTRANS, x, stream, 1, "ogs_halo_exchange_start");
}
ogs_status ogs_halo_exchange_finish(ogs_halo h, void* d_v, int k, int type, const ogs_exchange* x, void* stream) {
  return device_call(h, d_v, k, type, OGS_NOTRANS, x, stream, 2, "ogs_halo_exchange_finish");
}
ogs_status ogs_halo_exchange(ogs_halo h, void* d_v, int k, int type, const ogs_exchange* x, void* stream) {
  return device_call(h, d_v, k, type, OGS_NOTRANS, x, stream, 3, "ogs_halo_exchange");
}
ogs_status ogs_halo_combine_start(ogs_halo h, void* d_v, int k, int type, const ogs_exchange* x, void* stream) {
  return device_call(h, d_v, k, type, OGS_TRANS, x, stream, 1, "ogs_halo_combine_start");
}
ogs_status ogs_halo_combine_finish(ogs_halo h, void* d_v, int k, int type, const ogs_exchange* x, void* stream) {
  return device_call(h, d_v, k, type, OGS_TRANS, x, stream, 2, "ogs_halo_combine_finish");
}
ogs_status ogs_halo_combine(ogs_halo h, void* d_v, int k, int type, const ogs_exchange* x, void* stream) {
  return device_call(h, d_v, k, type, OGS_TRANS, x, stream, 3, "ogs_halo_combine");
}
ogs_status ogs_halo_exchange_host(ogs_halo h, void* v, int k, int type, const ogs_exchange* x, void* stream) {
  return host_call(h, v, k, type, OGS_NOTRANS, x, stream, "ogs_halo_exchange_host");
}
ogs_status ogs_halo_combine_host(ogs_halo h, void* v, int k, int type, const ogs_exchange* x, void* stream) {
  return host_call(h, v, k, type, OGS_TRANS, x, stream, "ogs_halo_combine_host");
}

}  // extern "C"
