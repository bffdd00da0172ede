// Test infrastructure: a C entry point to the reference's own host ogs
// operator (libs/ogs/ogsOperator.cpp, compiled unmodified from the reference
// tree by `make -C oracle refop`), so that the oracle's restatement of
// GatherScatter, Gather and Scatter (ogsOperator.cpp:36-55, 60-97, 206-238,
// 311-360) is checked against the reference's code itself, including the ogs
// identities that gslib does not share (Max starts at -max, not INT_MIN).
//
// The maps are handed in (the oracle's setup, itself pinned to gslib's member
// order): the reference's setup (ogsSetup.cpp) runs the MPI exchanges and is
// not compiled here.  occa.hpp and mpi.h in this directory stand in for the
// two libraries the reference's headers name; no device path is called.
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>

#include "ogs.hpp"
#include "ogs/ogsOperator.hpp"

namespace libp {

// The reference's error path (utils.hpp:103): report and stop.
void abort(const std::string& filename, const std::string& function, const int line, const std::string& message) {
  std::cerr << "ogsref: " << filename << ":" << line << " (" << function << "): " << message << std::endl;
  std::abort();
}

namespace ogs {
// Kernel set-up for the device paths, which the oracle never calls.
void InitializeKernels(platform_t&, const Type, const Op) {}
}  // namespace ogs

}  // namespace libp

namespace {

using libp::memory;
using libp::ogs::ogsOperator_t;

struct RefOp {
  libp::platform_t platform;
  ogsOperator_t op{platform};
};

memory<dlong> copy_ints(const int32_t* src, int64_t n) {
  memory<dlong> m(static_cast<size_t>(n));
  for (int64_t i = 0; i < n; ++i) m[i] = static_cast<dlong>(src[i]);
  return m;
}

template <typename T>
memory<T> to_memory(const void* src, int64_t n) {
  memory<T> m(static_cast<size_t>(n));
  if (n) std::memcpy(m.ptr(), src, static_cast<size_t>(n) * sizeof(T));
  return m;
}

template <typename T>
void from_memory(void* dst, memory<T>& m, int64_t n) {
  if (n) std::memcpy(dst, m.ptr(), static_cast<size_t>(n) * sizeof(T));
}

libp::ogs::Op op_of(int op) {
  switch (op) {
    case 0: return libp::ogs::Add;
    case 1: return libp::ogs::Mul;
    case 2: return libp::ogs::Max;
    default: return libp::ogs::Min;
  }
}

libp::ogs::Transpose trans_of(int t) {
  return t == 0 ? libp::ogs::Sym : (t == 1 ? libp::ogs::NoTrans : libp::ogs::Trans);
}

template <typename T>
void gs_typed(RefOp* h, void* v, int64_t n, int k, int op, int trans) {
  memory<T> m = to_memory<T>(v, n);
  h->op.GatherScatter(m, k, op_of(op), trans_of(trans));
  from_memory(v, m, n);
}

// Mean seconds of `reps` GatherScatter calls on one field held across the
// calls (as dawgs' PerformanceTest holds it), after `warm` untimed calls;
// the field ends as after warm + reps calls.
template <typename T>
double time_gs_typed(RefOp* h, void* v, int64_t n, int k, int op, int trans, int warm, int reps) {
  memory<T> m = to_memory<T>(v, n);
  for (int i = 0; i < warm; ++i) h->op.GatherScatter(m, k, op_of(op), trans_of(trans));
  const auto t0 = std::chrono::steady_clock::now();
  for (int i = 0; i < reps; ++i) h->op.GatherScatter(m, k, op_of(op), trans_of(trans));
  const auto t1 = std::chrono::steady_clock::now();
  from_memory(v, m, n);
  return std::chrono::duration<double>(t1 - t0).count() / (reps > 0 ? reps : 1);
}

template <typename T>
void gather_typed(RefOp* h, void* gv, int64_t ngv, const void* v, int64_t nv, int k, int op, int trans) {
  memory<T> g = to_memory<T>(gv, ngv);
  const memory<T> m = to_memory<T>(v, nv);
  h->op.Gather(g, m, k, op_of(op), trans_of(trans));
  from_memory(gv, g, ngv);
}

template <typename T>
void scatter_typed(RefOp* h, void* v, int64_t nv, const void* gv, int64_t ngv, int k, int trans) {
  memory<T> m = to_memory<T>(v, nv);
  const memory<T> g = to_memory<T>(gv, ngv);
  h->op.Scatter(m, g, k, trans_of(trans));
  from_memory(v, m, nv);
}

}  // namespace

extern "C" {

// Maps in the operator's layout (ogsSetup.cpp:580-631): T maps of NrowsT
// rows and N maps, CSR with ascending member ids, both with NrowsT + 1 row
// starts; NrowsN = the rows with a positive member, which come first; Ncols
// local nodes.
void* ogsref_create(int64_t Ncols, int64_t NrowsT, const int32_t* rsT, const int32_t* ciT, int64_t NrowsN,
                    const int32_t* rsN, const int32_t* ciN) {
  RefOp* h = new RefOp();
  ogsOperator_t& o = h->op;
  o.Ncols = static_cast<dlong>(Ncols);
  o.NrowsT = static_cast<dlong>(NrowsT);
  o.NrowsN = static_cast<dlong>(NrowsN);
  o.nnzT = rsT[NrowsT];
  o.nnzN = rsN[NrowsT];
  o.rowStartsT = copy_ints(rsT, NrowsT + 1);
  o.colIdsT = copy_ints(ciT, rsT[NrowsT]);
  o.rowStartsN = copy_ints(rsN, NrowsT + 1);
  o.colIdsN = copy_ints(ciN, rsN[NrowsT]);
  return h;
}

void ogsref_free(void* h) { delete static_cast<RefOp*>(h); }

// type: 0 float, 1 double, 2 int32, 3 int64; op: 0 Add, 1 Mul, 2 Max, 3 Min;
// trans: 0 Sym, 1 NoTrans, 2 Trans.  In place on the caller's array of n values.
void ogsref_gather_scatter(void* h, void* v, int64_t n, int type, int k, int op, int trans) {
  RefOp* r = static_cast<RefOp*>(h);
  switch (type) {
    case 0: gs_typed<float>(r, v, n, k, op, trans); break;
    case 1: gs_typed<double>(r, v, n, k, op, trans); break;
    case 2: gs_typed<int>(r, v, n, k, op, trans); break;
    default: gs_typed<long long int>(r, v, n, k, op, trans); break;
  }
}

double ogsref_time_gather_scatter(void* h, void* v, int64_t n, int type, int k, int op, int trans, int warm,
                                  int reps) {
  RefOp* r = static_cast<RefOp*>(h);
  switch (type) {
    case 0: return time_gs_typed<float>(r, v, n, k, op, trans, warm, reps);
    case 1: return time_gs_typed<double>(r, v, n, k, op, trans, warm, reps);
    case 2: return time_gs_typed<int>(r, v, n, k, op, trans, warm, reps);
    default: return time_gs_typed<long long int>(r, v, n, k, op, trans, warm, reps);
  }
}

void ogsref_gather(void* h, void* gv, int64_t ngv, const void* v, int64_t nv, int type, int k, int op, int trans) {
  RefOp* r = static_cast<RefOp*>(h);
  switch (type) {
    case 0: gather_typed<float>(r, gv, ngv, v, nv, k, op, trans); break;
    case 1: gather_typed<double>(r, gv, ngv, v, nv, k, op, trans); break;
    case 2: gather_typed<int>(r, gv, ngv, v, nv, k, op, trans); break;
    default: gather_typed<long long int>(r, gv, ngv, v, nv, k, op, trans); break;
  }
}

void ogsref_scatter(void* h, void* v, int64_t nv, const void* gv, int64_t ngv, int type, int k, int trans) {
  RefOp* r = static_cast<RefOp*>(h);
  switch (type) {
    case 0: scatter_typed<float>(r, v, nv, gv, ngv, k, trans); break;
    case 1: scatter_typed<double>(r, v, nv, gv, ngv, k, trans); break;
    case 2: scatter_typed<int>(r, v, nv, gv, ngv, k, trans); break;
    default: scatter_typed<long long int>(r, v, nv, gv, ngv, k, trans); break;
  }
}

}  // extern "C"
