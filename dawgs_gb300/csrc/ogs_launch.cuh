// ogs_launch.cuh -- per-type launch dispatch shared by ogs_kern_*.cu.
//
// Exact-degree rows of GatherScatter run on the warp pipeline with
// cp.async-staged gathers (ogs_async.cuh), those of Gather and Scatter on the
// register pipeline of ogs_warp.cuh (-DOGS_GATHER_REGISTERS=0: everything on
// the cp.async one; -DOGS_ASYNC=0: everything on the register one).  Rows
// above degree 8 run on the direct CTA kernel (ogs_kernels.cuh).  Building
// with -DOGS_KERNEL=2 runs the direct CTA kernel for every row instead (for
// comparisons).
//
// Why the split: a GatherScatter row is read and written in place, and two
// tiles' gathers in flight through the shared-memory ring beat one in
// registers (24^3 p=7 fp64: 28.3 vs 31.6 us; 32x32x16 p=5 permuted k=3: 41.1
// vs 42.4 us); a Gather writes one value per row and a Scatter reads one per
// row, and there the ring's shared-memory fills cost more than they hide
// (24^3 p=7: Gather Trans 25.2 vs 26.6 us, Scatter NoTrans 29.9 vs 30.6 us;
// k=3: Gather 32.9 vs 52.0 us, Scatter 47.3 vs 50.9 us).
#pragma once

#include "ogs_async.cuh"

#ifndef OGS_KERNEL
#define OGS_KERNEL 0
#endif
#ifndef OGS_GATHER_REGISTERS
#define OGS_GATHER_REGISTERS 1
#endif

namespace ogsgb {

template <typename T, int OP, int MODE>
inline cudaError_t launch_mode(const DevMaps& m, const FieldArgs& f, Pattern pat, cudaStream_t s) {
  if constexpr (OGS_KERNEL == 2) {
    return launch_direct<T, OP, MODE>(m, f, pat, s);
  } else if constexpr (OGS_ASYNC != 0) {
    if constexpr (MODE != kModeGS && OGS_GATHER_REGISTERS != 0) return launch_warp<T, OP, MODE>(m, f, pat, s);
    else return launch_async<T, OP, MODE>(m, f, pat, s);
  } else {
    return launch_warp<T, OP, MODE>(m, f, pat, s);
  }
}

template <typename T, int MODE>
inline cudaError_t launch_op(const DevMaps& m, const FieldArgs& f, int op, Pattern pat, cudaStream_t s) {
  switch (op) {
    case OGS_ADD: return launch_mode<T, OGS_ADD, MODE>(m, f, pat, s);
    case OGS_MUL: return launch_mode<T, OGS_MUL, MODE>(m, f, pat, s);
    case OGS_MAX: return launch_mode<T, OGS_MAX, MODE>(m, f, pat, s);
    default: return launch_mode<T, OGS_MIN, MODE>(m, f, pat, s);
  }
}

template <typename T>
inline int launch_typed(const DevMaps& m, const FieldArgs& f, int mode, int op, Pattern pat, void* stream) {
  if (m.ntiles == 0) return 0;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaError_t e;
  if (mode == kModeGS) e = launch_op<T, kModeGS>(m, f, op, pat, s);
  else if (mode == kModeGather) e = launch_op<T, kModeGather>(m, f, op, pat, s);
  else e = launch_mode<T, OGS_ADD, kModeScatter>(m, f, pat, s);  // a copy: op unused
  return static_cast<int>(e);
}

}  // namespace ogsgb
