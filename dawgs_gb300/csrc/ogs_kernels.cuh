// ogs_kernels.cuh -- sm_103a gather-scatter kernels over degree-bucketed tiles.
//
// Semantics follow the reference host operator, libs/ogs/ogsOperator.cpp:
//   Op_Add/Mul/Max/Min (36-55): identities 0, 1, -max, +max; updates a+=b,
//     a*=b, (b>a)?b:a, (b<a)?b:a -- including what the comparisons do with NaN;
//   Gather (60-97), Scatter (206-238), GatherScatter (311-360): one fold per
//     row, started from the identity and run over the row's members in
//     ascending local index, so fp32/fp64 sums and products are bit-identical
//     to the host result.
// One CTA of kBlock threads runs one tile: `count` rows of one exact-degree
// bucket (degree known at compile time, every thread owns 8/d rows whose
// column ids and values are all loaded before any fold) or of the general
// bucket (one row per thread, CSR loop).  Floating-point updates use the
// explicitly rounded intrinsics so that no contraction or flush-to-zero can
// change a bit; integer Add/Mul wrap modulo 2^bits like the host code.
#pragma once

#include <cfloat>
#include <climits>
#include <cstdint>
#include <type_traits>

#include <cuda_runtime.h>

#include "ogs_internal.hpp"

namespace ogsgb {

// A column or row id loaded from the maps, checked against [0, lim) in
// checked builds: an id outside is counted in *err and replaced by 0.
__device__ __forceinline__ int32_t checked_id(int32_t id, int32_t lim, unsigned int* err) {
#if OGS_CHECK_BOUNDS
  if (static_cast<uint32_t>(id) >= static_cast<uint32_t>(lim)) {
    if (err) atomicAdd(err, 1u);
    return 0;
  }
#else
  (void)lim;
  (void)err;
#endif
  return id;
}

template <typename T>
__device__ __forceinline__ T type_max() {
  if constexpr (std::is_same<T, float>::value) return FLT_MAX;
  else if constexpr (std::is_same<T, double>::value) return DBL_MAX;
  else if constexpr (std::is_same<T, int32_t>::value) return INT32_MAX;
  else return INT64_MAX;
}

template <typename T, int OP>
__device__ __forceinline__ T op_init() {
  if constexpr (OP == OGS_ADD) return T(0);
  else if constexpr (OP == OGS_MUL) return T(1);
  else if constexpr (OP == OGS_MAX) return -type_max<T>();
  else return type_max<T>();
}

template <typename T, int OP>
__device__ __forceinline__ void op_apply(T& a, const T b) {
  if constexpr (OP == OGS_ADD) {
    if constexpr (std::is_same<T, float>::value) a = __fadd_rn(a, b);
    else if constexpr (std::is_same<T, double>::value) a = __dadd_rn(a, b);
    else {
      using U = typename std::make_unsigned<T>::type;
      a = static_cast<T>(static_cast<U>(a) + static_cast<U>(b));
    }
  } else if constexpr (OP == OGS_MUL) {
    if constexpr (std::is_same<T, float>::value) a = __fmul_rn(a, b);
    else if constexpr (std::is_same<T, double>::value) a = __dmul_rn(a, b);
    else {
      using U = typename std::make_unsigned<T>::type;
      a = static_cast<T>(static_cast<U>(a) * static_cast<U>(b));
    }
  } else if constexpr (OP == OGS_MAX) {
    a = (b > a) ? b : a;
  } else {
    a = (b < a) ? b : a;
  }
}

// Add or Mul fold of D members that all take part, from member 0 instead of
// from the identity.  1 * x == x and 0 + x == x bit for bit, except
// 0 + (-0) == +0: the sum from the identity is never -0, the sum from member
// 0 is -0 only when every member is -0, so mapping -0 to +0 afterwards gives
// the identity-first result exactly.  NaN operands give NaN in the same
// places (a lone NaN member keeps its own bits instead of the GPU's quieted
// ones).  One add fewer per row: fp64 adds go to a narrow pipe on GB300 (2
// per SM per clock), which the identity-first fold kept about half busy.
template <typename T, int OP, int D, int N>
__device__ __forceinline__ T fold_from_first(const T (&V)[N], int at) {
  T a = V[at];
#pragma unroll
  for (int q = 1; q < D; ++q) op_apply<T, OP>(a, V[at + q]);
  if constexpr (OP == OGS_ADD && std::is_floating_point<T>::value) {
    using U = typename std::conditional<sizeof(T) == 8, unsigned long long, unsigned int>::type;
    constexpr U neg_zero = U(1) << (8 * sizeof(T) - 1);
    U bits;
    memcpy(&bits, &a, sizeof(T));
    if (bits == neg_zero) a = T(0);
  }
  return a;
}

// gslib's identities (3rdParty/gslib/src/gs_defs.h:44-52): as ogs, except
// integer Max, which starts from INT_MIN / LLONG_MIN.
template <typename T, int OP>
__device__ __forceinline__ T op_init_gs() {
  if constexpr (OP == OGS_MAX && std::is_same<T, int32_t>::value) return INT32_MIN;
  else if constexpr (OP == OGS_MAX && std::is_same<T, int64_t>::value) return INT64_MIN;
  else return op_init<T, OP>();
}

// Address of component k of node 0; node c lives at base[c * stride].
template <typename T>
__device__ __forceinline__ T* field_base(const FieldArgs& f, int k) {
  return f.is_many ? static_cast<T*>(f.many[k]) : static_cast<T*>(f.v) + k;
}

// Rows of exact degree D.
template <typename T, int OP, int MODE, bool K1, int D>
__device__ __forceinline__ void run_fixed(const DevBucket& b, const Tile& t, const FieldArgs& f,
                                          const Pattern& pat) {
  constexpr int RPT = rows_per_thread(D);
  int end = t.begin + t.count;
  if (pat.limit_n) end = min(end, b.nP);
  const int n = b.stride;
  const bool use_mask = (pat.gather_n || pat.scatter_n) && b.nmask != nullptr;

  int idx[RPT];
  bool ok[RPT];
  int32_t c[RPT][D];
  uint32_t msk[RPT];
  int32_t row[RPT];
#pragma unroll
  for (int j = 0; j < RPT; ++j) {
    idx[j] = t.begin + static_cast<int>(threadIdx.x) + j * kBlock;
    ok[j] = idx[j] < end;
    if (OGS_CHECK_BOUNDS && ok[j] && idx[j] >= b.n) ok[j] = checked_id(idx[j], b.n, b.err) != 0;
  }
#pragma unroll
  for (int j = 0; j < RPT; ++j) {
    msk[j] = 0xFFu;
    row[j] = 0;
    if (ok[j]) {
#pragma unroll
      for (int m = 0; m < D; ++m) c[j][m] = checked_id(__ldg(b.cols + m * n + idx[j]), b.nnodes, b.err);
      if (use_mask) msk[j] = __ldg(b.nmask + idx[j]);
      if (MODE != kModeGS) row[j] = checked_id(__ldg(b.rows + idx[j]), b.nrows, b.err);
    }
  }
  const uint32_t gmask_on = pat.gather_n ? 1u : 0u;
  const uint32_t smask_on = pat.scatter_n ? 1u : 0u;
  const int K = K1 ? 1 : f.K;
  const int64_t stride = K1 ? 1 : (f.is_many ? 1 : K);

  for (int k = 0; k < K; ++k) {
    T val[RPT];
    if (MODE == kModeScatter) {
      const T* gv = static_cast<const T*>(f.gv);
#pragma unroll
      for (int j = 0; j < RPT; ++j)
        if (ok[j]) val[j] = gv[static_cast<int64_t>(row[j]) * K + k];
    } else {
      const T* src = field_base<T>(f, k);
      T x[RPT][D];
#pragma unroll
      for (int j = 0; j < RPT; ++j) {
#pragma unroll
        for (int m = 0; m < D; ++m) {
          const bool take = ok[j] && (!gmask_on || ((msk[j] >> m) & 1u));
          if (take) x[j][m] = src[static_cast<int64_t>(c[j][m]) * stride];
        }
      }
#pragma unroll
      for (int j = 0; j < RPT; ++j) {
        T a;
        if ((OP == OGS_ADD || OP == OGS_MUL) && !gmask_on) {
          a = fold_from_first<T, OP, D>(x[j], 0);
        } else {
          a = op_init<T, OP>();
#pragma unroll
          for (int m = 0; m < D; ++m)
            if (!gmask_on || ((msk[j] >> m) & 1u)) op_apply<T, OP>(a, x[j][m]);
        }
        val[j] = a;
      }
    }
    if (MODE == kModeGather) {
      T* gv = static_cast<T*>(f.gv);
#pragma unroll
      for (int j = 0; j < RPT; ++j)
        if (ok[j]) gv[static_cast<int64_t>(row[j]) * K + k] = val[j];
    } else {
      T* dst = field_base<T>(f, k);
#pragma unroll
      for (int j = 0; j < RPT; ++j) {
#pragma unroll
        for (int m = 0; m < D; ++m)
          if (ok[j] && (!smask_on || ((msk[j] >> m) & 1u)))
            dst[static_cast<int64_t>(c[j][m]) * stride] = val[j];
      }
    }
  }
}

// Rows of degree > kDmax: one row per thread, CSR loops.
template <typename T, int OP, int MODE, bool K1>
__device__ __forceinline__ void run_general(const DevGeneral& g, const Tile& t, const FieldArgs& f,
                                            const Pattern& pat) {
  int end = t.begin + t.count;
  if (pat.limit_n) end = min(end, g.nP);
  const int i = t.begin + static_cast<int>(threadIdx.x);
  if (i >= end) return;
  const int32_t* gc = pat.gather_n ? g.colsN : g.colsT;
  const int32_t* gs = pat.gather_n ? g.startsN : g.startsT;
  const int32_t* sc = pat.scatter_n ? g.colsN : g.colsT;
  const int32_t* ss = pat.scatter_n ? g.startsN : g.startsT;
  const int32_t g0 = gs[i], g1 = gs[i + 1], s0 = ss[i], s1 = ss[i + 1];
  const int64_t r = (MODE != kModeGS) ? checked_id(g.rows[i], g.nrows, g.err) : 0;
  const int K = K1 ? 1 : f.K;
  const int64_t stride = K1 ? 1 : (f.is_many ? 1 : K);
  for (int k = 0; k < K; ++k) {
    T a;
    if (MODE == kModeScatter) {
      a = static_cast<const T*>(f.gv)[r * K + k];
    } else if (pat.gslib) {
      // gslib: fold from the first member taking part (gs_local.c:58-72)
      const T* src = field_base<T>(f, k);
      if (g1 > g0) {
        a = src[static_cast<int64_t>(checked_id(gc[g0], g.nnodes, g.err)) * stride];
        for (int32_t q = g0 + 1; q < g1; ++q)
          op_apply<T, OP>(a, src[static_cast<int64_t>(checked_id(gc[q], g.nnodes, g.err)) * stride]);
      } else {
        a = op_init_gs<T, OP>();
      }
    } else {
      const T* src = field_base<T>(f, k);
      a = op_init<T, OP>();
      for (int32_t q = g0; q < g1; ++q)
        op_apply<T, OP>(a, src[static_cast<int64_t>(checked_id(gc[q], g.nnodes, g.err)) * stride]);
    }
    if (MODE == kModeGather) {
      static_cast<T*>(f.gv)[r * K + k] = a;
    } else {
      T* dst = field_base<T>(f, k);
      if (pat.scatter_n == 2 && g.startsN[i + 1] == g.startsN[i]) {
        // no unflagged member: the primary only
        dst[static_cast<int64_t>(checked_id(g.colsT[g.startsT[i]], g.nnodes, g.err)) * stride] = a;
      } else {
        for (int32_t q = s0; q < s1; ++q) dst[static_cast<int64_t>(checked_id(sc[q], g.nnodes, g.err)) * stride] = a;
      }
    }
  }
}

template <typename T, int OP, int MODE, bool K1>
__global__ void __launch_bounds__(kBlock) ogs_tiles_kernel(const DevMaps m, const FieldArgs f,
                                                           const Pattern pat) {
  const Tile t = m.tiles[blockIdx.x];
  switch (t.bucket) {
    case 1: run_fixed<T, OP, MODE, K1, 1>(m.b[1], t, f, pat); break;
    case 2: run_fixed<T, OP, MODE, K1, 2>(m.b[2], t, f, pat); break;
    case 3: run_fixed<T, OP, MODE, K1, 3>(m.b[3], t, f, pat); break;
    case 4: run_fixed<T, OP, MODE, K1, 4>(m.b[4], t, f, pat); break;
    case 5: run_fixed<T, OP, MODE, K1, 5>(m.b[5], t, f, pat); break;
    case 6: run_fixed<T, OP, MODE, K1, 6>(m.b[6], t, f, pat); break;
    case 7: run_fixed<T, OP, MODE, K1, 7>(m.b[7], t, f, pat); break;
    case 8: run_fixed<T, OP, MODE, K1, 8>(m.b[8], t, f, pat); break;
    default: run_general<T, OP, MODE, K1>(m.g, t, f, pat); break;
  }
}

template <typename T, int OP, int MODE>
inline cudaError_t launch_direct(const DevMaps& m, const FieldArgs& f, Pattern pat, cudaStream_t s) {
  if (m.ntiles == 0) return cudaSuccess;
  const dim3 grid(static_cast<unsigned>(m.ntiles)), block(kBlock);
  if (f.K == 1 && !f.is_many) ogs_tiles_kernel<T, OP, MODE, true><<<grid, block, 0, s>>>(m, f, pat);
  else ogs_tiles_kernel<T, OP, MODE, false><<<grid, block, 0, s>>>(m, f, pat);
  return cudaGetLastError();
}

}  // namespace ogsgb

